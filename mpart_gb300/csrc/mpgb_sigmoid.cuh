// Sigmoid1d basis of the last input of a sigmoid expansion (device side).
#pragma once
#include "mpgb_types.h"

namespace mpgb {

// Sigmoid1d at y, k = 0..P (P <= PMAX at run time), with first and (D2)
// second derivatives (MParT/Sigmoid.h:214-366): f_0 = 1, f_1 = y,
// f_2 = -w_0 g(-b_0 (y - c_0)), f_3 = w_1 g(b_1 (y - c_1)) with the SoftPlus
// edge g, and f_k = sum_j w_j s(b_j (y - c_j)) with the logistic
// s(t) = 1/2 + tanh(t/2)/2, s' = s (1 - s), s'' = s (1 - s)(1 - 2 s).
template <int PMAX, bool D2>
__device__ __forceinline__ void sigmoidBasis(double y, int P, const CompDesc& c, double* v, double* d1, double* d2) {
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) {
        v[k] = (k == 0) ? 1.0 : 0.0;
        d1[k] = 0.0;
        if constexpr (D2) d2[k] = 0.0;
    }
    if (PMAX >= 1 && P >= 1) {
        v[1] = y;
        d1[1] = 1.0;
    }
    if (PMAX >= 2 && P >= 2) {
        const double b = __ldg(&c.sigW[0]), w = __ldg(&c.sigWt[0]);
        double g, gp;
        posEval<kPosSoftPlus>(-b * (y - __ldg(&c.sigC[0])), g, gp);
        v[2] = -w * g;
        d1[2] = w * b * gp;
        if constexpr (D2) d2[2] = -w * b * b * (gp * (1.0 - gp));
    }
    if (PMAX >= 3 && P >= 3) {
        const double b = __ldg(&c.sigW[1]), w = __ldg(&c.sigWt[1]);
        double g, gp;
        posEval<kPosSoftPlus>(b * (y - __ldg(&c.sigC[1])), g, gp);
        v[3] = w * g;
        d1[3] = w * b * gp;
        if constexpr (D2) d2[3] = w * b * b * (gp * (1.0 - gp));
    }
#pragma unroll
    for (int k = 4; k <= PMAX; ++k) {
        if (k <= P) {
            const int j0 = __ldg(&c.sigStart[k - 4]);
            const int j1 = (k - 3 < c.sigNStarts) ? __ldg(&c.sigStart[k - 3]) : c.sigN;
            double sv = 0.0, s1 = 0.0, s2 = 0.0;
            for (int j = j0; j < j1; ++j) {
                const double b = __ldg(&c.sigW[j]), w = __ldg(&c.sigWt[j]);
                const double f = 0.5 + 0.5 * tanh(0.5 * (b * (y - __ldg(&c.sigC[j]))));
                const double fp = f * (1.0 - f);
                sv = fma(w, f, sv);
                s1 = fma(w * b, fp, s1);
                if constexpr (D2) s2 = fma(w * b * b, fp * (1.0 - 2.0 * f), s2);
            }
            v[k] = sv;
            d1[k] = s1;
            if constexpr (D2) d2[k] = s2;
        }
    }
}

}  // namespace mpgb
