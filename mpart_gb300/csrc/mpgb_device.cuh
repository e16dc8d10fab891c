// Device-side building blocks of the monotone-component hot path (FP64).
//
// Factored integrand.  With prefix products Phi_m(x_<D) = prod_{(d,o) in m}
// phi_o(x_d) over the first D-1 coordinates, every term c_t of the expansion
// splits as t = (m, k) with k the order in the last coordinate, and
//     f(x_<D, y)      = sum_k a_k  phit_k(y),   a_k = sum_m c_(m,k) Phi_m
//     d_D f(x_<D, y)  = sum_k a_k  phit'_k(y)
// so each quadrature node costs O(p) instead of the reference's
// O(sum of nonzeros) term loop (MParT/MultivariateExpansionWorker.h:233-257).
// phit_0 == 1: order-0 factors are never read by the reference's term
// products (MultivariateExpansionWorker.h:423-459), so the constant is 1 for
// every basis, including normalised Hermite polynomials.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpgb_fastmath.cuh"

namespace mpgb {

constexpr int kBasisProbHermite = 0;
constexpr int kBasisHermiteFunctions = 2;
// Sigmoid expansion (RectifiedMultivariateExpansion / UnivariateExpansion):
// Hermite functions in the leading inputs, a Sigmoid1d basis in the last one,
// no quadrature.
constexpr int kBasisSigmoid = 3;
constexpr int kPosExp = 0;
constexpr int kPosSoftPlus = 1;

// Largest number of bisection levels the adaptive rule may use.  The
// reference keeps the branch path in a 32-bit unsigned (Quadrature.h:837,
// :925-944), so maxSub <= 32 is its own limit as well.
constexpr int kMaxSubCap = 32;
// Fused kernel: resident 128-thread blocks per SM its register budget is
// built for; reduced launches cut each component into this many work items
// per SM.
constexpr int kFusedBlocksPerSM = 4;
// Largest phase-A staging (coefficient doubles plus table words) a fused
// launch keeps in shared memory.
constexpr int kStageCap = 2048;
// Inverse: doubles of a saved root-solver state (RootSolve::save).
constexpr int kSolveStateDoubles = 14;
// Inverse warp pass: lanes per deferred point (32 / kWarpGroup points per warp).
constexpr int kWarpGroup = 8;
// Largest nested Clenshaw-Curtis level (coarse 2^L+1, fine 2^(L+1)+1 points).
constexpr int kMaxQuadLevel = 4;
constexpr int kMaxRulePts = (1 << (kMaxQuadLevel + 1)) + 1;
// Largest order in the last coordinate that the kernels are instantiated for.
constexpr int kMaxLastOrder = 12;
// Largest number of nonzero factors in a prefix product.
constexpr int kMaxDepth = 16;

// Per-point status bits (also OR-ed into the per-call status word).
constexpr int kStatusInf = 1;          // g(df) was +inf (the reference throws)
constexpr int kStatusNaN = 2;          // the integrand was NaN
constexpr int kStatusBudget = 4;       // interval budget exhausted
constexpr int kStatusNoBracket = 8;    // inverse: bracket search failed (info=-2)
// Inverse info code of a point whose bracket search ran out of its first-pass
// budget (solved again in the second pass; never returned to callers).
constexpr int kInfoDeferred = -3;
constexpr unsigned kBracketIts = 128;  // FindBracket's step limit (RootFinding.h:29)
// Inverse root solvers (InverseParams::method).
constexpr int kInverseITP = 0;     // the reference's FindBracket + ITP (default)
constexpr int kInverseNewton = 1;  // FindBracket + safeguarded Newton with the exact slope
// Largest sort key of a deferred inverse point: below 36, so that deferred
// points stay out of sortBucket's last bucket, which holds the NaN keys of
// the points that were not deferred.
constexpr double kDeferKeyMax = 30.0;

// Quadrature kinds (MapOptions::quadType values).
constexpr int kQuadFixedCC = 0;   // ClenshawCurtis: one fixed rule on [0, 1] (Quadrature.h:114-143)
constexpr int kQuadSimpson = 1;   // AdaptiveSimpson (Quadrature.h:497-716)
constexpr int kQuadACC = 2;       // AdaptiveClenshawCurtis (Quadrature.h:729-1009)

// Quadrature rule and tolerances.  The adaptive kinds share one traversal:
// a coarse and a nested fine rule on [-1, 1] (fine node 2i = coarse node i),
// scaled by the interval's half width; AdaptiveSimpson is the pair (Simpson
// on the interval, composite Simpson on its halves).  The fixed kind uses the
// fine rule alone.
struct QuadParams {
    double cPts[kMaxRulePts], cWts[kMaxRulePts];
    double fPts[kMaxRulePts], fWts[kMaxRulePts];
    int kind;
    int nCoarse, nFine;
    int maxSub, minSub;
    double absTol, relTol;
    long long maxIntervals;  // per-point interval budget (status kStatusBudget)
};

// Constants of the last-coordinate basis.
struct BasisConsts {
    // Probabilist Hermite: 1 / sqrt(sqrt(2 pi) k!) (or 1 when unnormalised).
    double invNorm[kMaxLastOrder + 1];
    // Hermite functions: psi_k = hfScale[k] * H_k(y) * exp(-y^2/2) with
    // hfScale[k] = pi^(-1/4) (2^k k!)^(-1/2)  (HermiteFunction.h:22-104).
    double hfScale[kMaxLastOrder + 1];
    // Hermite-function recurrence for the first coordinates (EvaluateAll,
    // HermiteFunction.h:26-46): r1[i] = sqrt((i-1)/2), r2[i] = 1/sqrt(i/2).
    double hfR1[kMaxLastOrder + 8], hfR2[kMaxLastOrder + 8];
    double piQuarter;  // pi^(-1/4)
    // Derivatives of the leading-coordinate basis from the basis itself:
    // probabilist Hermite phi_k' = leadDR[k] phi_(k-1) (k >= 2, leadDR[k] =
    // k invNorm[k] / invNorm[k-1]) and phi_1' = leadDR[1] = invNorm[1];
    // Hermite functions psi_j' = -x psi_j + hfSq2j[j] psi_(j-1), hfSq2j[j] = sqrt(2 j).
    double leadDR[kMaxLastOrder + 1];
    double hfSq2j[kMaxLastOrder + 8];
    // phit_k(0) for k = 0..kMaxLastOrder (phit_0 = 1).
    double v0[kMaxLastOrder + 1];
};

// acc[k] += phi * w[k * wstride] for k < nk, as a uniform jump into a chain
// of unconditional FMAs (no predicated FP64 slots).
template <int PMAX>
__device__ __forceinline__ void accumSlots(int nk, double phi, const double* w, int wstride, double* acc) {
    switch (nk) {
#define MPGB_ACC_CASE(K) \
    case K + 1:          \
        if constexpr (K <= PMAX) acc[K] = fma(phi, w[(K) * wstride], acc[K]); \
        [[fallthrough]];
        MPGB_ACC_CASE(12) MPGB_ACC_CASE(11) MPGB_ACC_CASE(10) MPGB_ACC_CASE(9) MPGB_ACC_CASE(8)
        MPGB_ACC_CASE(7) MPGB_ACC_CASE(6) MPGB_ACC_CASE(5) MPGB_ACC_CASE(4) MPGB_ACC_CASE(3)
        MPGB_ACC_CASE(2) MPGB_ACC_CASE(1) MPGB_ACC_CASE(0)
#undef MPGB_ACC_CASE
        default: break;
    }
}

// Same with coefficients read through the read-only path (uniform address).
template <int PMAX>
__device__ __forceinline__ void accumCoeffs(int nk, double phi, const double* __restrict__ cs, double* acc) {
    switch (nk) {
#define MPGB_ACC_CASE(K) \
    case K + 1:          \
        if constexpr (K <= PMAX) acc[K] = fma(__ldg(&cs[K]), phi, acc[K]); \
        [[fallthrough]];
        MPGB_ACC_CASE(12) MPGB_ACC_CASE(11) MPGB_ACC_CASE(10) MPGB_ACC_CASE(9) MPGB_ACC_CASE(8)
        MPGB_ACC_CASE(7) MPGB_ACC_CASE(6) MPGB_ACC_CASE(5) MPGB_ACC_CASE(4) MPGB_ACC_CASE(3)
        MPGB_ACC_CASE(2) MPGB_ACC_CASE(1) MPGB_ACC_CASE(0)
#undef MPGB_ACC_CASE
        default: break;
    }
}

// accumCoeffs with the coefficients in shared memory.
template <int PMAX>
__device__ __forceinline__ void accumCoeffsShared(int nk, double phi, const double* cs, double* acc) {
    switch (nk) {
#define MPGB_ACC_CASE(K) \
    case K + 1:          \
        if constexpr (K <= PMAX) acc[K] = fma(cs[K], phi, acc[K]); \
        [[fallthrough]];
        MPGB_ACC_CASE(12) MPGB_ACC_CASE(11) MPGB_ACC_CASE(10) MPGB_ACC_CASE(9) MPGB_ACC_CASE(8)
        MPGB_ACC_CASE(7) MPGB_ACC_CASE(6) MPGB_ACC_CASE(5) MPGB_ACC_CASE(4) MPGB_ACC_CASE(3)
        MPGB_ACC_CASE(2) MPGB_ACC_CASE(1) MPGB_ACC_CASE(0)
#undef MPGB_ACC_CASE
        default: break;
    }
}

// Product of the first `depth` entries of r (rows of the basis table) at
// column j: one multiply per factor after the first.
__device__ __forceinline__ double prefixProduct(int depth, const int* r, const double* B, int bstride, int j) {
    double phi = 1.0;
    if (depth > 0) {
        phi = B[r[0] * bstride + j];
        switch (depth) {
#define MPGB_PROD_CASE(Q) \
    case Q + 1:           \
        phi *= B[r[Q] * bstride + j]; \
        [[fallthrough]];
            MPGB_PROD_CASE(15) MPGB_PROD_CASE(14) MPGB_PROD_CASE(13) MPGB_PROD_CASE(12) MPGB_PROD_CASE(11)
            MPGB_PROD_CASE(10) MPGB_PROD_CASE(9) MPGB_PROD_CASE(8) MPGB_PROD_CASE(7) MPGB_PROD_CASE(6)
            MPGB_PROD_CASE(5) MPGB_PROD_CASE(4) MPGB_PROD_CASE(3) MPGB_PROD_CASE(2) MPGB_PROD_CASE(1)
#undef MPGB_PROD_CASE
            default: break;
        }
    }
    return phi;
}

// Sort bucket of a point by |x_D| (256 buckets): width 1/32 below 4, width 1/4
// from 4 to 36, then NaN and everything larger in the last.  The adaptive
// quadrature's cost grows with |x_D|; points of one bucket cost about the same.
__device__ __forceinline__ int sortBucket(double x) {
    const double a = fabs(x);
    if (a < 4.0) return (int)(a * 32.0);
    if (a < 36.0) return 128 + (int)((a - 4.0) * 4.0);
    return 255;
}

// --------------------------------------------------------------------------
// Positive bijectors (MParT/PositiveBijectors.h:12-57).  g and g' share one
// exponential; the formulas are the reference's, including log(1 + e) rather
// than log1p(e), so that the value is the same to rounding.  exp and log are
// the table-driven ones of mpgb_fastmath.cuh (about 1 ulp; the SoftPlus pair
// costs half the time of CUDA's exp and log).
// --------------------------------------------------------------------------
template <int POS>
__device__ __forceinline__ void posEval(double x, double& g, double& gp) {
    if constexpr (POS == kPosExp) {
        g = fm::expT(x);
        gp = g;
    } else {
        const double e = fm::expT(-fabs(x));
        g = fm::log1to2T(1.0 + e) + fmax(x, 0.0);
        const double r = 1.0 / (1.0 + e);
        gp = (x < 0.0) ? e * r : r;
    }
}

template <int POS>
__device__ __forceinline__ double posDeriv(double x) {
    double g, gp;
    posEval<POS>(x, g, gp);
    return gp;
}

template <int POS>
__device__ __forceinline__ double posValue(double x) {
    if constexpr (POS == kPosExp) return fm::expT(x);
    else return fm::log1to2T(1.0 + fm::expT(-fabs(x))) + fmax(x, 0.0);
}

// --------------------------------------------------------------------------
// Last-coordinate basis at y, k = 0..P (P <= PMAX at run time).
//   val[k]  = phit_k(y)      (val[0] = 1)
//   d1[k]   = phit'_k(y)
//   d2[k]   = phit''_k(y)
// Only what the caller asks for is computed.
// --------------------------------------------------------------------------
template <int BASIS, int PMAX, bool VAL, bool D1, bool D2>
__device__ __forceinline__ void lastBasis(double y, int P, const BasisConsts& bc, double* val, double* d1,
                                          double* d2) {
    if constexpr (BASIS == kBasisProbHermite) {
        // He_0 = 1, He_1 = y, He_k = y He_{k-1} - (k-1) He_{k-2}.
        double he[PMAX + 1];
        he[0] = 1.0;
        if (PMAX >= 1) he[1] = y;
#pragma unroll
        for (int k = 2; k <= PMAX; ++k) he[k] = (k <= P) ? (y * he[k - 1] - (k - 1.0) * he[k - 2]) : 0.0;
        if constexpr (VAL) {
            val[0] = 1.0;
#pragma unroll
            for (int k = 1; k <= PMAX; ++k) val[k] = (k <= P) ? he[k] * bc.invNorm[k] : 0.0;
        }
        if constexpr (D1) {
            d1[0] = 0.0;
#pragma unroll
            for (int k = 1; k <= PMAX; ++k) d1[k] = (k <= P) ? (double(k) * bc.invNorm[k]) * he[k - 1] : 0.0;
        }
        if constexpr (D2) {
            d2[0] = 0.0;
            if (PMAX >= 1) d2[1] = 0.0;
#pragma unroll
            for (int k = 2; k <= PMAX; ++k)
                d2[k] = (k <= P) ? (double(k) * (k - 1.0) * bc.invNorm[k]) * he[k - 2] : 0.0;
        }
    } else {
        // Hermite functions: phit_0 = 1, phit_1 = y, phit_{j+2} = psi_j(y).
        // psi_j = s_j H_j e, H_j physicist Hermite, e = exp(-y^2/2).
        // psi_j' = s_j e (2 j H_{j-1} - y H_j),  psi_j'' = -(2j + 1 - y^2) psi_j.
        double H[PMAX + 1];
        H[0] = 1.0;
        if (PMAX >= 1) H[1] = 2.0 * y;
#pragma unroll
        for (int j = 2; j <= PMAX; ++j) H[j] = (j + 2 <= P) ? (2.0 * y * H[j - 1] - 2.0 * (j - 1.0) * H[j - 2]) : 0.0;
        const double e = (P >= 2) ? fm::expT(-0.5 * y * y) : 0.0;
        if constexpr (VAL) {
            val[0] = 1.0;
            if (PMAX >= 1) val[1] = (P >= 1) ? y : 0.0;
#pragma unroll
            for (int k = 2; k <= PMAX; ++k) val[k] = (k <= P) ? (bc.hfScale[k - 2] * e) * H[k - 2] : 0.0;
        }
        if constexpr (D1) {
            d1[0] = 0.0;
            if (PMAX >= 1) d1[1] = (P >= 1) ? 1.0 : 0.0;
#pragma unroll
            for (int k = 2; k <= PMAX; ++k) {
                const int j = k - 2;
                const double hjm1 = (j >= 1) ? 2.0 * j * H[j > 0 ? j - 1 : 0] : 0.0;
                d1[k] = (k <= P) ? (bc.hfScale[j] * e) * (hjm1 - y * H[j]) : 0.0;
            }
        }
        if constexpr (D2) {
            d2[0] = 0.0;
            if (PMAX >= 1) d2[1] = 0.0;
#pragma unroll
            for (int k = 2; k <= PMAX; ++k) {
                const int j = k - 2;
                d2[k] = (k <= P) ? -(2.0 * j + 1.0 - y * y) * ((bc.hfScale[j] * e) * H[j]) : 0.0;
            }
        }
    }
}

// --------------------------------------------------------------------------
// Values of orders 1..p of the basis in one of the leading coordinates,
// written to out[(o-1)*stride].  Follows EvaluateAll (OrthogonalPolynomial.h:25-43,
// HermiteFunction.h:26-46) up to rounding.  Their derivatives follow from the
// values (leadDeriv).
// --------------------------------------------------------------------------
template <int BASIS>
__device__ __forceinline__ void leadBasis(double x, int p, const BasisConsts& bc, double* out, int stride) {
    if (p <= 0) return;
    if constexpr (BASIS == kBasisProbHermite) {
        double hm2 = 1.0, hm1 = x;  // He_0, He_1
        out[0] = x * bc.invNorm[1];
        for (int k = 2; k <= p; ++k) {
            const double h = x * hm1 - (k - 1.0) * hm2;
            out[(k - 1) * stride] = h * bc.invNorm[k];
            hm2 = hm1;
            hm1 = h;
        }
    } else {
        // phi_1 = x; phi_{i+2} = psi_i by the normalised recurrence.
        out[0] = x;
        if (p >= 2) {
            const double e = fm::expT(-0.5 * x * x);
            double pm2 = bc.piQuarter * e;             // psi_0
            out[1 * stride] = pm2;
            double pm1 = 0.0;
            if (p >= 3) {
                pm1 = 1.4142135623730951 * x * pm2;     // psi_1 = sqrt(2) x psi_0
                out[2 * stride] = pm1;
            }
            for (int i = 2; i + 2 <= p; ++i) {
                const double v = (x * pm1 - bc.hfR1[i] * pm2) * bc.hfR2[i];
                out[(i + 1) * stride] = v;
                pm2 = pm1;
                pm1 = v;
            }
        }
    }
}

// Derivative of the leading-coordinate basis function of order k at x, from
// its value v and the value vm1 of order k - 1 in the same coordinate
// (used for k >= 2): probabilist Hermite phi_k' = k invNorm[k] He_(k-1)
// (OrthogonalPolynomial.h:62-110); Hermite functions phi_1' = 1 and
// psi_j' = -x psi_j + sqrt(2 j) psi_(j-1) (HermiteFunction.h:56-104).
template <int BASIS>
__device__ __forceinline__ double leadDeriv(int k, double x, double v, double vm1, const BasisConsts& bc) {
    if constexpr (BASIS == kBasisProbHermite) {
        return (k == 1) ? bc.leadDR[1] : bc.leadDR[k] * vm1;
    } else {
        if (k == 1) return 1.0;
        if (k == 2) return -x * v;
        return fma(-x, v, bc.hfSq2j[k - 2] * vm1);
    }
}

}  // namespace mpgb
