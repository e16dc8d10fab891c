// Fused FP64 kernels for MParT monotone components on sm_103a.
//
// One thread per point.  A block holds a tile of points and walks a range of
// components; per point and component:
//   phase A  prefix products Phi_m over the leading coordinates (shared-memory
//            stack, one multiply per prefix node) and the per-order sums
//            a_k = sum_m c_(m,k) Phi_m;
//   phase B  adaptive Clenshaw-Curtis quadrature of the rectified diagonal
//            derivative (MParT/Quadrature.h:819-968) on a per-thread stack,
//            carrying the value integrand and, for adjoints, the per-order
//            integrals J_k = int x_D g'(d_D f) phit'_k dt and the x_D-derivative
//            integrand (MonotoneIntegrand.h:118-203);
//   phase C  adjoints: per-point weights w_k turn into dense per-term outputs
//            (Phi_m w_k), a per-block reduction over points (owner-computes:
//            one thread per prefix node) or an input gradient (forward-mode
//            over the prefix tree).
// No atomics on values: reduced adjoints go through per-item partial rows and
// a fixed-order reduction, so results are bitwise reproducible.
#pragma once
#include <algorithm>
#include <cstdio>
#include "mpgb_types.h"
#include "mpgb_launch.h"
#include "mpgb_sigmoid.cuh"

namespace mpgb {

// --------------------------------------------------------------------------
// Integrand at one node t in [0,1]:  h = x_D (g(df) + eps), plus adjoint parts.
// --------------------------------------------------------------------------
// NEEDE: 0 value (and J) only; 1 adds E; 2 (discrete derivative) adds E and
// K_k = d E / d a_k, the MixedCoeff integrand (MonotoneIntegrand.h:148-165).
template <int PMAX, bool NEEDJ, int NEEDE>
struct NodeVal {
    double h;
    double gn;                   // g(df) + eps: at t = 1, the x_D-slope of T
    double F[NEEDJ ? PMAX : 1];  // x_D g'(df) phit'_k(y), k = 1..P
    double E;                    // d/dx_D of the integrand (MonotoneIntegrand.h:193-201)
    double K[NEEDE == 2 ? PMAX : 1];
};

// Per-component constants folded into the coefficients once per point, so a
// quadrature node pays no per-term scaling:
//   d phit_k / dy   = cs_k * u_k(y) * env(y),   d2 phit_k / dy2 = cs_k * v_k(y) * env(y)
// ProbabilistHermite: cs_k = k invNorm_k, u_k = He_{k-1}, v_k = (k-1) He_{k-2}, env = 1.
// HermiteFunctions (k >= 2, j = k-2): cs_k = hfScale_j, u_k = 2j H_{j-1} - y H_j,
// v_k = -(2j+1-y^2) H_j, env = exp(-y^2/2); k = 1 (phit_1 = y): cs = 1, u = 1, env = 1.
template <int BASIS, int PMAX>
__device__ __forceinline__ void scaleCoeffs(const double* a, int P, const BasisConsts& bc, double* as) {
    as[0] = 0.0;
#pragma unroll
    for (int k = 1; k <= PMAX; ++k) {
        double cs;
        if constexpr (BASIS == kBasisProbHermite) cs = double(k) * bc.invNorm[k];
        else cs = (k == 1) ? 1.0 : bc.hfScale[k >= 2 ? k - 2 : 0];
        as[k] = (k <= P) ? a[k] * cs : 0.0;
    }
}

template <int BASIS, int POS, int PMAX, bool NEEDJ, int NEEDE>
__device__ __forceinline__ void evalNode(double t, double xd, const double* as, int P, const BasisConsts& bc,
                                         double nugget, NodeVal<PMAX, NEEDJ, NEEDE>& o, int& st) {
    (void)bc;
    const double y = t * xd;
    double u[PMAX + 1], v[PMAX + 1];
    double df, d2f = 0.0, env = 1.0;
    if constexpr (BASIS == kBasisProbHermite) {
        double he[PMAX + 1];
        he[0] = 1.0;
        if (PMAX >= 1) he[1] = y;
#pragma unroll
        for (int k = 2; k <= PMAX; ++k) he[k] = (k <= P) ? (y * he[k - 1] - (k - 1.0) * he[k - 2]) : 0.0;
        df = 0.0;
#pragma unroll
        for (int k = 1; k <= PMAX; ++k) {
            u[k] = he[k - 1];
            df = fma(as[k], u[k], df);
        }
        if constexpr (NEEDE) {
#pragma unroll
            for (int k = 2; k <= PMAX; ++k) {
                v[k] = (k - 1.0) * he[k - 2];
                d2f = fma(as[k], v[k], d2f);
            }
        }
    } else {
        double H[PMAX + 1];
        H[0] = 1.0;
        if (PMAX >= 1) H[1] = 2.0 * y;
#pragma unroll
        for (int j = 2; j <= PMAX; ++j) H[j] = (j + 2 <= P) ? (2.0 * y * H[j - 1] - 2.0 * (j - 1.0) * H[j - 2]) : 0.0;
        env = (P >= 2) ? fm::expT(-0.5 * y * y) : 0.0;
        double acc = 0.0, acc2 = 0.0;
        if (PMAX >= 1) u[1] = 1.0;
#pragma unroll
        for (int k = 2; k <= PMAX; ++k) {
            const int j = k - 2;
            const double hjm1 = (j >= 1) ? (2.0 * j) * H[j > 0 ? j - 1 : 0] : 0.0;
            u[k] = fma(-y, H[j], hjm1);
            acc = fma(as[k], u[k], acc);
            if constexpr (NEEDE) {
                v[k] = -(2.0 * j + 1.0 - y * y) * H[j];
                acc2 = fma(as[k], v[k], acc2);
            }
        }
        df = fma(env, acc, (PMAX >= 1) ? as[1] : 0.0);
        if constexpr (NEEDE) d2f = env * acc2;
    }
    double g, gp;
    posEval<POS>(df, g, gp);
    o.gn = g + nugget;
    o.h = xd * o.gn;
    if (isinf(g)) st |= kStatusInf;
    else if (isnan(o.h)) st |= kStatusNaN;
    if constexpr (NEEDE == 2) {
        // (x_D t g'' d2f + g') phit'_k + x_D t g' phit''_k, unscaled by cs_k
        // (g'' of PositiveBijectors.h:24-27 / :49-51).
        const double gpp = (POS == kPosExp) ? g : gp * (1.0 - gp);
        const double c1 = fma((xd * t) * gpp, d2f, gp);
        const double c2 = (xd * t) * gp;
#pragma unroll
        for (int k = 1; k <= PMAX; ++k) {
            const double vk = (k >= 2) ? v[k] : 0.0;
            const double kk = fma(c2, vk, c1 * u[k]);
            if constexpr (BASIS == kBasisProbHermite) o.K[k - 1] = kk;
            else o.K[k - 1] = (k == 1) ? kk : env * kk;
        }
    }
    if constexpr (NEEDJ) {
        // Unscaled: J_k is multiplied by cs_k once the integral is done.
        const double q = xd * gp;
        const double qe = q * env;
#pragma unroll
        for (int k = 1; k <= PMAX; ++k) {
            if constexpr (BASIS == kBasisProbHermite) o.F[k - 1] = q * u[k];
            else o.F[k - 1] = (k == 1) ? q : qe * u[k];
        }
    }
    if constexpr (NEEDE) {
        o.E = fma(d2f, (xd * t) * gp, g + nugget);
    } else {
        o.E = 0.0;
    }
    (void)v;
}

template <int PMAX, bool NEEDJ, int NEEDE>
struct QuadOut {
    double Ih;
    double J[NEEDJ ? PMAX : 1];
    double IE;
    double K[NEEDE == 2 ? PMAX : 1];
    int nInt;  // intervals the quadrature visited (its cost)
};

// Per-order constants cs_k of the basis derivatives (see scaleCoeffs).
template <int BASIS>
__device__ __forceinline__ double basisScale(int k, const BasisConsts& bc) {
    if constexpr (BASIS == kBasisProbHermite) return double(k) * bc.invNorm[k];
    else return (k == 1) ? 1.0 : bc.hfScale[k >= 2 ? k - 2 : 0];
}

// AdaptiveClenshawCurtis::Integrate on [0,1] (Quadrature.h:819-968) with the
// QuadError::First metric (:441-481).  Depth-first, left-first bisection; the
// stack keeps (right end, level, integrand at right end).  Intervals, nodes,
// accept/reject tests and the order in which accepted fine sums are added are
// the reference's.
template <int BASIS, int POS, int PMAX, bool NEEDJ, int NEEDE>
__device__ __forceinline__ void integrate(const double* a, int P, double xd, const QuadParams& Q, const BasisConsts& bc,
                                       double nugget, QuadOut<PMAX, NEEDJ, NEEDE>& R, int& st) {
    using NV = NodeVal<PMAX, NEEDJ, NEEDE>;
    constexpr int NJ = NEEDJ ? PMAX : 1;
    constexpr int NK = NEEDE == 2 ? PMAX : 1;
    double stX[kMaxSubCap];
    int stL[kMaxSubCap];
    double stH[kMaxSubCap];
    double stF[kMaxSubCap][NJ];
    double stE[kMaxSubCap];
    double stK[NEEDE == 2 ? kMaxSubCap : 1][NK];

    R.Ih = 0.0;
    R.IE = 0.0;
    R.nInt = 1;
#pragma unroll
    for (int k = 0; k < NJ; ++k) R.J[k] = 0.0;
#pragma unroll
    for (int k = 0; k < NK; ++k) R.K[k] = 0.0;

    double as[PMAX + 1];
    scaleCoeffs<BASIS, PMAX>(a, P, bc, as);
    NV A, B, M, V;
    if (Q.kind == kQuadFixedCC) {
        // ClenshawCurtisQuadrature::Integrate on [0, 1]: sum_i (w_i / 2) f((1 + x_i) / 2).
        for (int i = 0; i < Q.nFine; ++i) {
            evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(0.5 * (1.0 + Q.fPts[i]), xd, as, P, bc, nugget, V, st);
            const double w = 0.5 * Q.fWts[i];
            R.Ih = fma(w, V.h, R.Ih);
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) R.J[k] = fma(w, V.F[k], R.J[k]);
            }
            if constexpr (NEEDE) R.IE = fma(w, V.E, R.IE);
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) R.K[k] = fma(w, V.K[k], R.K[k]);
            }
        }
        if (st & (kStatusInf | kStatusNaN)) { R.Ih = __longlong_as_double(0x7ff8000000000000ULL); return; }
#pragma unroll
        for (int k = 1; k <= PMAX; ++k) {
            if constexpr (NEEDJ) R.J[k - 1] *= basisScale<BASIS>(k, bc);
            if constexpr (NEEDE == 2) R.K[k - 1] *= basisScale<BASIS>(k, bc);
        }
        return;
    }
    evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(0.0, xd, as, P, bc, nugget, A, st);
    evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(1.0, xd, as, P, bc, nugget, B, st);
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    if (st & (kStatusInf | kStatusNaN)) { R.Ih = nan; return; }

    const int cR = Q.nCoarse - 1, cM = cR / 2, fR = Q.nFine - 1, fM = fR / 2;
    double lo = 0.0, hi = 1.0;
    int level = 0, sp = 0;
    long long nIntervals = 0;
    while (true) {
        const double m = 0.5 * (lo + hi);
        const double s = 0.5 * (hi - lo);
        evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(m, xd, as, P, bc, nugget, M, st);
        double ic = (s * Q.cWts[0]) * A.h;
        ic = fma(s * Q.cWts[cM], M.h, ic);
        ic = fma(s * Q.cWts[cR], B.h, ic);
        const double w0 = s * Q.fWts[0], wM = s * Q.fWts[fM], wR = s * Q.fWts[fR];
        double ih = w0 * A.h;
        ih = fma(wM, M.h, ih);
        ih = fma(wR, B.h, ih);
        double iF[NJ], iK[NK];
        double iE = 0.0;
        if constexpr (NEEDJ) {
#pragma unroll
            for (int k = 0; k < NJ; ++k) iF[k] = fma(wR, B.F[k], fma(wM, M.F[k], w0 * A.F[k]));
        }
        if constexpr (NEEDE) iE = fma(wR, B.E, fma(wM, M.E, w0 * A.E));
        if constexpr (NEEDE == 2) {
#pragma unroll
            for (int k = 0; k < NK; ++k) iK[k] = fma(wR, B.K[k], fma(wM, M.K[k], w0 * A.K[k]));
        }
        // Coarse interior points other than the midpoint (level >= 2 rules).
        for (int i = 1; i < cR; ++i) {
            if (i == cM) continue;
            evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(m + s * Q.cPts[i], xd, as, P, bc, nugget, V, st);
            ic = fma(s * Q.cWts[i], V.h, ic);
            const double wf = s * Q.fWts[2 * i];
            ih = fma(wf, V.h, ih);
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) iF[k] = fma(wf, V.F[k], iF[k]);
            }
            if constexpr (NEEDE) iE = fma(wf, V.E, iE);
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) iK[k] = fma(wf, V.K[k], iK[k]);
            }
        }
        // Points only in the fine rule.
        for (int i = 1; i < Q.nFine; i += 2) {
            evalNode<BASIS, POS, PMAX, NEEDJ, NEEDE>(m + s * Q.fPts[i], xd, as, P, bc, nugget, V, st);
            const double wf = s * Q.fWts[i];
            ih = fma(wf, V.h, ih);
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) iF[k] = fma(wf, V.F[k], iF[k]);
            }
            if constexpr (NEEDE) iE = fma(wf, V.E, iE);
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) iK[k] = fma(wf, V.K[k], iK[k]);
            }
        }
        if (st & (kStatusInf | kStatusNaN)) { R.Ih = nan; return; }
        const double err = fabs(ih - ic);
        const double tol = fmax(Q.relTol * fabs(ic), Q.absTol);
        const bool accept = ((err < tol) || (level == Q.maxSub - 1)) && (level >= Q.minSub);
        if (accept) {
            R.Ih += ih;
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) R.J[k] += iF[k];
            }
            if constexpr (NEEDE) R.IE += iE;
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) R.K[k] += iK[k];
            }
            if (sp == 0) {
                R.nInt = (nIntervals + 1 > 0x7fffffffLL) ? 0x7fffffff : (int)(nIntervals + 1);
                break;
            }
            --sp;
            lo = hi;
            A = B;
            hi = stX[sp];
            level = stL[sp];
            B.h = stH[sp];
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) B.F[k] = stF[sp][k];
            }
            if constexpr (NEEDE) B.E = stE[sp];
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) B.K[k] = stK[sp][k];
            }
        } else {
            stX[sp] = hi;
            stL[sp] = level + 1;
            stH[sp] = B.h;
            if constexpr (NEEDJ) {
#pragma unroll
                for (int k = 0; k < NJ; ++k) stF[sp][k] = B.F[k];
            }
            if constexpr (NEEDE) stE[sp] = B.E;
            if constexpr (NEEDE == 2) {
#pragma unroll
                for (int k = 0; k < NK; ++k) stK[sp][k] = B.K[k];
            }
            ++sp;
            hi = m;
            B = M;
            ++level;
        }
        if (++nIntervals >= Q.maxIntervals) {
            st |= kStatusBudget;
            R.Ih = nan;
            return;
        }
    }
    // The nodes accumulated u_k (times env); apply the per-order constants.
#pragma unroll
    for (int k = 1; k <= PMAX; ++k) {
        if constexpr (NEEDJ) R.J[k - 1] *= basisScale<BASIS>(k, bc);
        if constexpr (NEEDE == 2) R.K[k - 1] *= basisScale<BASIS>(k, bc);
    }
}

// Value-only integral for the inverse solver.
template <int BASIS, int POS, int PMAX>
__device__ __forceinline__ double integrateValue(const double* a, int P, double xd, const QuadParams& Q,
                                                 const BasisConsts& bc, double nugget, int& st) {
    QuadOut<PMAX, false, 0> R;
    integrate<BASIS, POS, PMAX, false, 0>(a, P, xd, Q, bc, nugget, R, st);
    return R.Ih;
}

// --------------------------------------------------------------------------
// Shared-memory helpers.  Per-thread tables are stored row-major with one
// column per thread ([row][tpb + pad]) so that a warp reading the same row
// touches consecutive words.
// --------------------------------------------------------------------------
struct SmemLayout {
    double* X;   // [dmax][tpb]        coordinates of the tile's points
    double* B;   // [nBmax][tpb+1]     leading-coordinate basis values
    double* S;   // [depthMax+1][tpb]  prefix-product stack
    double* W;   // [PMAX+1][tpb]      per-point adjoint weights (the rows of S: a
                 //                    component writes W after its last use of S,
                 //                    and the next component's phase A starts after
                 //                    the reduction that reads W)
    double* GX;  // [dmax][tpb]        input gradient accumulators
    double* DS;  // [tri(depthMax+1)][tpb]  forward-mode derivative stack
    double* stage;  // [stageDoubles]  a component's gathered coefficients and prefix-tree tables (phase A)
    int bstride;
};

__host__ __device__ inline size_t smemBytes(int tpb, int dmax, int nBmax, int depthMax, int pmax, bool input,
                                            int stageDoubles = 0) {
    const int sw = (depthMax + 1 > pmax + 1) ? depthMax + 1 : pmax + 1;
    size_t n = (size_t)dmax * tpb + (size_t)nBmax * (tpb + 1) + (size_t)sw * tpb;
    if (input) {
        n += (size_t)dmax * tpb + (size_t)((depthMax + 1) * (depthMax + 2) / 2) * tpb;
    }
    return (n + (size_t)stageDoubles) * sizeof(double);
}

__device__ inline SmemLayout carveSmem(double* base, int tpb, int dmax, int nBmax, int depthMax, int pmax,
                                       bool input) {
    SmemLayout L;
    L.bstride = tpb + 1;
    double* p = base;
    L.X = p; p += (size_t)dmax * tpb;
    L.B = p; p += (size_t)nBmax * (tpb + 1);
    L.S = p;
    L.W = p;
    p += (size_t)((depthMax + 1 > pmax + 1) ? depthMax + 1 : pmax + 1) * tpb;
    if (input) {
        L.GX = p; p += (size_t)dmax * tpb;
        L.DS = p; p += (size_t)((depthMax + 1) * (depthMax + 2) / 2) * tpb;
    } else {
        L.GX = nullptr; L.DS = nullptr;
    }
    L.stage = p;
    return L;
}

// Fill the leading-coordinate basis table for one thread.
template <int BASIS>
__device__ __forceinline__ void fillLead(const CompDesc& c, const SmemLayout& L, int tid, const BasisConsts& bc) {
    for (int d = 0; d < c.D - 1; ++d) {
        const int p = __ldg(&c.leadDeg[d]);
        const int r = __ldg(&c.rowOff[d]);
        const double x = L.X[d * blockDim.x + tid];
        leadBasis<BASIS>(x, p, bc, &L.B[r * L.bstride + tid], L.bstride);
    }
}

// Depth from which phase A keeps the prefix products of monotone components
// for the reduction (shallower products cost the reduction at most one
// multiply and are formed again).
constexpr int kKeepMinDepth = 2;

// Phase A: a_k = sum_m c_(m,k) Phi_m for this thread's point.  With pc, the
// products of the term-carrying nodes of depth >= kKeepMinDepth are kept there
// (one row of blockDim doubles per node of nodeC) for the reduction, which
// would form them again from the basis table; the incremental product here
// multiplies the same factors in the same order as prefixProduct, so the
// values are equal.
template <int PMAX>
__device__ __forceinline__ void phaseA(const CompDesc& c, const SmemLayout& L, int tid, const double* cm,
                                       double* a, double* pc = nullptr) {
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) a[k] = 0.0;
    const int tpb = blockDim.x;
    L.S[tid] = 1.0;
    for (int n = 0; n < c.nNodes; ++n) {
        const uint32_t w = __ldg(&c.nodeA[n]);
        const int depth = w & 31;
        const int nk = (w >> 5) & 31;
        const int brow = w >> 18;
        double phi = 1.0;
        if (depth > 0) {
            phi = L.S[(depth - 1) * tpb + tid] * L.B[brow * L.bstride + tid];
            L.S[depth * tpb + tid] = phi;
        }
        if (nk) {
            if (pc && depth >= kKeepMinDepth) pc[(long long)__ldg(&c.nodeCIdx[n]) * tpb + tid] = phi;
            accumCoeffs<PMAX>(nk, phi, cm + __ldg(&c.nodeSlot[n]), a);
        }
    }
}

// Phase A from shared memory: the component's gathered coefficients (sCm,
// nSlots doubles) and its nodeA / nodeSlot tables (sA, sS), staged by the
// block for the tile.  The same operations in the same order as phaseA.
template <int PMAX>
__device__ __forceinline__ void phaseAStaged(const CompDesc& c, const SmemLayout& L, int tid, const double* sCm,
                                             const uint32_t* sA, const uint32_t* sS, double* a, double* pc) {
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) a[k] = 0.0;
    const int tpb = blockDim.x;
    L.S[tid] = 1.0;
    for (int n = 0; n < c.nNodes; ++n) {
        const uint32_t w = sA[n];
        const int depth = w & 31;
        const int nk = (w >> 5) & 31;
        const int brow = w >> 18;
        double phi = 1.0;
        if (depth > 0) {
            phi = L.S[(depth - 1) * tpb + tid] * L.B[brow * L.bstride + tid];
            L.S[depth * tpb + tid] = phi;
        }
        if (nk) {
            if (pc && depth >= kKeepMinDepth) pc[(long long)__ldg(&c.nodeCIdx[n]) * tpb + tid] = phi;
            accumCoeffsShared<PMAX>(nk, phi, sCm + sS[n], a);
        }
    }
}

// --------------------------------------------------------------------------
// Sigmoid expansions (no quadrature).
// --------------------------------------------------------------------------
// Phase A of a sigmoid expansion: a_0 = sum_m c_(m,0) Phi_m and, for k >= 1,
// a_k = sum_m c_(m,k) R(Phi_m) with R the rectifier when c.rectify, so that
// T = sum_k a_k f_k(x_D).  Terms with a last-input factor and no leading
// factor take R(1), as the reference's term products do
// (MultivariateExpansionWorker.h:423-441).
template <int PMAX, int POS>
__device__ __forceinline__ void phaseARect(const CompDesc& c, const SmemLayout& L, int tid, const double* cm,
                                           double* a, double* rc) {
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) a[k] = 0.0;
    const int tpb = blockDim.x;
    L.S[tid] = 1.0;
    for (int n = 0; n < c.nNodes; ++n) {
        const uint32_t w = __ldg(&c.nodeA[n]);
        const int depth = w & 31;
        const int nk = (w >> 5) & 31;
        const int brow = w >> 18;
        double phi = 1.0;
        if (depth > 0) {
            phi = L.S[(depth - 1) * tpb + tid] * L.B[brow * L.bstride + tid];
            L.S[depth * tpb + tid] = phi;
        }
        if (nk) {
            const double* cs = cm + __ldg(&c.nodeSlot[n]);
            const double a0 = fma(__ldg(&cs[0]), phi, a[0]);
            double r = phi;
            if (c.rectify && nk > 1) {
                r = posValue<POS>(phi);
                if (rc) rc[(long long)__ldg(&c.nodeCIdx[n]) * tpb + tid] = r;
            }
            accumCoeffs<PMAX>(nk, r, cs, a);
            a[0] = a0;
        }
    }
}

// --------------------------------------------------------------------------
// The fused kernel.
// --------------------------------------------------------------------------
// Point data of a work item: the launch-wide fields of FusedParams, or (in a
// batch of maps) the entry of the item's component in prm.ioTable.
#define MPGB_IO(f) (BATCH ? tio->f : prm.f)

template <int BASIS, int POS, int PMAX, bool NEEDJ, int NEEDE, bool BATCH>
__device__ __forceinline__ void fusedBody(const FusedParams& prm, const WorkItem& item, double* smem) {
    const int tid = threadIdx.x;
    const int tpb = blockDim.x;
    const bool inputMode = (prm.flags & kFlagInput) != 0;
    const SmemLayout L = carveSmem(smem, tpb, prm.dmax, prm.nBmax, prm.depthMax, PMAX, inputMode);
    const PointIO* tio = BATCH ? &prm.ioTable[item.c0] : nullptr;
    (void)tio;
    const int flags = prm.flags;
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const double ninf = __longlong_as_double(0xfff0000000000000ULL);

    for (int tj = 0; tj < item.nTiles; ++tj) {
        const int tile = item.tile0 + tj * item.tileStride;
        const long long slotIdx = (long long)tile * tpb + tid;
        const bool active = slotIdx < MPGB_IO(N);
        const long long i = (active && MPGB_IO(perm)) ? (long long)MPGB_IO(perm)[item.c0 * MPGB_IO(permStride) + slotIdx] : slotIdx;
        int st = 0;
        // Coordinates of the tile (the largest component of the range reads the most).
        const int dneed = prm.comps[item.c1 - 1].D;
        for (int d = 0; d < dneed; ++d)
            L.X[d * tpb + tid] = active ? MPGB_IO(pts)[d * MPGB_IO(ptsRs) + i * MPGB_IO(ptsCs)] : 0.0;
        double logdetSum = 0.0;
        double lossAcc = 0.0;
        if (inputMode) {
            const bool carry = (flags & kFlagImplicit) && !(flags & kFlagImplicitFirst) && active;
            for (int d = 0; d < dneed; ++d)
                L.GX[d * tpb + tid] = carry ? prm.outInput[d * prm.inputRs + i * prm.inputCs] : 0.0;
        }

        for (int ci = item.c0; ci < item.c1; ++ci) {
            const CompDesc& c = prm.comps[ci];
            const double* cm = prm.cm + c.slotOffset;
            const int P = c.P;
            fillLead<BASIS>(c, L, tid, prm.bc);

            double a[PMAX + 1];
            // (sigmoid expansions: the rectified products R(Phi_m) of this tile,
            // kept for the reduction below)
            // (monotone components: the products of the deeper prefix nodes)
            double* rc = (prm.rcache && (flags & kFlagCoefReduced)) ? prm.rcache + item.rcBase : nullptr;
            if constexpr (BASIS == kBasisSigmoid) {
                phaseARect<PMAX, POS>(c, L, tid, cm, a, rc);
            } else if (c.nSlots + c.nNodes <= prm.stageDoubles) {
                // The tree walk reads a coefficient and two table words per
                // node, the same addresses in every lane: from shared memory
                // (staged once per tile) rather than as uniform global loads.
                double* sCm = L.stage;
                uint32_t* sA = reinterpret_cast<uint32_t*>(L.stage + c.nSlots);
                uint32_t* sS = sA + c.nNodes;
                __syncthreads();
                for (int k = tid; k < c.nSlots; k += tpb) sCm[k] = __ldg(&cm[k]);
                for (int k = tid; k < c.nNodes; k += tpb) {
                    sA[k] = __ldg(&c.nodeA[k]);
                    sS[k] = __ldg(&c.nodeSlot[k]);
                }
                __syncthreads();
                phaseAStaged<PMAX>(c, L, tid, sCm, sA, sS, a, rc);
            } else {
                phaseA<PMAX>(c, L, tid, cm, a, rc);
            }
            const double xd = L.X[(c.D - 1) * tpb + tid];

            // wv[k] = dT/da_k; d1x, d2x: last-input basis derivatives at x_D;
            // ldx = d logdet / dx_D.
            double wv[PMAX + 1], d1x[PMAX + 1], d2x[PMAX + 1];
            double T, dT, gx, gpx, ldx;
            QuadOut<PMAX, NEEDJ, NEEDE> R;
            R.Ih = 0.0; R.IE = 0.0;
#pragma unroll
            for (int k = 0; k < (NEEDJ ? PMAX : 1); ++k) R.J[k] = 0.0;
            if constexpr (BASIS == kBasisSigmoid) {
                // T = sum_k a_k f_k(x_D), d_D T and d_D^2 T in closed form
                // (RectifiedMultivariateExpansion.h:40-75, :192-225).
                sigmoidBasis<PMAX, true>(xd, P, c, wv, d1x, d2x);
                double t = 0.0, dt = 0.0, d2t = 0.0;
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) {
                    t = fma(a[k], wv[k], t);
                    dt = fma(a[k], d1x[k], dt);
                    d2t = fma(a[k], d2x[k], d2t);
                }
                T = t;
                dT = dt;
                gx = dt;
                gpx = 0.0;
                ldx = d2t / dt;
            } else {
                // Last-coordinate basis at 0 and at x_D.
                const double* v0 = prm.bc.v0;
                lastBasis<BASIS, PMAX, false, true, true>(xd, P, prm.bc, nullptr, d1x, d2x);
                double dfx = 0.0, d2fx = 0.0, f0 = 0.0;
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) {
                    f0 = fma(a[k], v0[k], f0);
                    dfx = fma(a[k], d1x[k], dfx);
                    d2fx = fma(a[k], d2x[k], d2fx);
                }
                posEval<POS>(dfx, gx, gpx);

                // (The discrete-derivative variant, NEEDE == 2, always integrates:
                // its log-determinant is that of the quadrature approximation.)
                const bool needT = (flags & (kFlagEval | kFlagCoefDenseT | kFlagKL)) != 0 ||
                                   (NEEDJ && (flags & (kFlagCoefReduced | kFlagInput))) || NEEDE == 2;
                if (needT && active) {
                    integrate<BASIS, POS, PMAX, NEEDJ, NEEDE>(a, P, xd, prm.quad, prm.bc, prm.nugget, R, st);
                    // the point's cost in this component, a sort key for the next call
                    if (!BATCH && prm.costKey) prm.costKey[(long long)ci * prm.costStride + i] = 0.125 * R.nInt;
                }
                T = R.Ih + f0;
                // dT/dx_D: g(df(x)) (ContinuousDerivative) or the x_D-derivative of
                // the quadrature approximation (DiscreteDerivative, MonotoneComponent.h:585-638).
                dT = (NEEDE == 2) ? R.IE : gx;
                ldx = gpx * (1.0 / gx) * d2fx;
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) wv[k] = v0[k] + ((NEEDJ && k >= 1) ? R.J[k >= 1 ? k - 1 : 0] : 0.0);
            }
            // (A sigmoid expansion's derivative can be negative: log gives NaN
            // there, as the reference's does.)
            const double logdet = (BASIS != kBasisSigmoid && dT <= 0.0) ? ninf : log(dT);

            if ((flags & kFlagEval) && active && MPGB_IO(outEval)) MPGB_IO(outEval)[(long long)c.outRow * MPGB_IO(evalRs) + i * MPGB_IO(evalCs)] = T;
            if (flags & kFlagLogDet) logdetSum += logdet;

            // Per-point adjoint weights.
            double sens = 0.0, lsens = 0.0;
            if (flags & kFlagKL) {
                sens = T * prm.sensScale;
                lsens = prm.lsensScale;
                if (active) lossAcc += 0.5 * T * T - logdet;
            } else {
                if (MPGB_IO(sens) && active) sens = MPGB_IO(sens)[(long long)c.outRow * MPGB_IO(sensRs) + i * MPGB_IO(sensCs)];
                if (flags & (kFlagCoefReduced | kFlagInput))
                    lsens = prm.lsens ? (active ? prm.lsens[i * prm.lsensStride] : 0.0) : prm.lsensScale;
                if (flags & kFlagImplicit) {
                    // lambda = (w - sum_{m > k} lambda_m dT_m/dx_D) / (g(df) + nugget)
                    double* gd = &L.GX[(c.D - 1) * tpb + tid];
                    sens = active ? (sens - *gd) / (BASIS == kBasisSigmoid ? gx : gx + prm.nugget) : 0.0;
                    *gd = sens;
                    lsens = 0.0;
                }
            }
            if (!active) { sens = 0.0; lsens = 0.0; }
            const double ldScale = gpx * (1.0 / gx);
            // d logdet / d a_k: g'/g phit'_k(x_D), or (discrete) K_k / (dT/dx_D)
            // with K the MixedCoeff integral (DiscreteMixedJacobian, MonotoneComponent.h:928-980),
            // or (sigmoid expansion) f'_k(x_D) / d_D T.
            double dld[PMAX + 1];
#pragma unroll
            for (int k = 0; k <= PMAX; ++k) {
                // (inactive lanes did not integrate: keep their weights zero)
                if constexpr (BASIS == kBasisSigmoid) dld[k] = active ? d1x[k] * (1.0 / dT) : 0.0;
                else if constexpr (NEEDE == 2) dld[k] = (k >= 1 && active) ? R.K[k >= 1 ? k - 1 : 0] * (1.0 / R.IE) : 0.0;
                else dld[k] = ldScale * d1x[k];
            }
            double wT[PMAX + 1], wL[PMAX + 1];
#pragma unroll
            for (int k = 0; k <= PMAX; ++k) {
                wT[k] = sens * wv[k];
                // (a sigmoid expansion's d_D T may vanish, e.g. at zero coefficients:
                // without a log-det weight its terms stay out)
                if constexpr (BASIS == kBasisSigmoid) wL[k] = (lsens != 0.0) ? lsens * dld[k] : 0.0;
                else wL[k] = lsens * dld[k];
            }

            // Dense per-term outputs (CoeffGradImpl / LogDeterminantCoeffGradImpl).
            if ((flags & (kFlagCoefDenseT | kFlagCoefDenseL)) && active) {
                const bool useT = (flags & kFlagCoefDenseT) != 0;
                double wd[PMAX + 1];
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) wd[k] = useT ? wT[k] : dld[k];
                L.S[tid] = 1.0;
                for (int n = 0; n < c.nNodes; ++n) {
                    const uint32_t w = __ldg(&c.nodeA[n]);
                    const int depth = w & 31, nk = (w >> 5) & 31, brow = w >> 18;
                    double phi = 1.0;
                    if (depth > 0) {
                        phi = L.S[(depth - 1) * tpb + tid] * L.B[brow * L.bstride + tid];
                        L.S[depth * tpb + tid] = phi;
                    }
                    if (nk) {
                        const int slot = __ldg(&c.nodeSlot[n]);
                        double rv = phi;  // the term's leading factor for k >= 1
                        if constexpr (BASIS == kBasisSigmoid)
                            if (c.rectify && nk > 1) rv = posValue<POS>(phi);
#pragma unroll
                        for (int k = 0; k <= PMAX; ++k) {
                            if (k < nk) {
                                const int t = __ldg(&c.slotTerm[slot + k]);
                                if (t >= 0)
                                    prm.outDense[(long long)(c.coeffOffset + t) * prm.denseRs + i * prm.denseCs] =
                                        (k == 0 ? phi : rv) * wd[k];
                            }
                        }
                    }
                }
            }

            // Input gradient: forward mode over the prefix tree.
            if (inputMode) {
                double w[PMAX + 1];
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) w[k] = wT[k] + wL[k];
                // Triangular stack: DS[tri(l) + j] = d Phi_l / d (factor j), j = 1..l.
                int dims[kMaxDepth + 1];
                L.S[tid] = 1.0;
                for (int n = 0; n < c.nNodes; ++n) {
                    const uint32_t wd = __ldg(&c.nodeA[n]);
                    const int depth = wd & 31, nk = (wd >> 5) & 31, dim = (wd >> 10) & 255, brow = wd >> 18;
                    if (depth > 0) {
                        const double bv = L.B[brow * L.bstride + tid];
                        // order of this factor within its coordinate's rows
                        const int ko = brow - __ldg(&c.rowOff[dim]) + 1;
                        const double bd = leadDeriv<BASIS>(ko, L.X[dim * tpb + tid], bv,
                                                           ko > 1 ? L.B[(brow - 1) * L.bstride + tid] : 0.0, prm.bc);
                        const double pphi = L.S[(depth - 1) * tpb + tid];
                        L.S[depth * tpb + tid] = pphi * bv;
                        const int tl = depth * (depth + 1) / 2, tp = (depth - 1) * depth / 2;
                        for (int j = 1; j < depth; ++j)
                            L.DS[(tl + j) * tpb + tid] = L.DS[(tp + j) * tpb + tid] * bv;
                        L.DS[(tl + depth) * tpb + tid] = pphi * bd;
                        dims[depth] = dim;
                    }
                    if (nk && depth > 0) {
                        const double* cs = cm + __ldg(&c.nodeSlot[n]);
                        double beta = 0.0;
                        if constexpr (BASIS == kBasisSigmoid) {
                            // d/dPhi [c_0 Phi w_0 + R(Phi) sum_k c_k w_k]
                            double b1 = 0.0;
                            for (int k = 1; k < nk; ++k) b1 = fma(__ldg(&cs[k]), w[k < PMAX ? k : PMAX], b1);
                            const double rp = (c.rectify && nk > 1) ? posDeriv<POS>(L.S[depth * tpb + tid]) : 1.0;
                            beta = fma(__ldg(&cs[0]), w[0], rp * b1);
                        } else {
                            for (int k = 0; k < nk; ++k) beta = fma(__ldg(&cs[k]), w[k < PMAX ? k : PMAX], beta);
                        }
                        const int tl = depth * (depth + 1) / 2;
                        for (int j = 1; j <= depth; ++j) {
                            double* g = &L.GX[dims[j] * tpb + tid];
                            *g = fma(beta, L.DS[(tl + j) * tpb + tid], *g);
                        }
                    }
                }
                // Last coordinate: quadrature of the x_D-derivative integrand and the
                // log-det term (MonotoneComponent.h:811-815, :892-925).
                // (The host does not combine lsens with input gradients in the
                // discrete mode, which the reference does not provide.)
                double gxd = (NEEDE == 2) ? 0.0 : lsens * ldx;
                if constexpr (BASIS == kBasisSigmoid) gxd = fma(sens, dT, (lsens != 0.0) ? gxd : 0.0);
                else if constexpr (NEEDE) gxd = fma(sens, R.IE, gxd);
                double* g = &L.GX[(c.D - 1) * tpb + tid];
                if (!(flags & kFlagImplicit)) *g += gxd;  // implicit mode keeps lambda there
            }

            // Reduced combined adjoint: owner-computes over the block's points.
            if (flags & kFlagCoefReduced) {
#pragma unroll
                for (int k = 0; k <= PMAX; ++k) L.W[k * tpb + tid] = wT[k] + wL[k];
                __syncthreads();
                const bool first = (tj == 0);
                // Units (node, point segment); consecutive threads share a node.
                const int S = c.cSegs;
                const int segLen = tpb / S;
                const int units = c.nCNodes * S;
                for (int u = tid; u < units; u += tpb) {
                    const int n = (S == 4) ? (u >> 2) : (S == 1 ? u : u / S);
                    const int sg = u - n * S;
                    double* part = prm.partials + item.partialBase + (long long)sg * c.numTerms;
                    const uint32_t w = __ldg(&c.nodeC[n]);
                    const int depth = w & 31, nk = (w >> 5) & 31, slot = w >> 10;
                    const uint16_t* rows = c.nodeCRows + (size_t)n * kMaxDepth;
                    int r[kMaxDepth];
#pragma unroll
                    for (int q = 0; q < kMaxDepth; ++q) r[q] = (q < depth) ? (int)__ldg(&rows[q]) : 0;
                    double acc[PMAX + 1];
#pragma unroll
                    for (int k = 0; k <= PMAX; ++k) acc[k] = 0.0;
                    // (monotone components: products kept by phase A for the deeper nodes)
                    const double* kept =
                        (BASIS != kBasisSigmoid && rc && depth >= kKeepMinDepth) ? rc + (long long)n * tpb : nullptr;
                    if (kept && segLen % 8 == 0) {
                        // Eight loads in flight before their sums.
                        for (int j = sg * segLen; j < (sg + 1) * segLen; j += 8) {
                            double v[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) v[q] = kept[j + q];
#pragma unroll
                            for (int q = 0; q < 8; ++q) accumSlots<PMAX>(nk, v[q], L.W + j + q, tpb, acc);
                        }
                    } else if (kept) {
                        for (int j = sg * segLen; j < (sg + 1) * segLen; ++j)
                            accumSlots<PMAX>(nk, kept[j], L.W + j, tpb, acc);
                    } else {
                        for (int j = sg * segLen; j < (sg + 1) * segLen; ++j) {
                            const double phi = prefixProduct(depth, r, L.B, L.bstride, j);
                            if constexpr (BASIS == kBasisSigmoid) {
                                const double a0 = fma(phi, L.W[j], acc[0]);
                                double rv = phi;
                                if (c.rectify && nk > 1) rv = rc ? rc[(long long)n * tpb + j] : posValue<POS>(phi);
                                accumSlots<PMAX>(nk, rv, L.W + j, tpb, acc);
                                acc[0] = a0;
                            } else {
                                accumSlots<PMAX>(nk, phi, L.W + j, tpb, acc);
                            }
                        }
                    }
#pragma unroll
                    for (int k = 0; k <= PMAX; ++k) {
                        if (k < nk) {
                            const int t = __ldg(&c.slotTerm[slot + k]);
                            if (t >= 0) {
                                double* dst = part + t;
                                *dst = first ? acc[k] : (*dst + acc[k]);
                            }
                        }
                    }
                }
                __syncthreads();
            }
            if (prm.statusWord && st) atomicOr(prm.statusWord, st);
        }  // components

        if (active) {
            if (flags & kFlagLogDet)
                MPGB_IO(outLogDet)[(BATCH ? 0 : item.c0 * prm.logDetCompStride) + i * MPGB_IO(logDetStride)] =
                    logdetSum;
            if (inputMode) {
                const int dneed2 = prm.comps[item.c1 - 1].D;
                for (int d = 0; d < dneed2; ++d) {
                    const double v = L.GX[d * tpb + tid];
                    prm.outInput[d * prm.inputRs + i * prm.inputCs] = (d < prm.negRows) ? -v : v;
                }
            }
            if (flags & kFlagStatusArray) prm.status[i * prm.statusStride] = st;
        }
        if (flags & kFlagKL) {
            // Block sum of the loss in a fixed order (thread 0 adds the smem column).
            __syncthreads();
            L.W[tid] = lossAcc;
            __syncthreads();
            if (tid == 0) {
                double s = 0.0;
                for (int j = 0; j < tpb; ++j) s += L.W[j];
                double* dst = prm.lossPartials + item.lossSlot;
                *dst = (tj == 0) ? s : (*dst + s);
            }
            __syncthreads();
        }
        __syncthreads();
    }
    (void)nan;
}

template <int BASIS, int POS, int PMAX, bool NEEDJ, int NEEDE>
__global__ void __launch_bounds__(128, kFusedBlocksPerSM) fusedKernel(const __grid_constant__ FusedParams prm) {
    extern __shared__ double smem[];
    fusedBody<BASIS, POS, PMAX, NEEDJ, NEEDE, false>(prm, prm.items[blockIdx.x], smem);
}

// Persistent launch over the work items of a batch of maps (one component of
// one map per item, items in decreasing cost): each block takes the next item
// from a counter until none is left.  Every item owns its outputs (output
// rows, log-det scratch row, partial row), so results do not depend on which
// block runs it.  The item's component selects the body compiled for the
// smallest order class >= its last-coordinate order.  At most 128 threads a
// block.  The kernel is built per largest order class MAXC of the batch, so a
// batch pays the registers of its own bodies only: classes 2 and 4 keep 4
// blocks an SM; with order-6 or order-8 bodies the budget of 2 blocks an SM
// keeps them free of spills (with 4 blocks an SM they spilled, and the 64-map
// workload ran 11 % slower).
template <int BASIS, int POS, int MAXC>
__global__ void __launch_bounds__(128, (MAXC <= 4) ? 4 : 2) batchKernel(const __grid_constant__ FusedParams prm,
                                                                       int nItems, int* counter) {
    extern __shared__ double smem[];
    __shared__ int next;
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        __syncthreads();
        const int k = next;
        __syncthreads();
        if (k >= nItems) break;
        const WorkItem item = prm.items[k];
        const int P = prm.comps[item.c0].P;
        if (P <= 2) {
            fusedBody<BASIS, POS, 2, true, 0, true>(prm, item, smem);
        } else if constexpr (MAXC >= 4) {
            if (P <= 4) {
                fusedBody<BASIS, POS, 4, true, 0, true>(prm, item, smem);
            } else if constexpr (MAXC >= 6) {
                if (P <= 6) fusedBody<BASIS, POS, 6, true, 0, true>(prm, item, smem);
                else if constexpr (MAXC >= 8) fusedBody<BASIS, POS, 8, true, 0, true>(prm, item, smem);
            }
        }
    }
}
#undef MPGB_IO

// --------------------------------------------------------------------------
// Inverse: all components of the map, in order, for a tile of points
// (TriangularMap::InverseInplace, src/TriangularMap.cpp:161-184, with
// MonotoneComponent::InverseImpl, MonotoneComponent.h:330-443, and
// RootFinding::InverseSingleBracket, RootFinding.h:125-178).
// --------------------------------------------------------------------------
template <int PMAX>
struct ACoef {
    double a[PMAX + 1];
};

template <int BASIS, int POS, int PMAX>
__device__ __noinline__ double integrateValueNI(const ACoef<PMAX> A, int P, double xd, const QuadParams* Q,
                                                const BasisConsts* bc, double nugget, int* st) {
    int s = 0;
    const double I = integrateValue<BASIS, POS, PMAX>(A.a, P, xd, *Q, *bc, nugget, s);
    *st |= s;
    return I;
}

template <int BASIS, int POS, int PMAX>
struct InverseEval {
    ACoef<PMAX> A;
    int P;
    double f0;
    const QuadParams* Q;
    const BasisConsts* bc;
    double nugget;
    int* st;
    __device__ double operator()(double x) const {
        return integrateValueNI<BASIS, POS, PMAX>(A, P, x, Q, bc, nugget, st) + f0;
    }
    // dT/dx_D = g(df(x)) + nugget: no quadrature.  Formed as the integrand
    // node at t = 1 forms it, so that the queue pass, which reads the slope
    // off that node (KnownSlope), takes the same steps.
    __device__ double slope(double x) const {
        double as[PMAX + 1];
        scaleCoeffs<BASIS, PMAX>(A.a, P, *bc, as);
        NodeVal<PMAX, false, 0> V;
        int s = 0;
        evalNode<BASIS, POS, PMAX, false, 0>(1.0, x, as, P, *bc, nugget, V, s);
        return V.gn;
    }
};

// The slope at the point just evaluated, read off its quadrature's t = 1 node.
struct KnownSlope {
    double s;
    __device__ double slope(double) const { return s; }
};

// T(x_<D, y) of a sigmoid expansion as a function of y (the reference's
// SingleWorkerEvaluator, RectifiedMultivariateExpansion.h:392-405), and its slope.
template <int PMAX>
struct SigmoidInverseEval {
    ACoef<PMAX> A;
    int P;
    const CompDesc* c;
    __device__ double operator()(double y) const {
        double v[PMAX + 1], d1[PMAX + 1];
        sigmoidBasis<PMAX, false>(y, P, *c, v, d1, nullptr);
        double t = 0.0;
#pragma unroll
        for (int k = 0; k <= PMAX; ++k) t = fma(A.a[k], v[k], t);
        return t;
    }
    __device__ double slope(double y) const {
        double v[PMAX + 1], d1[PMAX + 1];
        sigmoidBasis<PMAX, false>(y, P, *c, v, d1, nullptr);
        double t = 0.0;
#pragma unroll
        for (int k = 0; k <= PMAX; ++k) t = fma(A.a[k], d1[k], t);
        return t;
    }
};

// 2^e for the integer-valued (or infinite / NaN) exponents of the ITP
// truncation, exactly as pow(2.0, e) gives them.
__device__ __forceinline__ double exp2Int(double e) {
    if (isnan(e)) return e;
    if (e > 4096.0) return __longlong_as_double(0x7ff0000000000000ULL);
    if (e < -4096.0) return 0.0;
    return ldexp(1.0, (int)e);
}

// The ITP point of RootFinding::Find_x_ITP (RootFinding.h:92-106) with the
// constants of InverseSingleBracket (k1 = 0.1, k2 = 2, n0 = 1, :145-149), in
// the reference's operation order and without FMA contraction, so that the
// iterates are those of the reference's host build.  pow(w, 2) is w * w
// (libm's pow returns the correctly rounded square).
__device__ __forceinline__ double itpPoint(double xlb, double xub, double ylb, double yub, double nhalf, unsigned it,
                                           double xtol) {
    const double xb = __dmul_rn(0.5, __dadd_rn(xub, xlb));
    double xf = __ddiv_rn(__dsub_rn(__dmul_rn(xub, ylb), __dmul_rn(xlb, yub)), __dsub_rn(ylb, yub));
    const double sigma = (__dsub_rn(xb, xf) > 0) ? 1.0 : -1.0;
    const double w = __dsub_rn(xub, xlb);
    const double delta = fmin(__dmul_rn(0.1, __dmul_rn(w, w)), fabs(__dsub_rn(xb, xf)));
    xf = __dadd_rn(xf, __dmul_rn(delta, sigma));
    const double p2 = exp2Int(__dsub_rn(__dadd_rn(nhalf, 1.0), (double)it));
    const double rho = fmin(__dsub_rn(__dmul_rn(xtol, p2), __dmul_rn(0.5, w)), fabs(__dsub_rn(xf, xb)));
    return __dsub_rn(xb, __dmul_rn(sigma, rho));
}

// Root of f(x) = yd for a monotone f (MonotoneComponent::InverseImpl with
// RootFinding::InverseSingleBracket and FindBracket, RootFinding.h:20-90,
// :125-178) as a state machine that asks for one evaluation of f per step,
// so that the lanes of a warp evaluate f together instead of one after the
// other.  The reference's bracket search is kept step for step (same
// evaluation points, so the same targets have no bracket and give NaN; its
// two repeated evaluations at x0 are taken from the first).
//
// kInverseITP closes the bracket as the reference does: ITP points
// (itpPoint), |f(x) - yd| < ftol returns x, and the loop stops when the
// bracket is narrower than xtol or its values differ by less than ftol,
// returning the midpoint; at most 10000 iterations.
//
// kInverseNewton closes it by a safeguarded Newton iteration with the exact
// slope dT/dx_D = g(df) + nugget: every evaluation narrows the bracket; a
// Newton step that leaves it, or two steps that do not halve it, give way to
// bisection.  Same stopping rules, so the answer meets the reference's
// tolerance, in about a seventh of ITP's evaluations; it is not the ITP
// iterate itself.
struct RootSolve {
    enum : int { kStart = 0, kBracket = 1, kNewton = 2, kDone = 3, kITP = 4 };
    int phase, dir, info;
    unsigned it;
    double x;  // next evaluation point
    double xlb, ylb, xub, yub, step, width, widthPrev, result;
    double nhalf;  // ITP: ceil(log2(0.5 (xub - xlb) / xtol)) of the initial bracket

    __device__ void start(double x0) {
        phase = kStart;
        info = 0;
        x = x0;
    }
    // The state as kSaveDoubles doubles (a deferred solve continues from it).
    static constexpr int kSaveDoubles = kSolveStateDoubles;
    __device__ void save(double* d) const {
        d[0] = (double)phase; d[1] = (double)dir; d[2] = (double)info; d[3] = (double)it;
        d[4] = x; d[5] = xlb; d[6] = ylb; d[7] = xub; d[8] = yub; d[9] = step;
        d[10] = width; d[11] = widthPrev; d[12] = result; d[13] = nhalf;
    }
    __device__ void load(const double* d) {
        phase = (int)d[0]; dir = (int)d[1]; info = (int)d[2]; it = (unsigned)d[3];
        x = d[4]; xlb = d[5]; ylb = d[6]; xub = d[7]; yub = d[8]; step = d[9];
        width = d[10]; widthPrev = d[11]; result = d[12]; nhalf = d[13];
    }
    __device__ void finish(double r, int inf) {
        result = r;
        info = inf;
        phase = kDone;
    }
    // The bracket is found: the reference's check of it and the first ITP point.
    __device__ void bracketedITP(double yd, double xtol) {
        if ((ylb > yd) || (yub < yd)) { finish(__longlong_as_double(0x7ff8000000000000ULL), -2); return; }
        nhalf = ceil(log2(__ddiv_rn(__dmul_rn(0.5, __dsub_rn(xub, xlb)), xtol)));
        it = 0;
        x = itpPoint(xlb, xub, ylb, yub, nhalf, it, xtol);
        phase = kITP;
    }
    // The bracket is found: the checks before the solver loop and its first point.
    __device__ void bracketed(double yd, double xtol, double ftol) {
        if ((ylb > yd) || (yub < yd)) { finish(__longlong_as_double(0x7ff8000000000000ULL), -2); return; }
        if (fabs(ylb - yd) < ftol) { finish(xlb, 0); return; }
        if (fabs(yub - yd) < ftol) { finish(xub, 0); return; }
        if (((xub - xlb) < xtol) || ((yub - ylb) < ftol)) { finish(0.5 * (xub + xlb), 0); return; }
        double xc = xlb + (yd - ylb) * (xub - xlb) / (yub - ylb);  // secant point of the bracket
        if (!(xc > xlb && xc < xub)) xc = 0.5 * (xlb + xub);
        width = xub - xlb;
        widthPrev = 2.0 * width;
        it = 0;
        x = xc;
        phase = kNewton;
    }
    // Consumes y = f(x).  maxBracket < kBracketIts is a first-pass budget:
    // running out of it gives kInfoDeferred instead of "no bracket".
    template <class F>
    __device__ void step_(double y, double yd, const F& f, double xtol, double ftol, unsigned maxBracket,
                          int method) {
        const double nan = __longlong_as_double(0x7ff8000000000000ULL);
        if (phase == kITP) {
            // One iteration of InverseSingleBracket's loop (RootFinding.h:152-170).
            const double xc = x;
            if (fabs(y - yd) < ftol) { finish(xc, 0); return; }
            if (y > yd) { xub = xc; yub = y; }
            else { xlb = xc; ylb = y; }
            if (((xub - xlb) < xtol) || ((yub - ylb) < ftol)) { finish(0.5 * (xub + xlb), 0); return; }
            if (++it >= 10000u) { finish(0.5 * (xub + xlb), 0); return; }
            x = itpPoint(xlb, xub, ylb, yub, nhalf, it, xtol);
            return;
        }
        if (phase == kStart) {
            xlb = xub = x;
            ylb = yub = y;
            step = 1.0;
            it = 0;
            dir = (ylb > yd) ? -1 : 1;
            x = (dir < 0) ? xub - step : xlb + step;
            phase = kBracket;
            return;
        }
        if (phase == kBracket) {
            bool more;
            if (dir < 0) {
                xlb = x;
                ylb = y;
                if ((fabs((yub - ylb) / (xub - xlb)) < 1e-12) && ((xub - xlb) > 10)) { finish(nan, -2); return; }
                more = ylb > yd;
                if (more) { yub = ylb; xub = xlb; step *= 2.0; }
            } else {
                xub = x;
                yub = y;
                if ((fabs((yub - ylb) / (xub - xlb)) < 1e-12) && ((xub - xlb) > 10)) { finish(nan, -2); return; }
                more = yub < yd;
                if (more) { ylb = yub; xlb = xub; step *= 2.0; }
            }
            if (!more) {
                if (method == kInverseITP) bracketedITP(yd, xtol);
                else bracketed(yd, xtol, ftol);
                return;
            }
            if (++it >= maxBracket) {
                // Out of a first-pass budget: the result is a root estimate
                // for ordering the second pass (a Newton step from here).
                if (maxBracket < kBracketIts) finish(x + (yd - y) / f.slope(x), kInfoDeferred);
                else finish(nan, -2);
                return;
            }
            x = (dir < 0) ? xub - step : xlb + step;
            return;
        }
        // Newton / bisection (at most 10000 evaluations).
        const double xc = x;
        if (fabs(y - yd) < ftol) { finish(xc, 0); return; }
        if (y > yd) { xub = xc; yub = y; }
        else { xlb = xc; ylb = y; }
        if (((xub - xlb) < xtol) || ((yub - ylb) < ftol)) { finish(0.5 * (xub + xlb), 0); return; }
        const double w = xub - xlb;
        double xn = xc - (y - yd) / f.slope(xc);
        // Bisection when Newton leaves the bracket or the bracket shrinks too slowly.
        if (!(xn > xlb && xn < xub) || w > 0.5 * widthPrev) xn = 0.5 * (xlb + xub);
        widthPrev = width;
        width = w;
        x = xn;
        if (++it >= 10000u) finish(0.5 * (xub + xlb), 0);
    }
};

// Solves f(x) = yd for the lanes with `need` set; every lane of the warp
// takes part in the loop (the step count is the warp's maximum), and in each
// step the lanes still solving evaluate f together.
template <class F>
__device__ __forceinline__ void solveLockstep(bool need, const F& f, double yd, double x0, double xtol, double ftol,
                                              unsigned maxBracket, int method, double& result, int& info) {
    RootSolve rs;
    if (need) rs.start(x0);
    while (__any_sync(0xffffffffu, need)) {
        if (need) {
            const double y = f(rs.x);
            rs.step_(y, yd, f, xtol, ftol, maxBracket, method);
            need = rs.phase != RootSolve::kDone;
            if (!need) {
                result = rs.result;
                info = rs.info;
            }
        }
    }
}

template <int BASIS, int POS, int PMAX>
__global__ void __launch_bounds__(256) inverseKernel(const __grid_constant__ InverseParams prm) {
    extern __shared__ double smem[];
    const int tid = threadIdx.x;
    const int tpb = blockDim.x;
    const SmemLayout L = carveSmem(smem, tpb, prm.dmax, prm.nBmax, prm.depthMax, PMAX, false);
    const long long slot = (long long)blockIdx.x * tpb + tid;
    const bool second = prm.listCount != nullptr;
    const long long n = second ? (long long)*prm.listCount : prm.N;
    const bool active = slot < n;
    // perm lists the points by increasing cost estimate; both passes take it
    // from the end, so the expensive blocks start first and the cheap ones
    // fill the tail of the launch.
    const long long i = !active ? slot : prm.perm ? (long long)prm.perm[n - 1 - slot] : slot;
    const int cStart = prm.compBegin;
    const int cEnd = prm.compEnd > 0 ? prm.compEnd : prm.nComps;
    const unsigned budget = (unsigned)prm.bracketBudget;
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const int inDim = prm.comps[prm.nComps - 1].D;
    // fullOut = [x1; 0] (TriangularMap.cpp:146-159); the coordinates of the
    // components solved before (earlier launches, or the first pass) come
    // from out.
    const long long xi = (prm.x1Cols == 1) ? 0 : i;
    for (int d = 0; d < inDim; ++d) {
        double v = 0.0;
        if (active) {
            if (d < prm.x1Rows) v = prm.x1[d * prm.x1Rs + xi * prm.x1Cs];
            else if (d - prm.extra < cStart) v = prm.out[(long long)(d - prm.extra) * prm.outRs + i * prm.outCs];
        }
        L.X[d * tpb + tid] = v;
    }
    int stAll = 0;
    bool stopped = !active;
    // Every thread runs every component (the warp-wide solver loop needs all
    // lanes); lanes that are inactive, stopped or before their start component
    // only take part in the loop.
    for (int ci = prm.compBegin; ci < cEnd; ++ci) {
        const CompDesc& c = prm.comps[ci];
        const bool mine = !stopped && ci >= cStart;
        const double* cm = prm.cm + c.slotOffset;
        ACoef<PMAX> A;
        if (mine && prm.acoef) {
#pragma unroll
            for (int k = 0; k <= PMAX; ++k) A.a[k] = prm.acoef[(long long)k * prm.N + i];
        } else if (mine) {
            fillLead<BASIS>(c, L, tid, prm.bc);
            if constexpr (BASIS == kBasisSigmoid) phaseARect<PMAX, POS>(c, L, tid, cm, A.a, nullptr);
            else phaseA<PMAX>(c, L, tid, cm, A.a);
        } else {
#pragma unroll
            for (int k = 0; k <= PMAX; ++k) A.a[k] = 0.0;
        }
        double result = nan;
        int info = 0;
        bool hasNan = false;
        for (int d = 0; mine && d < c.D; ++d) hasNan |= isnan(L.X[d * tpb + tid]);
        const double yd = mine ? prm.r[(long long)ci * prm.rRs + i * prm.rCs] : 0.0;
        const double x0 = mine ? L.X[(c.D - 1) * tpb + tid] : 0.0;
        if constexpr (BASIS == kBasisSigmoid) {
            // (RectifiedMultivariateExpansion.h:227-277; UnivariateExpansion.h:213-250.
            // A NaN target gives NaN.)
            SigmoidInverseEval<PMAX> f{A, c.P, &c};
            solveLockstep(mine && !hasNan && !isnan(yd), f, yd, x0, prm.xtol, prm.ytol, budget, prm.method, result, info);
        } else {
            double f0 = 0.0;
#pragma unroll
            for (int k = 0; k <= PMAX; ++k) f0 = fma(A.a[k], prm.bc.v0[k], f0);
            int st = 0;
            InverseEval<BASIS, POS, PMAX> f{A, c.P, f0, &prm.quad, &prm.bc, prm.nugget, &st};
            solveLockstep(mine && !hasNan, f, yd, x0, prm.xtol, prm.ytol, budget, prm.method, result, info);
            stAll |= st;
        }
        if (!mine) continue;
        if (info == kInfoDeferred) {
            // Out of the first pass's budget: the second pass solves the point.
            // result is a root estimate (a Newton step from the last bracket
            // point); the key orders the deferred points by its magnitude.
            const double kk = log2(1.0 + fabs(result));
            prm.deferKey[i] = isnan(kk) ? kDeferKeyMax : fmin(kk, kDeferKeyMax);
            atomicAdd(prm.deferCount, 1);
            stopped = true;
            continue;
        }
        if (info < 0) stAll |= kStatusNoBracket;
        L.X[(c.D - 1) * tpb + tid] = result;
        prm.out[(long long)ci * prm.outRs + i * prm.outCs] = result;
        if (prm.info) prm.info[(long long)ci * prm.infoStride + i] = info;
    }
    if (prm.statusWord && stAll) atomicOr(prm.statusWord, stAll);
}

// Queue pass: once the queue is empty, a solve that has taken kDrainNodes
// integrand nodes (or more) is left to the warp pass.
constexpr int kDrainNodes = 256;

// Inverse of one monotone component (compBegin) from a queue of points, one
// integrand node per lane and loop iteration.
//
// A lane owns one point at a time.  The adaptive quadrature of T at its
// solver's current iterate is a small state machine: the endpoint t = 1,
// then per interval the midpoint, the other interior coarse nodes and the
// fine-only nodes, then the accept test of AdaptiveClenshawCurtis::Integrate
// (Quadrature.h:819-968).  Every loop iteration each lane evaluates exactly
// one node, so the lanes of a warp evaluate the integrand together whatever
// the interval counts of their quadratures and the step counts of their
// solves (a lockstep solver waits for the slowest lane at every quadrature
// and every step).  A lane whose solve ends writes the root and takes the
// next point; one atomic per warp serves all its lanes that need one.  The
// points come in perm order from the expensive end (root estimates from the
// key pass), so the launch ends on cheap points.  Solves that grow too long,
// meet too wide a quadrature or are still running once the queue is empty go,
// with their solver state, to the warp pass (inverseWarpKernel).  A Newton
// step's slope is read off the quadrature's t = 1 node.
//
// The operations of each quadrature are those of `integrate`, in the same
// order, so T and the solver's iterates are those of one sequential solve.
// t = 0 is the same node for every quadrature of a point:
// h(0) = x_D (g(d_D f(x_<D, 0)) + nugget) is formed from its per-point factor.
template <int BASIS, int POS, int PMAX>
__global__ void __launch_bounds__(128) inverseQueueKernel(const __grid_constant__ InverseParams prm) {
    __shared__ double sOff[kMaxRulePts], sCw[kMaxRulePts], sFw[kMaxRulePts];
    __shared__ int sIsC[kMaxRulePts];
    __shared__ int sPer;
    const QuadParams& Q = prm.quad;
    const bool fixed = Q.kind == kQuadFixedCC;
    const int cR = Q.nCoarse - 1, cM = cR / 2, fR = Q.nFine - 1, fM = fR / 2;
    if (threadIdx.x == 0) {
        // Nodes of an interval after its midpoint, in the order of `integrate`.
        sOff[0] = 0.0; sCw[0] = 0.0; sFw[0] = 0.0; sIsC[0] = 1;
        int j = 1;
        for (int i = 1; i < cR; ++i) {
            if (i == cM) continue;
            sOff[j] = Q.cPts[i]; sCw[j] = Q.cWts[i]; sFw[j] = Q.fWts[2 * i]; sIsC[j] = 1;
            ++j;
        }
        for (int i = 1; i < Q.nFine; i += 2) {
            sOff[j] = Q.fPts[i]; sCw[j] = 0.0; sFw[j] = Q.fWts[i]; sIsC[j] = 0;
            ++j;
        }
        sPer = fixed ? Q.nFine : j;
    }
    __syncthreads();
    const int nPer = sPer;
    const int comp = prm.compBegin;
    const CompDesc& c = prm.comps[comp];
    const int D = c.D, P = c.P;
    const long long N = prm.N;
    const int lane = threadIdx.x & 31;
    const unsigned kFull = 0xffffffffu;
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const double nugget = prm.nugget;

    bool have = false, need = true;
    long long i = 0;
    double yd = 0.0, f0 = 0.0, G0 = 0.0;
    ACoef<PMAX> A;
    double as[PMAX + 1];
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) { A.a[k] = 0.0; as[k] = 0.0; }
    RootSolve rs;
    rs.phase = RootSolve::kDone;
    double xd = 0.0, lo = 0.0, hi = 1.0, hA = 0.0, hB = 0.0, hM = 0.0, ic = 0.0, ih = 0.0, Ih = 0.0, slopeB = 0.0;
    int level = 0, sp = 0, j = 0, qst = 0, stAll = 0;
    long long nInt = 0;
    int nodes = 0;  // integrand nodes of the current point's solve
    double stX[kMaxSubCap], stH[kMaxSubCap];
    int stL[kMaxSubCap];
    auto startQuad = [&](double xq) {
        xd = xq; lo = 0.0; hi = 1.0; level = 0; sp = 0; Ih = 0.0; nInt = 0; qst = 0;
        if (fixed) {
            j = 0;
        } else {
            hA = xd * G0;  // evalNode at t = 0
            if (isinf(G0)) qst |= kStatusInf;
            else if (isnan(hA)) qst |= kStatusNaN;
            j = -1;
        }
    };

    for (;;) {
        // Hand the next points to the lanes that need one.
        const unsigned needMask = __ballot_sync(kFull, need);
        if (needMask) {
            const int leader = __ffs(needMask) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(prm.queue, __popc(needMask));
            base = __shfl_sync(kFull, base, leader);
            if (need) {
                const long long slot = (long long)base + __popc(needMask & ((1u << lane) - 1u));
                need = false;
                if (slot < N) {
                    i = prm.perm ? (long long)prm.perm[N - 1 - slot] : slot;
                    // fullOut = [x1; outputs so far] (TriangularMap.cpp:146-184); the
                    // last coordinate is the initial guess.
                    const long long xi = (prm.x1Cols == 1) ? 0 : i;
                    bool hasNan = false;
                    double x0 = 0.0;
                    for (int d = 0; d < D; ++d) {
                        double v = 0.0;
                        if (d < prm.x1Rows) v = prm.x1[d * prm.x1Rs + xi * prm.x1Cs];
                        else if (d - prm.extra < comp) v = prm.out[(long long)(d - prm.extra) * prm.outRs + i * prm.outCs];
                        hasNan |= isnan(v);
                        x0 = v;
                    }
                    if (hasNan) {
                        // (MonotoneComponent.h:407-413)
                        prm.out[(long long)comp * prm.outRs + i * prm.outCs] = nan;
                        if (prm.info) prm.info[(long long)comp * prm.infoStride + i] = 0;
                        need = true;
                    } else {
                        yd = prm.r[(long long)comp * prm.rRs + i * prm.rCs];
                        f0 = 0.0;
#pragma unroll
                        for (int k = 0; k <= PMAX; ++k) {
                            A.a[k] = prm.acoef[(long long)k * N + i];
                            f0 = fma(A.a[k], prm.bc.v0[k], f0);
                        }
                        scaleCoeffs<BASIS, PMAX>(A.a, P, prm.bc, as);
                        NodeVal<PMAX, false, 0> V0;
                        int s0 = 0;
                        evalNode<BASIS, POS, PMAX, false, 0>(0.0, 1.0, as, P, prm.bc, nugget, V0, s0);
                        G0 = V0.h;
                        rs.start(x0);
                        startQuad(x0);
                        nodes = 0;
                        have = true;
                    }
                } else {
                    have = false;
                    // The queue is empty: from now on the launch ends with
                    // the solves still running, one lane each.
                    if (prm.drained) *(volatile int*)prm.drained = 1;
                }
            }
        }
        if (!__any_sync(kFull, have || need)) break;
        if (!have) continue;

        // One integrand node.
        double t, m = 0.0, s = 0.0;
        if (fixed) {
            t = 0.5 * (1.0 + Q.fPts[j]);
        } else if (j < 0) {
            t = 1.0;
        } else {
            m = 0.5 * (lo + hi);
            s = 0.5 * (hi - lo);
            t = (j == 0) ? m : m + s * sOff[j];
        }
        NodeVal<PMAX, false, 0> V;
        evalNode<BASIS, POS, PMAX, false, 0>(t, xd, as, P, prm.bc, nugget, V, qst);
        const double h = V.h;
        // An expensive solve -- a quadrature wider than wideQuad intervals
        // (a far iterate) or a solve longer than nodeBudget nodes -- is left
        // to the warp pass, which continues it with kWarpGroup lanes per
        // quadrature.
        // Once the queue is empty, solves past kDrainNodes nodes go too: the
        // warp pass runs them side by side, kWarpGroup lanes each, instead
        // of one lane each in a few warps.
        ++nodes;
        const bool drainedNow = prm.drained && (nodes & 63) == 0 && nodes >= kDrainNodes &&
                                *(volatile int*)prm.drained != 0;
        if (prm.nodeBudget > 0 && (nodes > prm.nodeBudget || nInt >= prm.wideQuad || drainedNow)) {
            // The solver's state as of the current quadrature's start goes
            // with the point (its earlier steps are not repeated).
            const int slot = atomicAdd(prm.deferCount, 1);
            prm.deferList[slot] = (int)i;
            if (prm.deferState && slot < prm.deferStateCap) rs.save(prm.deferState + (long long)slot * RootSolve::kSaveDoubles);
            have = false;
            need = true;
            continue;
        }
        bool qdone = false;
        double T = 0.0;
        if (fixed) {
            Ih = fma(0.5 * Q.fWts[j], h, Ih);
            if (++j == nPer) {
                qdone = true;
                T = (qst & (kStatusInf | kStatusNaN)) ? nan : Ih;
            }
        } else if (j < 0) {
            hB = h;
            slopeB = V.gn;
            if (qst & (kStatusInf | kStatusNaN)) { qdone = true; T = nan; }
            else j = 0;
        } else {
            // The interval's sums, as `integrate` forms them: at the midpoint
            // (j = 0) ic = (s c_0) hA + (s c_M) hM + (s c_R) hB and ih likewise
            // with the fine weights; at a later node one more product.  Both
            // cases as one sequence of selects, so that the lanes of a warp at
            // different nodes issue one path.
            const bool mid = (j == 0);
            if (mid) hM = h;
            const double cwj = mid ? Q.cWts[cM] : sCw[j];
            const double fwj = mid ? Q.fWts[fM] : sFw[j];
            const double icA = (s * Q.cWts[0]) * hA, ihA = (s * Q.fWts[0]) * hA;
            const double icN = fma(s * cwj, h, mid ? icA : ic);
            const double ihN = fma(s * fwj, h, mid ? ihA : ih);
            const double icB = fma(s * Q.cWts[cR], hB, icN), ihB = fma(s * Q.fWts[fR], hB, ihN);
            ic = mid ? icB : (sIsC[j] ? icN : ic);
            ih = mid ? ihB : ihN;
            if (++j == nPer) {
                j = 0;
                if (qst & (kStatusInf | kStatusNaN)) {
                    qdone = true;
                    T = nan;
                } else {
                    const double err = fabs(ih - ic);
                    const double tol = fmax(Q.relTol * fabs(ic), Q.absTol);
                    const bool accept = ((err < tol) || (level == Q.maxSub - 1)) && (level >= Q.minSub);
                    if (accept) {
                        Ih += ih;
                        if (sp == 0) {
                            qdone = true;
                            T = Ih;
                        } else {
                            --sp;
                            lo = hi;
                            hA = hB;
                            hi = stX[sp];
                            level = stL[sp];
                            hB = stH[sp];
                        }
                    } else {
                        stX[sp] = hi;
                        stL[sp] = level + 1;
                        stH[sp] = hB;
                        ++sp;
                        hi = m;
                        hB = hM;
                        ++level;
                    }
                    if (!qdone && ++nInt >= Q.maxIntervals) {
                        qst |= kStatusBudget;
                        qdone = true;
                        T = nan;
                    }
                }
            }
        }
        if (!qdone) continue;
        // The quadrature is done: one solver step with T(x) = integral + f(x_<D, 0).
        stAll |= qst;
        if (fixed) {
            int dummy = 0;
            const InverseEval<BASIS, POS, PMAX> f{A, P, f0, &prm.quad, &prm.bc, nugget, &dummy};
            rs.step_(T + f0, yd, f, prm.xtol, prm.ytol, kBracketIts, prm.method);
        } else {
            rs.step_(T + f0, yd, KnownSlope{slopeB}, prm.xtol, prm.ytol, kBracketIts, prm.method);
        }
        if (rs.phase == RootSolve::kDone) {
            prm.out[(long long)comp * prm.outRs + i * prm.outCs] = rs.result;
            if (prm.info) prm.info[(long long)comp * prm.infoStride + i] = rs.info;
            if (rs.info < 0) stAll |= kStatusNoBracket;
            have = false;
            need = true;
        } else {
            startQuad(rs.x);
        }
    }
    if (prm.statusWord && stAll) atomicOr(prm.statusWord, stAll);
}

// Inverse of the points the queue pass left over (deferList), one group of
// G lanes per point (G = kWarpGroup; 32 / G points per warp), each solve
// continuing from the state the queue pass saved for it (deferState).  The solver
// state is the same in every lane of a group; each quadrature of T is shared
// by the group's lanes: the pending intervals live on a per-group stack in
// global scratch (prm.stack, the leftmost on top), each round the lanes take
// the top min(G, depth) entries, evaluate one interval each (its midpoint,
// other coarse nodes and fine-only nodes, as `integrate`) and replace it by
// its two halves or by an accepted marker; accepted markers that reach the
// top are added to the integral in order.  The intervals, their values, the
// accept tests and the order of the sum of accepted fine values are those of
// the depth-first `integrate`, so T -- and every solver iterate -- is bitwise
// the same as in one lane.  Near the stack's capacity the rounds take one
// interval (a depth-first walk needs at most maxSub more entries).
template <int BASIS, int POS, int PMAX>
__global__ void __launch_bounds__(128) inverseWarpKernel(const __grid_constant__ InverseParams prm) {
    constexpr int G = kWarpGroup;
    static_assert(G == 4 || G == 8 || G == 16 || G == 32, "group size");
    __shared__ double sOff[kMaxRulePts], sCw[kMaxRulePts], sFw[kMaxRulePts];
    __shared__ int sIsC[kMaxRulePts];
    __shared__ int sPer;
    const QuadParams& Q = prm.quad;
    const bool fixed = Q.kind == kQuadFixedCC;
    const int cR = Q.nCoarse - 1, cM = cR / 2, fR = Q.nFine - 1, fM = fR / 2;
    if (threadIdx.x == 0) {
        int j = 1;
        for (int i = 1; i < cR; ++i) {
            if (i == cM) continue;
            sOff[j] = Q.cPts[i]; sCw[j] = Q.cWts[i]; sFw[j] = Q.fWts[2 * i]; sIsC[j] = 1;
            ++j;
        }
        for (int i = 1; i < Q.nFine; i += 2) {
            sOff[j] = Q.fPts[i]; sCw[j] = 0.0; sFw[j] = Q.fWts[i]; sIsC[j] = 0;
            ++j;
        }
        sPer = j;
    }
    __syncthreads();
    const int nPer = sPer;
    const int comp = prm.compBegin;
    const CompDesc& c = prm.comps[comp];
    const int D = c.D, P = c.P;
    const long long N = prm.N;
    const int lane = threadIdx.x & 31;
    const int gl = lane % G;  // lane within the group
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane - gl));
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const double nugget = prm.nugget;
    const int cap = prm.stackCap;
    const long long group = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    QEntry* stk = prm.stack + group * cap;
    const int listN = *prm.listCount;
    int stAll = 0;

    for (;;) {
        int k = 0;
        if (gl == 0) k = atomicAdd(prm.queue, 1);
        k = __shfl_sync(gmask, k, 0, G);
        if (k >= listN) break;
        const long long i = prm.deferList[k];
        // The point (the same in every lane of the group).
        const long long xi = (prm.x1Cols == 1) ? 0 : i;
        double x0 = 0.0;
        for (int d = 0; d < D; ++d) {
            double v = 0.0;
            if (d < prm.x1Rows) v = prm.x1[d * prm.x1Rs + xi * prm.x1Cs];
            else if (d - prm.extra < comp) v = prm.out[(long long)(d - prm.extra) * prm.outRs + i * prm.outCs];
            x0 = v;
        }
        const double yd = prm.r[(long long)comp * prm.rRs + i * prm.rCs];
        ACoef<PMAX> A;
        double f0 = 0.0;
#pragma unroll
        for (int kk = 0; kk <= PMAX; ++kk) {
            A.a[kk] = prm.acoef[(long long)kk * N + i];
            f0 = fma(A.a[kk], prm.bc.v0[kk], f0);
        }
        double as[PMAX + 1];
        scaleCoeffs<BASIS, PMAX>(A.a, P, prm.bc, as);
        double G0;
        {
            NodeVal<PMAX, false, 0> V0;
            int s0 = 0;
            evalNode<BASIS, POS, PMAX, false, 0>(0.0, 1.0, as, P, prm.bc, nugget, V0, s0);
            G0 = V0.h;
        }
        int dummy = 0;
        const InverseEval<BASIS, POS, PMAX> f{A, P, f0, &prm.quad, &prm.bc, nugget, &dummy};
        RootSolve rs;
        if (prm.deferState && k < prm.deferStateCap) rs.load(prm.deferState + (long long)k * RootSolve::kSaveDoubles);
        else rs.start(x0);
        while (rs.phase != RootSolve::kDone) {
            const double xd = rs.x;
            // T(x) - f0: the quadrature of x (g(df(t x)) + nugget) over t in [0, 1].
            int qst = 0;
            double Ih = 0.0;  // (group lane 0)
            bool failed = false;
            if (fixed) {
                // one fixed rule: the group's first lane alone
                if (gl == 0) {
                    for (int jn = 0; jn < Q.nFine; ++jn) {
                        NodeVal<PMAX, false, 0> V;
                        evalNode<BASIS, POS, PMAX, false, 0>(0.5 * (1.0 + Q.fPts[jn]), xd, as, P, prm.bc, nugget, V,
                                                             qst);
                        Ih = fma(0.5 * Q.fWts[jn], V.h, Ih);
                    }
                }
                qst = __shfl_sync(gmask, qst, 0, G);
                failed = (qst & (kStatusInf | kStatusNaN)) != 0;
            } else {
                const double hA0 = xd * G0;
                if (isinf(G0)) qst |= kStatusInf;
                else if (isnan(hA0)) qst |= kStatusNaN;
                NodeVal<PMAX, false, 0> VB;
                evalNode<BASIS, POS, PMAX, false, 0>(1.0, xd, as, P, prm.bc, nugget, VB, qst);
                failed = (qst & (kStatusInf | kStatusNaN)) != 0;
                int sp = 0;
                if (!failed) {
                    if (gl == 0) stk[0] = QEntry{0.0, hA0, VB.h, 0, 0};
                    sp = 1;
                    __syncwarp(gmask);
                }
                long long processed = 0;
                while (sp > 0) {
                    int m = min(G, sp);
                    if (sp + m > cap - kMaxSubCap - 2) m = 1;
                    const bool has = gl < m;
                    QEntry e{0.0, 0.0, 0.0, 0, 1};
                    if (has) e = stk[sp - 1 - gl];
                    __syncwarp(gmask);
                    const bool pend = has && !e.done;
                    double ic = 0.0, ih = 0.0, hM = 0.0, mm = 0.0;
                    int lst = 0;
                    bool accept = false;
                    if (pend) {
                        const double lo = e.lo, hi = e.lo + ldexp(1.0, -e.level);
                        mm = 0.5 * (lo + hi);
                        const double s = 0.5 * (hi - lo);
                        NodeVal<PMAX, false, 0> V;
                        evalNode<BASIS, POS, PMAX, false, 0>(mm, xd, as, P, prm.bc, nugget, V, lst);
                        hM = V.h;
                        ic = (s * Q.cWts[0]) * e.hA;
                        ic = fma(s * Q.cWts[cM], hM, ic);
                        ic = fma(s * Q.cWts[cR], e.hB, ic);
                        const double w0 = s * Q.fWts[0], wM = s * Q.fWts[fM], wR = s * Q.fWts[fR];
                        ih = w0 * e.hA;
                        ih = fma(wM, hM, ih);
                        ih = fma(wR, e.hB, ih);
                        for (int jn = 1; jn < nPer; ++jn) {
                            evalNode<BASIS, POS, PMAX, false, 0>(mm + s * sOff[jn], xd, as, P, prm.bc, nugget, V, lst);
                            if (sIsC[jn]) ic = fma(s * sCw[jn], V.h, ic);
                            ih = fma(s * sFw[jn], V.h, ih);
                        }
                        const double err = fabs(ih - ic);
                        const double tol = fmax(Q.relTol * fabs(ic), Q.absTol);
                        accept = ((err < tol) || (e.level == Q.maxSub - 1)) && (e.level >= Q.minSub);
                    }
                    qst |= __reduce_or_sync(gmask, lst);
                    if (qst & (kStatusInf | kStatusNaN)) {
                        failed = true;
                        break;
                    }
                    processed += __popc(__ballot_sync(gmask, pend) & gmask);
                    if (processed > Q.maxIntervals) {
                        qst |= kStatusBudget;
                        failed = true;
                        break;
                    }
                    // New entries, the leftmost on top: lane j's outputs lie
                    // below those of the lanes left of it.
                    const int nout = !has ? 0 : ((pend && !accept) ? 2 : 1);
                    int incl = nout;  // sum over the group's lanes >= this one
#pragma unroll
                    for (int off = 1; off < G; off <<= 1) {
                        const int v = __shfl_down_sync(gmask, incl, off, G);
                        if (gl + off < G) incl += v;
                    }
                    const int total = __shfl_sync(gmask, incl, 0, G);
                    const int base = sp - m + (incl - nout);
                    if (has) {
                        if (!pend) {
                            stk[base] = e;
                        } else if (accept) {
                            stk[base] = QEntry{e.lo, ih, 0.0, e.level, 1};
                        } else {
                            stk[base] = QEntry{mm, hM, e.hB, e.level + 1, 0};         // right half
                            stk[base + 1] = QEntry{e.lo, e.hA, hM, e.level + 1, 0};  // left half (on top)
                        }
                    }
                    sp = sp - m + total;
                    __syncwarp(gmask);
                    // Accepted intervals that reach the top, in order.
                    if (gl == 0) {
                        while (sp > 0) {
                            const QEntry t = stk[sp - 1];
                            if (!t.done) break;
                            Ih += t.hA;
                            --sp;
                        }
                    }
                    sp = __shfl_sync(gmask, sp, 0, G);
                    __syncwarp(gmask);
                }
            }
            stAll |= qst;
            double T = __shfl_sync(gmask, Ih, 0, G);
            if (failed) T = nan;
            rs.step_(T + f0, yd, f, prm.xtol, prm.ytol, kBracketIts, prm.method);
        }
        if (gl == 0) {
            prm.out[(long long)comp * prm.outRs + i * prm.outCs] = rs.result;
            if (prm.info) prm.info[(long long)comp * prm.infoStride + i] = rs.info;
            if (rs.info < 0) stAll |= kStatusNoBracket;
        }
    }
    if (gl == 0 && prm.statusWord && stAll) atomicOr(prm.statusWord, stAll);
}

// Key pass of the Inverse for component compBegin (monotone components):
// phase A of every point, kept in acoef for the solver launches, and the root
// estimate (r_c - T(x_<c, 0)) / dT/dx_D(x_<c, 0) of one Newton step from 0 as
// the sort key.  The quadratures of a point's solver steps cost in proportion
// to the range [0, x] they integrate, which the estimate predicts.
template <int BASIS, int POS, int PMAX>
__global__ void __launch_bounds__(256) inverseKeyKernel(const __grid_constant__ InverseParams prm) {
    extern __shared__ double smem[];
    const int tid = threadIdx.x;
    const int tpb = blockDim.x;
    const SmemLayout L = carveSmem(smem, tpb, prm.dmax, prm.nBmax, prm.depthMax, PMAX, false);
    const long long i = (long long)blockIdx.x * tpb + tid;
    if (i >= prm.N) return;  // no block-wide synchronisation below
    const CompDesc& c = prm.comps[prm.compBegin];
    const long long xi = (prm.x1Cols == 1) ? 0 : i;
    for (int d = 0; d < c.D; ++d) {
        double v = 0.0;
        if (d < prm.x1Rows) v = prm.x1[d * prm.x1Rs + xi * prm.x1Cs];
        else if (d - prm.extra < prm.compBegin) v = prm.out[(long long)(d - prm.extra) * prm.outRs + i * prm.outCs];
        L.X[d * tpb + tid] = v;
    }
    ACoef<PMAX> A;
    fillLead<BASIS>(c, L, tid, prm.bc);
    phaseA<PMAX>(c, L, tid, prm.cm + c.slotOffset, A.a);
    double f0 = 0.0;
#pragma unroll
    for (int k = 0; k <= PMAX; ++k) {
        prm.acoef[(long long)k * prm.N + i] = A.a[k];
        f0 = fma(A.a[k], prm.bc.v0[k], f0);
    }
    int st = 0;
    const InverseEval<BASIS, POS, PMAX> f{A, c.P, f0, &prm.quad, &prm.bc, prm.nugget, &st};
    const double yd = prm.r[(long long)prm.compBegin * prm.rRs + i * prm.rCs];
    prm.key[i] = (yd - f0) / f.slope(0.0);
}

// --------------------------------------------------------------------------
// Per-order launchers (instantiated in mpgb_inst_*.cu).
// --------------------------------------------------------------------------
template <int BASIS, int POS, int PMAX>
cudaError_t launchFusedP(const FusedParams& prm, int nItems, int needJ, int needE, cudaStream_t stream) {
    const bool input = (prm.flags & kFlagInput) != 0;
    const size_t smem = smemBytes(prm.tpb, prm.dmax, prm.nBmax, prm.depthMax, PMAX, input, prm.stageDoubles);
    auto run = [&](auto kern) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<nItems, prm.tpb, smem, stream>>>(prm);
        e = cudaGetLastError();
        countLaunches(stream, 1);
        return e;
    };
    if constexpr (BASIS == kBasisSigmoid) {
        (void)needJ;
        (void)needE;
        return run(fusedKernel<BASIS, POS, PMAX, false, 0>);
    } else {
        if (needE == 2) return run(fusedKernel<BASIS, POS, PMAX, true, 2>);
        if (needE) return run(fusedKernel<BASIS, POS, PMAX, true, 1>);
        if (needJ) return run(fusedKernel<BASIS, POS, PMAX, true, 0>);
        return run(fusedKernel<BASIS, POS, PMAX, false, 0>);
    }
}

// Persistent batch launch: as many blocks as fit on the device at once (at
// most one per item); `counter` must be zero on entry.
template <int BASIS, int POS>
cudaError_t launchBatchP(const FusedParams& prm, int nItems, int pmaxClass, int* counter, cudaStream_t stream) {
    const size_t smem = smemBytes(prm.tpb, prm.dmax, prm.nBmax, prm.depthMax, pmaxClass, false, prm.stageDoubles);
    void (*kern)(FusedParams, int, int*) = nullptr;
    switch (pmaxClass) {
        case 2: kern = batchKernel<BASIS, POS, 2>; break;
        case 4: kern = batchKernel<BASIS, POS, 4>; break;
        case 6: kern = batchKernel<BASIS, POS, 6>; break;
        case 8: kern = batchKernel<BASIS, POS, 8>; break;
        default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int perSM = 0, dev = 0, nSM = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, prm.tpb, smem)) != cudaSuccess) return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int grid = std::max(1, std::min(nItems, std::max(1, perSM) * nSM));
    kern<<<grid, prm.tpb, smem, stream>>>(prm, nItems, counter);
    e = cudaGetLastError();
    countLaunches(stream, 1);
    return e;
}

template <int BASIS, int POS, int PMAX>
cudaError_t launchInverseP(const InverseParams& prm, int nBlocks, cudaStream_t stream) {
    // Solver launches that read phase A from acoef use the coordinate rows of
    // the layout (its first part) only.
    const size_t smem = (prm.acoef && !prm.keyPass)
                            ? (size_t)prm.dmax * prm.tpb * sizeof(double)
                            : smemBytes(prm.tpb, prm.dmax, prm.nBmax, prm.depthMax, PMAX, false);
    void (*kern)(InverseParams) = inverseKernel<BASIS, POS, PMAX>;
    if (prm.keyPass) {
        if constexpr (BASIS == kBasisSigmoid) return cudaErrorInvalidValue;
        else kern = inverseKeyKernel<BASIS, POS, PMAX>;
    }
    if (prm.warpPass) {
        // Persistent: nBlocks blocks of four warps, 128 / kWarpGroup groups
        // each (the host sized the stack scratch for them).
        if constexpr (BASIS == kBasisSigmoid) {
            return cudaErrorInvalidValue;
        } else {
            if (!prm.queue || !prm.acoef || !prm.stack || !prm.listCount || !prm.deferList ||
                prm.stackCap < 4 * kMaxSubCap || nBlocks < 1)
                return cudaErrorInvalidValue;
            kern = inverseWarpKernel<BASIS, POS, PMAX>;
            kern<<<nBlocks, 128, 0, stream>>>(prm);
            cudaError_t e = cudaGetLastError();
            countLaunches(stream, 1);
            return e;
        }
    }
    if (prm.queuePass) {
        // Persistent: as many 128-thread blocks as are resident at once (at
        // most one per 128 points).
        if constexpr (BASIS == kBasisSigmoid) {
            return cudaErrorInvalidValue;
        } else {
            if (prm.tpb != 128 || !prm.queue || !prm.acoef) return cudaErrorInvalidValue;
            if (prm.nodeBudget > 0 && (!prm.deferList || !prm.deferCount)) return cudaErrorInvalidValue;
            kern = inverseQueueKernel<BASIS, POS, PMAX>;
            int perSM = 0, dev = 0, nSM = 0;
            cudaError_t e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, 128, 0)) != cudaSuccess) return e;
            if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            const long long need = (prm.N + 127) / 128;
            const int grid = (int)std::max(1LL, std::min(need, (long long)std::max(1, perSM) * nSM));
            kern<<<grid, 128, 0, stream>>>(prm);
            e = cudaGetLastError();
            countLaunches(stream, 1);
            return e;
        }
    }
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nBlocks, prm.tpb, smem, stream>>>(prm);
    e = cudaGetLastError();
    countLaunches(stream, 1);
    return e;
}

}  // namespace mpgb
