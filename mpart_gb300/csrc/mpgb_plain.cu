// Reference-structured ("plain") GPU path, kept as the comparator of the fused
// kernels.  It has the reference's structure on the device
// (MParT/MonotoneComponent.h:255-299, :487-531, :684-741, :824-874):
// one thread per point, a per-thread cache of 1-D basis values
// (MultivariateExpansionWorker.h:19-40), term loops over every term at every
// quadrature node, the adaptive Clenshaw-Curtis rule integrating the full
// fdim = numTerms + 1 vector with a per-thread workspace in global memory
// ((maxSub + 5) fdim + 2 maxSub doubles, Quadrature.h:786), dense
// numTerms x N outputs, and a separate launch per operation followed by
// column sums.  Nothing here is used by the fused path.
#include <cmath>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "mpgb_device.cuh"
#include "mpgb_launch.h"

namespace mpgb {
namespace plain {

struct PlainComp {
    int D, T, basis, pos;
    int cacheSize;
    int startPos[2 * 64 + 2];
    int maxDeg[64];
    const uint32_t* starts;
    const uint32_t* dims;
    const uint32_t* orders;
    const double* coeffs;
    double invNorm[kMaxLastOrder + 8];
    double nugget;
    QuadParams quad;
    int wsPerThread;  // doubles of scratch per thread
};

// EvaluateAll / EvaluateDerivatives (OrthogonalPolynomial.h:25-111, HermiteFunction.h:26-87).
__device__ void evalAll(const PlainComp& c, double* out, int p, double x) {
    if (c.basis == kBasisProbHermite) {
        out[0] = 1.0;
        if (p > 0) out[1] = x;
        for (int k = 2; k <= p; ++k) out[k] = x * out[k - 1] - (k - 1.0) * out[k - 2];
        for (int k = 0; k <= p; ++k) out[k] *= c.invNorm[k];
    } else {
        out[0] = 1.0;
        if (p > 0) {
            out[1] = x;
            if (p > 1) {
                out[2] = 0.75112554446494248286 * exp(-0.5 * x * x);
                if (p > 2) {
                    out[3] = 1.4142135623730951 * x * out[2];
                    for (int i = 2; i <= p - 2; ++i) out[i + 2] = (x * out[i + 1] - sqrt(0.5 * (i - 1)) * out[i]) / sqrt(0.5 * i);
                }
            }
        }
    }
}

__device__ void evalDerivs(const PlainComp& c, double* v, double* d, int p, double x) {
    if (c.basis == kBasisProbHermite) {
        v[0] = 1.0;
        d[0] = 0.0;
        if (p > 0) { v[1] = x; d[1] = 1.0; }
        for (int k = 2; k <= p; ++k) {
            v[k] = x * v[k - 1] - (k - 1.0) * v[k - 2];
            d[k] = v[k - 1] + x * d[k - 1] - (k - 1.0) * d[k - 2];
        }
        for (int k = 0; k <= p; ++k) { v[k] *= c.invNorm[k]; d[k] *= c.invNorm[k]; }
    } else {
        v[0] = 1.0;
        d[0] = 0.0;
        if (p > 0) {
            v[1] = x;
            d[1] = 1.0;
            if (p > 1) {
                double hm2 = 1.0, hm1 = 2.0 * x, dm2 = 0.0, dm1 = 2.0;
                const double e = 0.75112554446494248286 * exp(-0.5 * x * x);
                double fact = 1.0;
                for (int i = 0; i <= p - 2; ++i) {
                    double h, dh;
                    if (i == 0) { h = 1.0; dh = 0.0; }
                    else if (i == 1) { h = hm1; dh = dm1; }
                    else {
                        h = 2.0 * x * hm1 - 2.0 * (i - 1.0) * hm2;
                        dh = 2.0 * hm1 + 2.0 * x * dm1 - 2.0 * (i - 1.0) * dm2;
                        hm2 = hm1; hm1 = h; dm2 = dm1; dm1 = dh;
                    }
                    if (i > 0) fact *= i;
                    const double scale = e * pow(pow(2.0, (double)i) * fact, -0.5);
                    v[i + 2] = h * scale;
                    d[i + 2] = (dh - x * h) * scale;
                }
            }
        }
    }
}

__device__ double termProd(const PlainComp& c, int t, const double* cache, bool diag, bool& hasLast) {
    const int b = c.starts[t], e = c.starts[t + 1];
    hasLast = (e > b) && (int)c.dims[e - 1] == c.D - 1;
    double v = 1.0;
    for (int i = b; i < e - 1; ++i) v *= cache[c.startPos[c.dims[i]] + c.orders[i]];
    if (e > b) {
        const int posIndex = diag ? 2 * c.D - 1 : c.dims[e - 1];
        v *= cache[c.startPos[posIndex] + c.orders[e - 1]];
    }
    return v;
}

__device__ double posG(int pos, double x) {
    return pos == kPosSoftPlus ? log(1.0 + exp(-fabs(x))) + fmax(x, 0.0) : exp(x);
}
__device__ double posGp(int pos, double x) {
    return pos == kPosSoftPlus ? (x < 0 ? exp(x) / (exp(x) + 1.0) : 1.0 / (1.0 + exp(-x))) : exp(x);
}

// MonotoneIntegrand::operator() for modes None (fdim 1) and Parameters (fdim T+1).
__device__ void integrand(const PlainComp& c, double* cache, double xd, bool params, double t, double* out) {
    evalDerivs(c, &cache[c.startPos[c.D - 1]], &cache[c.startPos[2 * c.D - 1]], c.maxDeg[c.D - 1], t * xd);
    double df = 0.0;
    for (int k = 0; k < c.T; ++k) {
        bool last;
        const bool cst = c.starts[k] == c.starts[k + 1];
        double tv = 0.0;
        if (!cst) {
            tv = termProd(c, k, cache, true, last);
            if (!last) tv = 0.0;
        }
        df += tv * c.coeffs[k];
        if (params) out[1 + k] = tv;
    }
    if (params) {
        const double sc = xd * posGp(c.pos, df);
        for (int k = 0; k < c.T; ++k) out[1 + k] *= sc;
    }
    // (The value-only use is Evaluate, which integrates without the nugget,
    // MonotoneComponent.h:290; CoeffGrad integrates with it, :721.)
    out[0] = xd * (posG(c.pos, df) + (params ? c.nugget : 0.0));
}

// AdaptiveClenshawCurtis::Integrate with the reference's workspace layout.
__device__ void accIntegrate(const PlainComp& c, double* ws, double* cache, double xd, bool params, int fdim,
                             double* res) {
    const QuadParams& Q = c.quad;
    for (int i = 0; i < fdim; ++i) res[i] = 0.0;
    unsigned currLevel = 0, currSegment = 0;
    double* leftFunc = &ws[0];
    integrand(c, cache, xd, params, 0.0, leftFunc);
    double* rightFunc = &ws[fdim];
    integrand(c, cache, xd, params, 1.0, rightFunc);
    double* fval = &ws[2 * fdim];
    double* intCoarse = &ws[3 * fdim];
    double* intFine = &ws[4 * fdim];
    ws[5 * fdim] = 0.0;
    ws[5 * fdim + 1] = 1.0;
    unsigned workStart = 5 * fdim;
    const int cR = Q.nCoarse - 1, cM = cR / 2, fR = Q.nFine - 1, fM = fR / 2;
    long long guard = 0;
    while (true) {
        const double lp = ws[workStart], rp = ws[workStart + 1];
        const double midPt = 0.5 * (lp + rp), scale = 0.5 * (rp - lp);
        double* midFunc = &ws[workStart + 2];
        integrand(c, cache, xd, params, midPt, midFunc);
        for (int i = 0; i < fdim; ++i) {
            intCoarse[i] = scale * Q.cWts[0] * leftFunc[i];
            intCoarse[i] += scale * Q.cWts[cM] * midFunc[i];
            intCoarse[i] += scale * Q.cWts[cR] * rightFunc[i];
            intFine[i] = scale * Q.fWts[0] * leftFunc[i];
            intFine[i] += scale * Q.fWts[fM] * midFunc[i];
            intFine[i] += scale * Q.fWts[fR] * rightFunc[i];
        }
        for (int i = 1; i < cR; ++i) {
            if (i == cM) continue;
            integrand(c, cache, xd, params, midPt + scale * Q.cPts[i], fval);
            for (int j = 0; j < fdim; ++j) {
                intCoarse[j] += scale * Q.cWts[i] * fval[j];
                intFine[j] += scale * Q.fWts[2 * i] * fval[j];
            }
        }
        for (int i = 1; i < Q.nFine; i += 2) {
            integrand(c, cache, xd, params, midPt + scale * Q.fPts[i], fval);
            for (int j = 0; j < fdim; ++j) intFine[j] += scale * Q.fWts[i] * fval[j];
        }
        const double err = fabs(intFine[0] - intCoarse[0]);
        const double tol = fmax(Q.relTol * fabs(intCoarse[0]), Q.absTol);
        if (isnan(err) || ++guard > Q.maxIntervals) {
            for (int i = 0; i < fdim; ++i) res[i] = __longlong_as_double(0x7ff8000000000000ULL);
            return;
        }
        if ((((err < tol) || ((int)currLevel == Q.maxSub - 1)) && ((int)currLevel >= Q.minSub))) {
            for (int i = 0; i < fdim; ++i) res[i] += intFine[i];
            while (((currSegment >> currLevel) & 1U) && (currLevel > 0)) {
                currSegment &= ~(1U << currLevel);
                currLevel--;
            }
            if (currLevel == 0) break;
            currSegment |= 1U << currLevel;
            workStart = (currLevel + 5) * fdim + 2 * currLevel;
            const unsigned prev = ((currLevel - 1) + 5) * fdim + 2 * (currLevel - 1);
            ws[workStart] = 0.5 * (ws[prev] + ws[prev + 1]);
            ws[workStart + 1] = ws[prev + 1];
            leftFunc = &ws[0];
            rightFunc = &ws[fdim];
            for (unsigned lv = 0; lv < currLevel; ++lv) {
                if ((currSegment >> (lv + 1)) & 1U) leftFunc = &ws[(lv + 5) * fdim + 2 * (lv + 1)];
                else rightFunc = &ws[(lv + 5) * fdim + 2 * (lv + 1)];
            }
        } else {
            currLevel++;
            rightFunc = midFunc;
            workStart = (currLevel + 5) * fdim + 2 * currLevel;
            ws[workStart] = lp;
            ws[workStart + 1] = midPt;
        }
    }
}

__device__ void fillCache1(const PlainComp& c, double* cache, const double* pts, long long rs, long long i) {
    for (int d = 0; d < c.D - 1; ++d) evalAll(c, &cache[c.startPos[d]], c.maxDeg[d], pts[d * rs + i]);
}

// mode 0 Evaluate, 1 log-det (ContinuousDerivative + log), 2 CoeffJacobian x sens,
// 3 ContinuousMixedJacobian / g (LogDeterminantCoeffGrad).
__global__ void plainKernel(const __grid_constant__ PlainComp c, int mode, const double* pts, long long rs,
                            long long N, const double* sens, double* out, double* dense, double* scratch) {
    const long long nThreads = (long long)gridDim.x * blockDim.x;
    const long long tIdx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double* cache = scratch + tIdx * c.wsPerThread;
    double* ws = cache + c.cacheSize;
    for (long long i = tIdx; i < N; i += nThreads) {
        fillCache1(c, cache, pts, rs, i);
        const double xd = pts[(c.D - 1) * rs + i];
        if (mode == 0) {
            double r;
            accIntegrate(c, ws, cache, xd, false, 1, &r);
            evalAll(c, &cache[c.startPos[c.D - 1]], c.maxDeg[c.D - 1], 0.0);
            double f = 0.0;
            for (int k = 0; k < c.T; ++k) {
                bool last;
                if (c.starts[k] == c.starts[k + 1]) { f += c.coeffs[k]; continue; }
                f += termProd(c, k, cache, false, last) * c.coeffs[k];
            }
            out[i] = r + f;
        } else if (mode == 1 || mode == 3) {
            evalDerivs(c, &cache[c.startPos[c.D - 1]], &cache[c.startPos[2 * c.D - 1]], c.maxDeg[c.D - 1], xd);
            double df = 0.0;
            for (int k = 0; k < c.T; ++k) {
                bool last;
                if (c.starts[k] == c.starts[k + 1]) {
                    if (mode == 3) dense[(long long)k * N + i] = 0.0;
                    continue;
                }
                double tv = termProd(c, k, cache, true, last);
                if (!last) tv = 0.0;
                df += tv * c.coeffs[k];
                if (mode == 3) dense[(long long)k * N + i] = tv;
            }
            const double g = posG(c.pos, df);
            if (mode == 1) {
                out[i] = (g <= 0) ? -INFINITY : log(g);
            } else {
                const double s = posGp(c.pos, df) * (1.0 / g);
                for (int k = 0; k < c.T; ++k) dense[(long long)k * N + i] *= s;
            }
        } else {
            const int fdim = c.T + 1;
            double* integral = ws + ((c.quad.maxSub + 5) * fdim + 2 * c.quad.maxSub);
            accIntegrate(c, ws, cache, xd, true, fdim, integral);
            evalAll(c, &cache[c.startPos[c.D - 1]], c.maxDeg[c.D - 1], 0.0);
            const double sv = sens[i];
            for (int k = 0; k < c.T; ++k) {
                bool last;
                double tv = 1.0;
                if (c.starts[k] != c.starts[k + 1]) tv = termProd(c, k, cache, false, last);
                dense[(long long)k * N + i] = (tv + integral[1 + k]) * sv;
            }
        }
    }
}

// Row sums of a dense T x N matrix (the reduction the reference leaves to its caller).
__global__ void rowSumKernel(const double* dense, int T, long long N, double* out, int accumulate) {
    __shared__ double red[256];
    const int row = blockIdx.x;
    double s = 0.0;
    for (long long i = threadIdx.x; i < N; i += blockDim.x) s += dense[(long long)row * N + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[row] = accumulate ? out[row] + red[0] : red[0];
}

}  // namespace plain
}  // namespace mpgb

// ---------------------------------------------------------------------------
// C ABI of the plain path (one total-order component, device memory only).
// ---------------------------------------------------------------------------
using namespace mpgb;
using namespace mpgb::plain;

namespace {
thread_local std::string g_plainErr;

void ccRuleP(unsigned n, double* w, double* p) {
    const double PI = 3.14159265358979323846;
    for (unsigned i = 0; i < n; ++i) p[i] = cos((n - (i + 1)) * PI / (n - 1));
    p[0] = -1.0;
    if (n % 2 == 1) p[(n - 1) / 2] = 0.0;
    p[n - 1] = 1.0;
    for (unsigned i = 0; i < n; ++i) {
        w[i] = 1.0;
        const double th = i * PI / (n - 1);
        for (unsigned j = 0; j < (n - 1) / 2; ++j) {
            const double b = (2 * (j + 1) == (n - 1)) ? 1.0 : 2.0;
            w[i] = w[i] - b * cos(2.0 * (j + 1) * th) / (4 * (j + 1) * (j + 1) - 1);
        }
    }
    w[0] /= (n - 1.0);
    for (unsigned i = 1; i < n - 1; ++i) w[i] = 2.0 * w[i] / (n - 1.0);
    w[n - 1] /= (n - 1.0);
}
}  // namespace

struct mpgb_plain {
    PlainComp c;
    uint32_t *dStarts = nullptr, *dDims = nullptr, *dOrders = nullptr;
    double* scratch = nullptr;
    double* dense = nullptr;
    size_t denseN = 0;
    int blocks = 0, threads = 128;
};

extern "C" {

int mpgb_plain_create(unsigned int dim, unsigned int order, const mpgb_map_options* o, mpgb_plain** out) {
    try {
        if (!out || !o || dim == 0 || dim > 64) throw std::invalid_argument("bad arguments");
        // total-order set in the reference's term order
        std::vector<unsigned> s, d, r, work(dim, 0);
        std::function<void(unsigned, unsigned)> rec = [&](unsigned cd, unsigned rem) {
            for (unsigned p = 0; p <= rem; ++p) {
                work[cd] = p;
                if (cd + 1 < dim) rec(cd + 1, rem - p);
                else {
                    s.push_back((unsigned)d.size());
                    for (unsigned i = 0; i < dim; ++i)
                        if (work[i]) { d.push_back(i); r.push_back(work[i]); }
                }
            }
        };
        rec(0, order);
        s.push_back((unsigned)d.size());
        auto* h = new mpgb_plain();
        PlainComp& c = h->c;
        c.D = (int)dim;
        c.T = (int)s.size() - 1;
        c.basis = o->basis_type;
        c.pos = o->pos_func_type;
        c.nugget = o->nugget;
        for (unsigned i = 0; i < dim; ++i) c.maxDeg[i] = (int)order;
        int up = 0;
        for (unsigned i = 0; i < 2 * dim + 2; ++i) {
            c.startPos[i] = up;
            up += (i < 2 * dim) ? c.maxDeg[i % dim] + 1 : c.maxDeg[dim - 1] + 1;
        }
        c.cacheSize = c.startPos[2 * dim + 1];
        for (int k = 0; k < kMaxLastOrder + 8; ++k) {
            double f = 1.0;
            for (int i = 2; i <= k; ++i) f *= i;
            c.invNorm[k] = o->basis_norm ? 1.0 / sqrt(sqrt(2.0 * 3.14159265358979323846) * f) : 1.0;
        }
        const unsigned level = (unsigned)std::log2((double)(o->quad_pts - 2));
        c.quad.nCoarse = (1 << level) + 1;
        c.quad.nFine = (1 << (level + 1)) + 1;
        ccRuleP(c.quad.nCoarse, c.quad.cWts, c.quad.cPts);
        ccRuleP(c.quad.nFine, c.quad.fWts, c.quad.fPts);
        c.quad.maxSub = (int)o->quad_max_sub;
        c.quad.minSub = (int)o->quad_min_sub;
        c.quad.absTol = o->quad_abs_tol;
        c.quad.relTol = o->quad_rel_tol;
        c.quad.maxIntervals = 1LL << 24;
        const int fdim = c.T + 1;
        c.wsPerThread = c.cacheSize + (c.quad.maxSub + 5) * fdim + 2 * c.quad.maxSub + fdim;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        h->blocks = sms * 2;
        auto up32 = [](const std::vector<unsigned>& v) {
            uint32_t* p = nullptr;
            cudaMalloc(&p, std::max<size_t>(1, v.size()) * 4);
            if (!v.empty()) cudaMemcpy(p, v.data(), v.size() * 4, cudaMemcpyHostToDevice);
            return p;
        };
        h->dStarts = up32(s);
        h->dDims = up32(d);
        h->dOrders = up32(r);
        c.starts = h->dStarts;
        c.dims = h->dDims;
        c.orders = h->dOrders;
        const size_t nThreads = (size_t)h->blocks * h->threads;
        if (cudaMalloc(&h->scratch, nThreads * c.wsPerThread * sizeof(double)) != cudaSuccess)
            throw std::runtime_error("plain path: scratch allocation failed");
        *out = h;
        return MPGB_OK;
    } catch (std::exception const& e) {
        g_plainErr = e.what();
        return MPGB_ERR_RUNTIME;
    }
}

int mpgb_plain_destroy(mpgb_plain* h) {
    if (!h) return MPGB_OK;
    cudaFree(h->dStarts);
    cudaFree(h->dDims);
    cudaFree(h->dOrders);
    cudaFree(h->scratch);
    cudaFree(h->dense);
    delete h;
    return MPGB_OK;
}

int mpgb_plain_num_terms(const mpgb_plain* h, unsigned int* n) {
    if (!h || !n) return MPGB_ERR_INVALID_ARGUMENT;
    *n = (unsigned)h->c.T;
    return MPGB_OK;
}

int mpgb_plain_fwd_adj(mpgb_plain* h, const double* coeffs, const double* pts, long long N, const double* sens,
                       double* out_eval, double* out_logdet, double* coeff_grad, void* stream) {
    if (!h || !coeffs || !pts || N <= 0) return MPGB_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    PlainComp c = h->c;
    c.coeffs = coeffs;
    if (h->denseN < (size_t)N) {
        cudaStreamSynchronize(s);
        cudaFree(h->dense);
        h->dense = nullptr;
        if (cudaMalloc(&h->dense, (size_t)c.T * N * sizeof(double)) != cudaSuccess) return MPGB_ERR_CUDA;
        h->denseN = N;
    }
    const long long rs = N;
    if (out_eval) plainKernel<<<h->blocks, h->threads, 0, s>>>(c, 0, pts, rs, N, nullptr, out_eval, nullptr, h->scratch);
    if (out_logdet) plainKernel<<<h->blocks, h->threads, 0, s>>>(c, 1, pts, rs, N, nullptr, out_logdet, nullptr, h->scratch);
    if (coeff_grad) {
        plainKernel<<<h->blocks, h->threads, 0, s>>>(c, 2, pts, rs, N, sens, nullptr, h->dense, h->scratch);
        rowSumKernel<<<c.T, 256, 0, s>>>(h->dense, c.T, N, coeff_grad, 0);
        plainKernel<<<h->blocks, h->threads, 0, s>>>(c, 3, pts, rs, N, nullptr, nullptr, h->dense, h->scratch);
        rowSumKernel<<<c.T, 256, 0, s>>>(h->dense, c.T, N, coeff_grad, 1);
    }
    const cudaError_t e = cudaGetLastError();
    mpgb::countLaunches(s, (out_eval ? 1 : 0) + (out_logdet ? 1 : 0) + (coeff_grad ? 4 : 0));
    return e == cudaSuccess ? MPGB_OK : MPGB_ERR_CUDA;
}

}  // extern "C"
