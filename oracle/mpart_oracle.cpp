// ============================================================================
// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of MParT's per-point monotone-component path, written to
// follow the reference's operation order and summation order so that it can
// serve as the parity checker for the GPU product.  Only tests/, the smoke()
// entry point and bench.py's CPU-baseline leg may load this library.  The
// product path never links, loads or calls it.
//
// Parity pin: the reference cannot be compiled here (Kokkos 4.2, Eigen 3.4,
// NLopt 2.7.1, cereal 1.3.2 and Catch2 3.2.1 are all absent).  This
// restatement is pinned by porting the reference's own known-answer tests
// (closed forms, FD consistency, cross-routine identities); see
// tests/test_oracle_pins.py.
//
// Compile with -ffp-contract=off so that every a*b+c is rounded twice, as the
// reference's host build does on x86-64 without -march flags.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#include <algorithm>
#include <functional>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

static const double kPi = 3.14159265358979323846;

// ----------------------------------------------------------------------------
// FixedMultiIndexSet, total-order constructor.
// Follows src/MultiIndices/FixedMultiIndexSet.cpp:208-233 (constructor),
// :488-506 (TotalOrderSize) and :508-549 (FillTotalOrder): dimension 0 is the
// outermost loop, the last dimension varies fastest, and each term lists its
// nonzero (dim, order) pairs in increasing dim.
// ----------------------------------------------------------------------------
struct MultiSet {
    unsigned dim = 0;
    std::vector<unsigned> starts, dims, orders, maxDeg;
    unsigned size() const { return (unsigned)starts.size() - 1; }

    void calcMaxDegrees() {
        maxDeg.assign(dim, 0);
        for (size_t i = 0; i < orders.size(); ++i)
            maxDeg[dims[i]] = std::max(maxDeg[dims[i]], orders[i]);
    }
};

static void fillTotalOrder(MultiSet& ms, unsigned maxOrder, unsigned minOrder,
                           std::vector<unsigned>& work, unsigned currDim,
                           unsigned& currTerm, unsigned& currNz) {
    if (currDim < ms.dim - 1) {
        for (unsigned pow = 0; pow <= maxOrder; ++pow) {
            work[currDim] = pow;
            fillTotalOrder(ms, maxOrder - pow, minOrder, work, currDim + 1, currTerm, currNz);
        }
    } else {
        for (unsigned pow = 0; pow <= maxOrder; ++pow) {
            work[currDim] = pow;
            unsigned currOrder = 0;
            for (unsigned i = 0; i < currDim + 1; ++i) currOrder += work[i];
            if (currOrder >= minOrder) {
                ms.starts.push_back(currNz);
                for (unsigned i = 0; i < ms.dim; ++i) {
                    if (work[i] > 0) {
                        ms.dims.push_back(i);
                        ms.orders.push_back(work[i]);
                        currNz++;
                    }
                }
                currTerm++;
            }
        }
    }
    if (currDim == 0) ms.starts.push_back(currNz);
}

static MultiSet totalOrder(unsigned dim, unsigned maxOrder, unsigned minOrder = 0) {
    MultiSet ms;
    ms.dim = dim;
    std::vector<unsigned> work(dim, 0);
    unsigned currTerm = 0, currNz = 0;
    fillTotalOrder(ms, maxOrder, minOrder, work, 0, currTerm, currNz);
    ms.calcMaxDegrees();
    return ms;
}

// ----------------------------------------------------------------------------
// Factorial as an unsigned int product (MParT/Utilities/MathFunctions.h).
// ----------------------------------------------------------------------------
static unsigned factorialU(unsigned d) {
    unsigned out = 1;
    for (unsigned i = 2; i <= d; ++i) out *= i;
    return out;
}

// ----------------------------------------------------------------------------
// Probabilist Hermite polynomials: OrthogonalPolynomial<ProbabilistHermiteMixer>
// (MParT/OrthogonalPolynomial.h:25-156, mixer :294-309).  a_k=1, b_k=0,
// c_k=k-1, optional division by sqrt(sqrt(2 pi) k!).
// Physicist Hermite (mixer :312-327): a_k=2, b_k=0, c_k=2(k-1), phi1=2x.
// ----------------------------------------------------------------------------
struct Poly {
    bool physicist = false;
    bool normalize = false;
    double ak(unsigned) const { return physicist ? 2.0 : 1.0; }
    double bk(unsigned) const { return 0.0; }
    double ck(unsigned k) const { return physicist ? 2.0 * (k - 1.0) : k - 1.0; }
    double phi0(double) const { return 1.0; }
    double phi1(double x) const { return physicist ? 2.0 * x : x; }
    double phi1d(double) const { return physicist ? 2.0 : 1.0; }
    double norm(unsigned k) const {
        if (physicist) return std::sqrt(std::sqrt(kPi) * std::pow(2.0, (double)k) * factorialU(k));
        return std::sqrt(std::sqrt(2.0 * kPi) * factorialU(k));
    }

    void evalAll(double* out, unsigned maxOrder, double x) const {
        out[0] = phi0(x);
        if (maxOrder > 0) out[1] = phi1(x);
        for (unsigned k = 2; k <= maxOrder; ++k)
            out[k] = (ak(k) * x + bk(k)) * out[k - 1] - ck(k) * out[k - 2];
        if (normalize)
            for (unsigned k = 0; k <= maxOrder; ++k) out[k] /= norm(k);
    }
    void evalDerivs(double* vals, double* derivs, unsigned maxOrder, double x) const {
        vals[0] = phi0(x);
        derivs[0] = 0.0;
        if (maxOrder > 0) { vals[1] = phi1(x); derivs[1] = phi1d(x); }
        for (unsigned k = 2; k <= maxOrder; ++k) {
            double a = ak(k), b = bk(k), c = ck(k);
            vals[k] = (a * x + b) * vals[k - 1] - c * vals[k - 2];
            derivs[k] = a * vals[k - 1] + (a * x + b) * derivs[k - 1] - c * derivs[k - 2];
        }
        if (normalize)
            for (unsigned k = 0; k <= maxOrder; ++k) {
                double n = norm(k);
                vals[k] /= n;
                derivs[k] /= n;
            }
    }
    void evalSecond(double* vals, double* derivs, double* d2, unsigned maxOrder, double x) const {
        vals[0] = phi0(x);
        derivs[0] = 0.0;
        d2[0] = 0.0;
        if (maxOrder > 0) { vals[1] = phi1(x); derivs[1] = phi1d(x); d2[1] = 0.0; }
        for (unsigned k = 2; k <= maxOrder; ++k) {
            double a = ak(k), b = bk(k), c = ck(k);
            vals[k] = (a * x + b) * vals[k - 1] - c * vals[k - 2];
            derivs[k] = a * vals[k - 1] + (a * x + b) * derivs[k - 1] - c * derivs[k - 2];
            d2[k] = a * derivs[k - 1] + a * derivs[k - 1] + (a * x + b) * d2[k - 1] - c * d2[k - 2];
        }
        if (normalize)
            for (unsigned k = 0; k <= maxOrder; ++k) {
                double n = norm(k);
                vals[k] /= n;
                derivs[k] /= n;
                d2[k] /= n;
            }
    }
};

// ----------------------------------------------------------------------------
// Hermite functions (MParT/HermiteFunction.h:22-104): phi_0=1, phi_1=x,
// phi_{k+2}=psi_k (normalised Hermite functions).  EvaluateAll uses the
// normalised three-term recurrence; EvaluateDerivatives goes through the
// unnormalised physicist polynomials and rescales -- the two give slightly
// different roundings of the values and both are reproduced.
// ----------------------------------------------------------------------------
struct HermiteFn {
    Poly base{true, false};
    void evalAll(double* out, unsigned maxOrder, double x) const {
        out[0] = 1.0;
        if (maxOrder > 0) {
            out[1] = x;
            if (maxOrder > 1) {
                out[2] = std::pow(kPi, -0.25) * std::exp(-0.5 * x * x);
                if (maxOrder > 2) {
                    out[3] = std::sqrt(2.0) * x * out[2];
                    for (unsigned i = 2; i <= maxOrder - 2; ++i)
                        out[i + 2] = (x * out[i + 1] - std::sqrt(0.5 * (i - 1)) * out[i]) / std::sqrt(0.5 * i);
                }
            }
        }
    }
    void evalDerivs(double* vals, double* derivs, unsigned maxOrder, double x) const {
        vals[0] = 1.0;
        derivs[0] = 0.0;
        if (maxOrder > 0) {
            vals[1] = x;
            derivs[1] = 1.0;
            if (maxOrder > 1) {
                base.evalDerivs(&vals[2], &derivs[2], maxOrder - 2, x);
                const double baseScaling = std::pow(kPi, -0.25) * std::exp(-0.5 * x * x);
                double scale;
                double currFactorial = 1;
                scale = baseScaling;
                derivs[2] -= x * vals[2];
                derivs[2] *= scale;
                vals[2] *= scale;
                for (unsigned i = 1; i <= maxOrder - 2; ++i) {
                    currFactorial *= i;
                    scale = baseScaling * std::pow(std::pow(2, i) * currFactorial, -0.5);
                    derivs[i + 2] -= x * vals[i + 2];
                    derivs[i + 2] *= scale;
                    vals[i + 2] *= scale;
                }
            }
        }
    }
    void evalSecond(double* vals, double* derivs, double* d2, unsigned maxOrder, double x) const {
        evalDerivs(vals, derivs, maxOrder, x);
        d2[0] = 0.0;
        if (maxOrder > 0) {
            d2[1] = 0.0;
            if (maxOrder > 1)
                for (unsigned i = 0; i <= maxOrder - 2; ++i)
                    d2[i + 2] = -(2.0 * i + 1.0 - x * x) * vals[i + 2];
        }
    }
};

enum BasisKind { kProbHermite = 0, kHermiteFunctions = 2 };
enum PosKind { kExp = 0, kSoftPlus = 1 };

struct Basis1d {
    int kind = kProbHermite;
    Poly prob{false, true};
    HermiteFn hf;
    void evalAll(double* o, unsigned p, double x) const { if (kind == kProbHermite) prob.evalAll(o, p, x); else hf.evalAll(o, p, x); }
    void evalDerivs(double* v, double* d, unsigned p, double x) const { if (kind == kProbHermite) prob.evalDerivs(v, d, p, x); else hf.evalDerivs(v, d, p, x); }
    void evalSecond(double* v, double* d, double* d2, unsigned p, double x) const { if (kind == kProbHermite) prob.evalSecond(v, d, d2, p, x); else hf.evalSecond(v, d, d2, p, x); }
};

// ----------------------------------------------------------------------------
// Positive bijectors (MParT/PositiveBijectors.h:12-57).
// ----------------------------------------------------------------------------
static double posEval(int kind, double x) {
    if (kind == kSoftPlus) return std::log(1.0 + std::exp(-1.0 * std::abs(x))) + std::fmax(x, 0.0);
    return std::exp(x);
}
static double posDeriv(int kind, double x) {
    if (kind == kSoftPlus) return x < 0 ? std::exp(x) / (std::exp(x) + 1.0) : 1.0 / (1.0 + std::exp(-1.0 * x));
    return std::exp(x);
}
static double posSecondDeriv(int kind, double x) {
    if (kind == kSoftPlus) {
        const double fx = posDeriv(kind, x);
        return fx * (1.0 - fx);
    }
    return std::exp(x);
}

// ----------------------------------------------------------------------------
// Sigmoid1d (MParT/Sigmoid.h:87-446) with the Logistic sigmoid (:23-40) and
// SoftPlus edge terms: f_0 = 1, f_1 = x, f_2 = -w_0 g(-b_0 (x - c_0)),
// f_3 = w_1 g(b_1 (x - c_1)), f_k = sum_j w_j s(b_j (x - c_j)) over the
// centers of term k (starting indices as in CSR).  The product of each
// weight/width factor is formed left to right as in the reference.
// ----------------------------------------------------------------------------
struct Sigmoid1d {
    std::vector<double> centers, widths, weights;
    std::vector<unsigned> starts;
    int order = 0;

    static double logistic(double x) { return 0.5 + 0.5 * std::tanh(x / 2); }
    static double logisticD(double x) {
        double fx = logistic(x);
        return fx * (1 - fx);
    }
    static double logisticD2(double x) {
        double fx = logistic(x);
        return fx * (1 - fx) * (1 - 2 * fx);
    }
    // ConstructStartInds (:95-130).  Returns false when the Linear sum type
    // does not fit the number of centers.
    static int numSigmoids(unsigned numCenters, int sumType) {
        if (sumType == 1) return (int)numCenters - 2;
        return (int)((std::sqrt(1 + 8 * ((double)numCenters - 2)) - 1) / 2);
    }
    static bool constructStarts(unsigned centerSize, int sumType, std::vector<unsigned>& out) {
        out.clear();
        int numTerms = numSigmoids(centerSize, sumType);
        if (centerSize <= 2) return true;
        if (sumType == 0) {
            if ((int)(centerSize - 2) != (numTerms * (numTerms + 1) / 2)) return false;
            out.resize(numTerms);
            out[0] = 2;
            for (int i = 1; i < numTerms; ++i) out[i] = out[i - 1] + i;
        } else {
            numTerms = (int)centerSize - 2;
            out.resize(numTerms);
            out[0] = 2;
            for (int i = 1; i < numTerms; ++i) out[i] = out[i - 1] + 1;
        }
        return true;
    }
    // Validate (:386-431).
    bool validate() {
        if (centers.size() != widths.size() || centers.size() != weights.size() || centers.size() < starts.size())
            return false;
        if (centers.size() < 2) return false;
        if (!starts.empty()) {
            if (starts[0] != 2) return false;
            for (size_t i = 1; i < starts.size(); ++i) {
                if (starts[i] <= starts[i - 1]) return false;
                if (starts[i] >= centers.size()) return false;
            }
        }
        order = (int)starts.size() + 1 + 2;
        return true;
    }
    void range(int k, int& b, int& e) const {
        b = (int)starts[k - 4];
        e = (int)centers.size();
        if ((size_t)(k - 4 + 1) < starts.size()) e = (int)starts[k - 4 + 1];
    }
    void evalAll(double* out, unsigned maxOrder, double x) const {
        out[0] = 1.;
        if (maxOrder == 0) return;
        out[1] = x;
        if (maxOrder == 1) return;
        out[2] = -weights[0] * posEval(kSoftPlus, -widths[0] * (x - centers[0]));
        if (maxOrder == 2) return;
        out[3] = weights[1] * posEval(kSoftPlus, widths[1] * (x - centers[1]));
        if (maxOrder == 3) return;
        for (int k = 4; k <= (int)maxOrder; ++k) {
            out[k] = 0.;
            int b, e;
            range(k, b, e);
            for (int j = b; j < e; ++j) out[k] += weights[j] * logistic(widths[j] * (x - centers[j]));
        }
    }
    void evalDerivs(double* out, double* d1, unsigned maxOrder, double x) const {
        out[0] = 1.;
        d1[0] = 0.;
        if (maxOrder == 0) return;
        out[1] = x;
        d1[1] = 1.;
        if (maxOrder == 1) return;
        out[2] = -weights[0] * posEval(kSoftPlus, -widths[0] * (x - centers[0]));
        d1[2] = weights[0] * widths[0] * posDeriv(kSoftPlus, -widths[0] * (x - centers[0]));
        if (maxOrder == 2) return;
        out[3] = weights[1] * posEval(kSoftPlus, widths[1] * (x - centers[1]));
        d1[3] = weights[1] * widths[1] * posDeriv(kSoftPlus, widths[1] * (x - centers[1]));
        if (maxOrder == 3) return;
        for (int k = 4; k <= (int)maxOrder; ++k) {
            out[k] = 0.;
            d1[k] = 0.;
            int b, e;
            range(k, b, e);
            for (int j = b; j < e; ++j) {
                out[k] += weights[j] * logistic(widths[j] * (x - centers[j]));
                d1[k] += weights[j] * widths[j] * logisticD(widths[j] * (x - centers[j]));
            }
        }
    }
    void evalSecond(double* out, double* d1, double* d2, unsigned maxOrder, double x) const {
        out[0] = 1.;
        d1[0] = 0.;
        d2[0] = 0.;
        if (maxOrder == 0) return;
        out[1] = x;
        d1[1] = 1.;
        d2[1] = 0.;
        if (maxOrder == 1) return;
        out[2] = -weights[0] * posEval(kSoftPlus, -widths[0] * (x - centers[0]));
        d1[2] = weights[0] * widths[0] * posDeriv(kSoftPlus, -widths[0] * (x - centers[0]));
        d2[2] = -weights[0] * widths[0] * widths[0] * posSecondDeriv(kSoftPlus, -widths[0] * (x - centers[0]));
        if (maxOrder == 2) return;
        out[3] = weights[1] * posEval(kSoftPlus, widths[1] * (x - centers[1]));
        d1[3] = weights[1] * widths[1] * posDeriv(kSoftPlus, widths[1] * (x - centers[1]));
        d2[3] = weights[1] * widths[1] * widths[1] * posSecondDeriv(kSoftPlus, widths[1] * (x - centers[1]));
        if (maxOrder == 3) return;
        for (int k = 4; k <= (int)maxOrder; ++k) {
            out[k] = 0.;
            d1[k] = 0.;
            d2[k] = 0.;
            int b, e;
            range(k, b, e);
            for (int j = b; j < e; ++j) {
                out[k] += weights[j] * logistic(widths[j] * (x - centers[j]));
                d1[k] += weights[j] * widths[j] * logisticD(widths[j] * (x - centers[j]));
                d2[k] += weights[j] * widths[j] * widths[j] * logisticD2(widths[j] * (x - centers[j]));
            }
        }
    }
};

// CreateSigmoid (src/MapFactory.cpp:181-254): edge terms get width edgeShape
// and weight 1/edgeShape; Linear sums set the widths of all but the last
// sigmoid of each term from the neighbouring centers (the last keeps width
// 0); Constant sums sort the interior centers and use neighbour spacings.
static bool sigmoidFromCenters(const double* c, unsigned n, double edgeShape, int sumType, Sigmoid1d& S) {
    int numSig = Sigmoid1d::numSigmoids(n, sumType);
    std::vector<double> hW(n, 0.0), hWt(n, 1.0), hC(c, c + n);
    if (n < 2) return false;
    hW[0] = edgeShape;
    hWt[0] = 1.0 / edgeShape;
    hW[1] = edgeShape;
    hWt[1] = 1.0 / edgeShape;
    if (sumType == 0) {
        for (int i = 0; i < numSig; i++) {
            int start = 2 + (i * (i + 1)) / 2;
            for (int j = 0; j < i; j++) {
                double prev, next;
                if (j == 0 || i == 0) prev = c[0];
                else prev = c[start + j - 1];
                if (j == i - 1 || i == 0) next = c[1];
                else next = c[start + j];
                hW[start + j] = 2 / (next - prev);
                hWt[start + j] = 1.;
            }
        }
    } else if (numSig > 0) {
        std::sort(hC.begin() + 2, hC.end());
        if (numSig > 1) hW[2] = 4.0 / (hC[3] - hC[2]);
        else hW[2] = 8.0 / std::abs(hC[1] - hC[0]);
        for (int i = 1; i < numSig - 1; i++) hW[2 + i] = 8.0 / (hC[3 + i] - hC[1 + i]);
        if (numSig > 1) hW[2 + numSig - 1] = 4.0 / (hC[2 + numSig - 1] - hC[2 + numSig - 2]);
    }
    S.centers = hC;
    S.widths = hW;
    S.weights = hWt;
    if (!Sigmoid1d::constructStarts(n, sumType, S.starts)) return false;
    return S.validate();
}

// ----------------------------------------------------------------------------
// MultivariateExpansionWorker (MParT/MultivariateExpansionWorker.h).
// Cache layout :19-40 and :94-107; FillCache1 :142-158; FillCache2 :172-201;
// term loops :204-397; per-term products :423-554 (Identity rectifier).
// ----------------------------------------------------------------------------
enum DerivType { dNone, dParameters, dDiagonal, dDiagonal2, dInput, dMixedInput, dMixedCoeff };

struct Expansion {
    MultiSet ms;
    Basis1d basis;
    unsigned D = 0;
    // BasisEvaluator<OffdiagHomogeneous, pair<offdiag, Sigmoid1d>, Rectifier>
    // (MParT/BasisEvaluator.h:221-330): a sigmoid basis in the last input and
    // a rectifier (-1 Identity, else a positive bijector) applied to the
    // leading-input product of every term that depends on the last input.
    const Sigmoid1d* diag = nullptr;
    int rect = -1;
    std::vector<unsigned> startPos;
    unsigned cacheSize = 0;

    void setup() {
        D = ms.dim;
        startPos.assign(2 * D + 2, 0);
        unsigned upd = 0;
        for (unsigned i = 0; i < 2 * D + 2; ++i) {
            startPos[i] = upd;
            if (i < 2 * D) upd += ms.maxDeg[i % D] + 1;
            else upd += ms.maxDeg[D - 1] + 1;
        }
        cacheSize = startPos[2 * D + 1];
    }
    unsigned numTerms() const { return ms.size(); }
    bool isConst(unsigned t) const { return ms.starts[t] == ms.starts[t + 1]; }

    void fillCache1(double* c, const double* pt, DerivType dt) const {
        if (dt == dInput || dt == dMixedInput) {
            for (unsigned d = 0; d + 1 < D; ++d)
                basis.evalDerivs(&c[startPos[d]], &c[startPos[d + D]], ms.maxDeg[d], pt[d]);
        } else {
            for (unsigned d = 0; d + 1 < D; ++d)
                basis.evalAll(&c[startPos[d]], ms.maxDeg[d], pt[d]);
        }
    }
    void fillCache2(double* c, double xd, DerivType dt) const {
        if (diag) {
            if (dt == dNone || dt == dParameters) diag->evalAll(&c[startPos[D - 1]], ms.maxDeg[D - 1], xd);
            else if (dt == dDiagonal || dt == dInput || dt == dMixedCoeff)
                diag->evalDerivs(&c[startPos[D - 1]], &c[startPos[2 * D - 1]], ms.maxDeg[D - 1], xd);
            else
                diag->evalSecond(&c[startPos[D - 1]], &c[startPos[2 * D - 1]], &c[startPos[2 * D]], ms.maxDeg[D - 1],
                                 xd);
            return;
        }
        if (dt == dNone || dt == dParameters) {
            basis.evalAll(&c[startPos[D - 1]], ms.maxDeg[D - 1], xd);
        } else if (dt == dDiagonal || dt == dInput || dt == dMixedCoeff) {
            basis.evalDerivs(&c[startPos[D - 1]], &c[startPos[2 * D - 1]], ms.maxDeg[D - 1], xd);
        } else {
            basis.evalSecond(&c[startPos[D - 1]], &c[startPos[2 * D - 1]], &c[startPos[2 * D]], ms.maxDeg[D - 1], xd);
        }
    }
    double cv(const double* c, unsigned i) const { return c[startPos[ms.dims[i]] + ms.orders[i]]; }

    double termVal(unsigned t, const double* c) const {
        double v = 1.0;
        unsigned e = ms.starts[t + 1] - 1;
        for (unsigned i = ms.starts[t]; i < e; ++i) v *= cv(c, i);
        double last = cv(c, e);
        if (rect >= 0) v = (ms.dims[e] == D - 1) ? posEval(rect, v) * last : v * last;
        else v *= last;
        return v;
    }
    double termValDiag(unsigned t, const double* c, unsigned posIndex) const {
        double v = 1.0;
        unsigned e = ms.starts[t + 1] - 1;
        if (ms.dims[e] != D - 1) return 0.;
        for (unsigned i = ms.starts[t]; i < e; ++i) v *= cv(c, i);
        double dv = c[startPos[posIndex] + ms.orders[e]];
        if (rect >= 0) v = posEval(rect, v);
        v *= dv;
        return v;
    }
    double termValInputDeriv(unsigned t, int wrt, const double* c) const {
        double v = 1.0, wrtVal = 1.0, wrtDeriv = (wrt == -1);
        unsigned e = ms.starts[t + 1] - 1;
        for (unsigned i = ms.starts[t]; i < e; ++i) {
            if (int(ms.dims[i]) == wrt) {
                wrtVal = c[startPos[wrt] + ms.orders[i]];
                wrtDeriv = c[startPos[D + wrt] + ms.orders[i]];
            } else {
                v *= cv(c, i);
            }
        }
        int d = ms.dims[e];
        double last;
        if (wrt == d) {
            last = 1;
            wrtVal = c[startPos[d] + ms.orders[e]];
            wrtDeriv = c[startPos[D + d] + ms.orders[e]];
        } else {
            last = c[startPos[d] + ms.orders[e]];
        }
        if (rect >= 0) {
            const bool isRect = d == int(D) - 1;
            if (wrt == int(D) - 1) v = posEval(rect, v) * wrtDeriv;
            else if (wrt == -1) v = isRect ? posEval(rect, v) * last : v * last;
            else if (!isRect) v *= last * wrtDeriv;
            else v = posDeriv(rect, v * wrtVal) * v * wrtDeriv * last;
            return v;
        }
        v *= last * wrtDeriv;
        return v;
    }
    double termValMixedDeriv(unsigned t, int wrt, const double* c) const {
        double v = 1.0, wrtVal = 1.0, wrtDeriv = (wrt == int(D) - 1 || wrt == -1);
        unsigned e = ms.starts[t + 1] - 1;
        if (ms.dims[e] != D - 1) return 0.;
        for (unsigned i = ms.starts[t]; i < e; ++i) {
            if (int(ms.dims[i]) == wrt) {
                wrtVal = c[startPos[wrt] + ms.orders[i]];
                wrtDeriv = c[startPos[D + wrt] + ms.orders[i]];
            } else {
                v *= cv(c, i);
            }
        }
        unsigned posInd = (wrt == int(D) - 1) ? (2 * D) : (2 * D - 1);
        double dv = c[startPos[posInd] + ms.orders[e]];
        if (rect >= 0) {
            if (wrt == int(D) - 1 || wrt == -1) v = posEval(rect, v) * dv;
            else v = posDeriv(rect, v * wrtVal) * v * wrtDeriv * dv;
            return v;
        }
        v *= (dv * wrtDeriv);
        return v;
    }
    double termValMixedCoeff(unsigned t, const double* c, unsigned posIndex) const {
        double v = 1.0;
        if (isConst(t)) return 0.;
        unsigned e = ms.starts[t + 1] - 1;
        if (ms.dims[e] != D - 1) return 0.;
        for (unsigned i = ms.starts[t]; i < e; ++i) v *= cv(c, i);
        double dv = c[startPos[posIndex] + ms.orders[e]];
        if (rect >= 0) v = posEval(rect, v);
        v *= dv;
        return v;
    }

    double evaluate(const double* c, const double* coeffs) const {
        double out = 0.0;
        for (unsigned t = 0; t < numTerms(); ++t) {
            if (isConst(t)) { out += coeffs[t]; continue; }
            double tv = termVal(t, c);
            out += tv * coeffs[t];
        }
        return out;
    }
    double diagonalDerivative(const double* c, const double* coeffs, unsigned derivOrder) const {
        double out = 0.0;
        unsigned posIndex = 2 * D + derivOrder - 2;
        for (unsigned t = 0; t < numTerms(); ++t) {
            if (isConst(t)) continue;
            double tv = termValDiag(t, c, posIndex);
            out += tv * coeffs[t];
        }
        return out;
    }
    double coeffDerivative(const double* c, const double* coeffs, double* grad, long gstride) const {
        double f = 0;
        for (unsigned t = 0; t < numTerms(); ++t) {
            if (isConst(t)) { f += coeffs[t]; grad[t * gstride] = 1.0; continue; }
            double tv = termVal(t, c);
            f += tv * coeffs[t];
            grad[t * gstride] = tv;
        }
        return f;
    }
    double inputDerivative(const double* c, const double* coeffs, double* grad, long gstride) const {
        double f = 0.0;
        for (int wrt = -1; wrt < int(D); ++wrt) {
            if (wrt >= 0) grad[wrt * gstride] = 0;
            for (unsigned t = 0; t < numTerms(); ++t) {
                if (isConst(t)) { if (wrt < 0) f += coeffs[t]; continue; }
                double tv = termValInputDeriv(t, wrt, c);
                if (wrt < 0) f += tv * coeffs[t];
                else grad[wrt * gstride] += tv * coeffs[t];
            }
        }
        return f;
    }
    double mixedInputDerivative(const double* c, const double* coeffs, double* grad, long gstride) const {
        double df = 0.0;
        for (int wrt = -1; wrt < int(D); ++wrt) {
            if (wrt >= 0) grad[wrt * gstride] = 0;
            for (unsigned t = 0; t < numTerms(); ++t) {
                if (isConst(t)) continue;
                double tv = termValMixedDeriv(t, wrt, c);
                if (wrt < 0) df += tv * coeffs[t];
                else grad[wrt * gstride] += tv * coeffs[t];
            }
        }
        return df;
    }
    double mixedCoeffDerivative(const double* c, const double* coeffs, unsigned derivOrder, double* grad, long gstride) const {
        double df = 0;
        unsigned posIndex = 2 * D + derivOrder - 2;
        for (unsigned t = 0; t < numTerms(); ++t) {
            double tv = termValMixedCoeff(t, c, posIndex);
            df += tv * coeffs[t];
            grad[t * gstride] = tv;
        }
        return df;
    }
};

// ----------------------------------------------------------------------------
// MonotoneIntegrand::operator() (MParT/MonotoneIntegrand.h:118-203), modes
// None, Diagonal, Parameters and Input.  Instead of aborting when g(df) is
// infinite (the reference's failOnNaN path, :183-190), a status flag is set.
// ----------------------------------------------------------------------------
struct Integrand {
    const Expansion* ex;
    double* cache;
    double xd;
    const double* coeffs;
    DerivType dt;
    double nugget;
    int pos;
    double* work = nullptr;  // numTerms doubles for the MixedCoeff mode
    mutable long nevals = 0;
    mutable int infFlag = 0;
    // Status for the quadrature loop: 1 = g(df) was infinite (the reference
    // throws at MonotoneIntegrand.h:183-190), 2 = the integrand was NaN (the
    // reference would subdivide to maxSub on every branch; this restatement
    // and the GPU kernels stop and return NaN instead).
    int failed() const { return infFlag; }

    unsigned fdim() const {
        unsigned n = 1;
        if (dt == dDiagonal) n++;
        if (dt == dParameters || dt == dMixedCoeff) n += ex->numTerms();
        if (dt == dInput) n += ex->D;
        return n;
    }
    void operator()(double t, double* out) const {
        nevals++;
        const unsigned dim = ex->D;
        if (dt == dDiagonal || dt == dInput || dt == dMixedCoeff) ex->fillCache2(cache, t * xd, dDiagonal2);
        else ex->fillCache2(cache, t * xd, dDiagonal);
        double df = 0;
        if (dt == dMixedCoeff) {
            // d/dc of the Diagonal integrand (MonotoneIntegrand.h:148-165).
            df = ex->diagonalDerivative(cache, coeffs, 1);
            const double dgdf = posDeriv(pos, df);
            const double df2 = ex->mixedCoeffDerivative(cache, coeffs, 2, work, 1);
            double scale = xd * t * dgdf;
            for (unsigned i = 0; i < ex->numTerms(); ++i) work[i] *= scale;
            df = ex->mixedCoeffDerivative(cache, coeffs, 1, &out[1], 1);
            scale = xd * t * df2 * posSecondDeriv(pos, df) + dgdf;
            for (unsigned i = 0; i < ex->numTerms(); ++i) out[1 + i] = scale * out[1 + i] + work[i];
        } else if (dt == dParameters) {
            df = ex->mixedCoeffDerivative(cache, coeffs, 1, &out[1], 1);
            double scale = xd * posDeriv(pos, df);
            for (unsigned i = 0; i < ex->numTerms(); ++i) out[1 + i] *= scale;
        } else if (dt == dInput) {
            df = ex->mixedInputDerivative(cache, coeffs, &out[1], 1);
            double scale = xd * posDeriv(pos, df);
            for (unsigned i = 0; i + 1 < dim; ++i) out[1 + i] *= scale;
        } else {
            df = ex->diagonalDerivative(cache, coeffs, 1);
        }
        double gf = posEval(pos, df);
        out[0] = xd * (gf + nugget);
        if (std::isinf(gf)) infFlag = 1;
        else if (std::isnan(out[0]) && !infFlag) infFlag = 2;
        if (dt == dDiagonal || dt == dInput) {
            unsigned ind = (dt == dDiagonal) ? 1 : dim;
            out[ind] = ex->diagonalDerivative(cache, coeffs, 2);
            out[ind] *= xd * t * posDeriv(pos, df);
            out[ind] += (gf + nugget);
        }
    }
};

// ----------------------------------------------------------------------------
// Clenshaw-Curtis rule (MParT/Quadrature.h:212-258) and
// AdaptiveClenshawCurtis::Integrate (:819-968) with the QuadError::First
// error metric (:441-481).  The workspace layout and traversal are those of
// the reference: depth-first, left-first bisection with a per-level record
// [left, right, midFunc(fdim)].
// ----------------------------------------------------------------------------
static void ccRule(unsigned numPts, double* wts, double* pts) {
    if (numPts == 0) return;
    if (numPts == 1) { pts[0] = 0.0; wts[0] = 2.0; return; }
    for (unsigned i = 0; i < numPts; ++i) pts[i] = std::cos((numPts - (i + 1)) * kPi / (numPts - 1));
    pts[0] = -1.0;
    if (numPts % 2 == 1) pts[(numPts - 1) / 2] = 0.0;
    pts[numPts - 1] = 1.0;
    double theta;
    for (unsigned i = 0; i < numPts; ++i) {
        wts[i] = 1.0;
        theta = i * kPi / (numPts - 1);
        for (unsigned j = 0; j < (numPts - 1) / 2; ++j) {
            double b;
            if (2 * (j + 1) == (numPts - 1)) b = 1.0;
            else b = 2.0;
            wts[i] = wts[i] - b * std::cos(2.0 * (j + 1) * theta) / (4 * (j + 1) * (j + 1) - 1);
        }
    }
    wts[0] = wts[0] / (numPts - 1.0);
    for (unsigned i = 1; i < (numPts - 1); ++i) wts[i] = 2.0 * wts[i] / (numPts - 1.0);
    wts[numPts - 1] = wts[numPts - 1] / (numPts - 1.0);
}

// The three quadrature rules of MapOptions::quadType (MParT/MapOptions.h,
// src/MapFactoryImpl4.cpp:14-31): kind 0 ClenshawCurtis (fixed, quadPts
// points), 1 AdaptiveSimpson, 2 AdaptiveClenshawCurtis.
struct ACC {
    int kind = 2;
    std::vector<double> cPts, cWts, fPts, fWts;
    std::vector<double> ruleP, ruleW;  // fixed ClenshawCurtis rule
    unsigned maxSub = 30, minSub = 0;
    double absTol = 1e-6, relTol = 1e-6;

    unsigned wsSize(unsigned fdim) const {
        if (kind == 0) return fdim;
        if (kind == 1) return (2 * maxSub + 5) * fdim + 2 * maxSub;
        return workspaceSize(maxSub, fdim);
    }

    // ClenshawCurtisQuadrature::Integrate (Quadrature.h:114-143).
    template <class F>
    void integrateFixed(double* ws, const F& f, unsigned fdim, double lb, double ub, double* res) const {
        if ((ub - lb) < 15.0 * std::numeric_limits<double>::epsilon()) {
            f(0.5 * (ub + lb), res);
            for (unsigned i = 0; i < fdim; ++i) res[i] *= (ub - lb);
            return;
        }
        for (unsigned j = 0; j < fdim; ++j) res[j] = 0.0;
        double* fval = ws;
        for (unsigned i = 0; i < ruleP.size(); ++i) {
            f(0.5 * (ub + lb + (ub - lb) * ruleP[i]), fval);
            if (f.failed()) {
                for (unsigned j = 0; j < fdim; ++j) res[j] = std::numeric_limits<double>::quiet_NaN();
                return;
            }
            for (unsigned j = 0; j < fdim; ++j) res[j] += 0.5 * (ub - lb) * ruleW[i] * fval[j];
        }
    }

    // AdaptiveSimpson::Integrate (Quadrature.h:497-716): depth-first,
    // left-first bisection; per level a record [left, right, f(leftMid),
    // f(rightMid)]; coarse Simpson on the interval against composite Simpson
    // on its halves; QuadError::First.
    template <class F>
    void integrateSimpson(double* ws, const F& f, unsigned fdim, double lb, double ub, double* res) const {
        for (unsigned i = 0; i < fdim; ++i) res[i] = 0;
        auto bail = [&]() {
            if (!f.failed()) return false;
            for (unsigned i = 0; i < fdim; ++i) res[i] = std::numeric_limits<double>::quiet_NaN();
            return true;
        };
        unsigned currLevel = 0, currSegment = 0;
        double midPt = 0.5 * (lb + ub);
        double* leftFunc = &ws[0];
        f(lb, leftFunc);
        double* rightFunc = &ws[fdim];
        f(ub, rightFunc);
        double* midFunc = &ws[2 * fdim];
        f(midPt, midFunc);
        if (bail()) return;
        double* intCoarse = &ws[3 * fdim];
        double* intFine = &ws[4 * fdim];
        unsigned workStart = 5 * fdim;
        ws[workStart] = lb;
        ws[workStart + 1] = ub;
        while (true) {
            double* leftPt = &ws[workStart];
            double* rightPt = &ws[workStart + 1];
            midPt = 0.5 * ((*leftPt) + (*rightPt));
            const double leftMidPt = 0.5 * ((*leftPt) + midPt);
            const double rightMidPt = 0.5 * (midPt + (*rightPt));
            double* leftMidFunc = &ws[workStart + 2];
            f(leftMidPt, leftMidFunc);
            double* rightMidFunc = &ws[workStart + 2 + fdim];
            f(rightMidPt, rightMidFunc);
            if (bail()) return;
            for (unsigned i = 0; i < fdim; ++i) {
                intCoarse[i] = (((*rightPt) - (*leftPt)) / 6.0) * (leftFunc[i] + 4.0 * midFunc[i] + rightFunc[i]);
                intFine[i] = ((midPt - (*leftPt)) / 6.0) * (leftFunc[i] + 4.0 * leftMidFunc[i] + midFunc[i]);
                intFine[i] += (((*rightPt) - midPt) / 6.0) * (midFunc[i] + 4.0 * rightMidFunc[i] + rightFunc[i]);
            }
            const double error = std::fabs(intFine[0] - intCoarse[0]);
            const double errorTol = std::fmax(relTol * std::fabs(intCoarse[0]), absTol);
            if ((((error < errorTol) || (currLevel == maxSub - 1)) && (currLevel >= minSub)) ||
                (std::abs(ub - lb) < 1e-14)) {
                for (unsigned i = 0; i < fdim; ++i) res[i] += intFine[i];
                while (((currSegment >> currLevel) & 1U) && (currLevel > 0)) {
                    currSegment &= ~(1UL << currLevel);
                    currLevel--;
                }
                if (currLevel == 0) break;
                currSegment |= 1UL << currLevel;
                workStart = (2 * currLevel + 5) * fdim + 2 * currLevel;
                const unsigned prev = (2 * (currLevel - 1) + 5) * fdim + 2 * (currLevel - 1);
                ws[workStart] = 0.5 * (ws[prev] + ws[prev + 1]);
                ws[workStart + 1] = ws[prev + 1];
                // values at the new interval's left, middle and right ends
                leftFunc = &ws[0];
                midFunc = &ws[2 * fdim];
                rightFunc = &ws[fdim];
                for (unsigned level = 0; level < currLevel; ++level) {
                    if ((currSegment >> (level + 1)) & 1U) {
                        leftFunc = midFunc;
                        midFunc = &ws[(2 * level + 5 + 1) * fdim + 2 * level + 2];
                    } else {
                        rightFunc = midFunc;
                        midFunc = &ws[(2 * level + 5) * fdim + 2 * level + 2];
                    }
                }
            } else {
                currLevel++;
                rightFunc = midFunc;
                midFunc = leftMidFunc;
                workStart = (2 * currLevel + 5) * fdim + 2 * currLevel;
                ws[workStart] = *leftPt;
                ws[workStart + 1] = midPt;
            }
        }
    }

    void init(unsigned level, unsigned maxSub_, double absTol_, double relTol_, unsigned minSub_) {
        unsigned nc = (unsigned)std::pow(2, level) + 1, nf = (unsigned)std::pow(2, level + 1) + 1;
        cPts.resize(nc); cWts.resize(nc); fPts.resize(nf); fWts.resize(nf);
        ccRule(nc, cWts.data(), cPts.data());
        ccRule(nf, fWts.data(), fPts.data());
        maxSub = maxSub_; absTol = absTol_; relTol = relTol_; minSub = minSub_;
    }
    static unsigned workspaceSize(unsigned maxSub, unsigned fdim) { return (maxSub + 5) * fdim + 2 * maxSub; }

    template <class F>
    void integrate(double* ws, const F& f, unsigned fdim, double lb, double ub, double* res) const {
        if (kind == 0) return integrateFixed(ws, f, fdim, lb, ub, res);
        if (kind == 1) return integrateSimpson(ws, f, fdim, lb, ub, res);
        for (unsigned i = 0; i < fdim; ++i) res[i] = 0;
        auto bail = [&]() {
            if (!f.failed()) return false;
            for (unsigned i = 0; i < fdim; ++i) res[i] = std::numeric_limits<double>::quiet_NaN();
            return true;
        };
        unsigned currLevel = 0, currSegment = 0;
        double midPt = 0.5 * (lb + ub);
        double scale = (ub - lb);
        double* leftFunc = &ws[0];
        f(lb, leftFunc);
        double* rightFunc = &ws[fdim];
        f(ub, rightFunc);
        if (bail()) return;
        double* fval = &ws[2 * fdim];
        double* intCoarse = &ws[3 * fdim];
        double* intFine = &ws[4 * fdim];
        double* leftPt = &ws[5 * fdim];
        *leftPt = lb;
        double* rightPt = &ws[5 * fdim + 1];
        *rightPt = ub;
        double* midFunc;
        unsigned workStartInd = 5 * fdim, prevStartInd = 0;
        double error, errorTol;
        unsigned coarseRightIndex, coarseMidIndex, fineRightIndex, fineMidIndex;
        while (true) {
            leftPt = &ws[workStartInd];
            rightPt = &ws[workStartInd + 1];
            midPt = 0.5 * ((*leftPt) + (*rightPt));
            scale = 0.5 * ((*rightPt) - (*leftPt));
            midFunc = &ws[workStartInd + 2];
            f(midPt, midFunc);
            if (bail()) return;
            coarseRightIndex = (unsigned)cWts.size() - 1;
            coarseMidIndex = coarseRightIndex / 2;
            fineRightIndex = (unsigned)fWts.size() - 1;
            fineMidIndex = fineRightIndex / 2;
            for (unsigned i = 0; i < fdim; ++i) {
                intCoarse[i] = scale * cWts[0] * leftFunc[i];
                intCoarse[i] += scale * cWts[coarseMidIndex] * midFunc[i];
                intCoarse[i] += scale * cWts[coarseRightIndex] * rightFunc[i];
                intFine[i] = scale * fWts[0] * leftFunc[i];
                intFine[i] += scale * fWts[fineMidIndex] * midFunc[i];
                intFine[i] += scale * fWts[fineRightIndex] * rightFunc[i];
            }
            for (unsigned i = 1; i < coarseMidIndex; ++i) {
                f(midPt + scale * cPts[i], fval);
                if (bail()) return;
                for (unsigned j = 0; j < fdim; ++j) {
                    intCoarse[j] += scale * cWts[i] * fval[j];
                    intFine[j] += scale * fWts[2 * i] * fval[j];
                }
            }
            for (unsigned i = coarseMidIndex + 1; i < coarseRightIndex; ++i) {
                f(midPt + scale * cPts[i], fval);
                if (bail()) return;
                for (unsigned j = 0; j < fdim; ++j) {
                    intCoarse[j] += scale * cWts[i] * fval[j];
                    intFine[j] += scale * fWts[2 * i] * fval[j];
                }
            }
            for (unsigned i = 1; i < fPts.size(); i += 2) {
                f(midPt + scale * fPts[i], fval);
                if (bail()) return;
                for (unsigned j = 0; j < fdim; ++j) intFine[j] += scale * fWts[i] * fval[j];
            }
            // QuadError::First
            error = std::fabs(intFine[0] - intCoarse[0]);
            double relRefVal = std::fabs(intCoarse[0]);
            errorTol = std::fmax(relTol * relRefVal, absTol);
            if ((((error < errorTol) || (currLevel == maxSub - 1)) && (currLevel >= minSub)) || (std::abs(ub - lb) < 1e-14)) {
                for (unsigned i = 0; i < fdim; ++i) res[i] += intFine[i];
                while (((currSegment >> currLevel) & 1U) && (currLevel > 0)) {
                    currSegment &= ~(1UL << currLevel);
                    currLevel--;
                }
                if (currLevel == 0) break;
                currSegment |= 1UL << currLevel;
                workStartInd = (currLevel + 5) * fdim + 2 * currLevel;
                if (currLevel > 0) {
                    prevStartInd = ((currLevel - 1) + 5) * fdim + 2 * (currLevel - 1);
                    ws[workStartInd] = 0.5 * (ws[prevStartInd] + ws[prevStartInd + 1]);
                    ws[workStartInd + 1] = ws[prevStartInd + 1];
                } else {
                    ws[workStartInd] = midPt;
                    ws[workStartInd + 1] = ub;
                }
                // UpdateValues (:977-992)
                leftFunc = &ws[0];
                rightFunc = &ws[fdim];
                for (unsigned level = 0; level < currLevel; ++level) {
                    if ((currSegment >> (level + 1)) & 1U) leftFunc = &ws[(level + 5) * fdim + 2 * (level + 1)];
                    else rightFunc = &ws[(level + 5) * fdim + 2 * (level + 1)];
                }
            } else {
                currLevel++;
                rightFunc = midFunc;
                workStartInd = (currLevel + 5) * fdim + 2 * currLevel;
                ws[workStartInd] = *leftPt;
                ws[workStartInd + 1] = midPt;
            }
        }
    }
};

// ----------------------------------------------------------------------------
// RootFinding (MParT/Utilities/RootFinding.h:20-178).
// ----------------------------------------------------------------------------
template <class F>
static void findBracket(F& f, double& xlb, double& ylb, double& xub, double& yub, const double yd, int& info) {
    const unsigned maxIts = 128;
    double stepSize = 1.0;
    info = 0;
    ylb = f(xlb);
    yub = f(xub);
    if (ylb > yd) {
        std::swap(ylb, yub);
        std::swap(xlb, xub);
        unsigned i;
        for (i = 0; i < maxIts; ++i) {
            xlb = xub - stepSize;
            ylb = f(xlb);
            if ((std::fabs((yub - ylb) / (xub - xlb)) < 1e-12) && ((xub - xlb) > 10)) { info = -1; return; }
            if (ylb > yd) { yub = ylb; xub = xlb; stepSize *= 2.0; }
            else break;
        }
        if (i >= maxIts) info = -2;
    } else {
        unsigned i;
        for (i = 0; i < maxIts; ++i) {
            xub = xlb + stepSize;
            yub = f(xub);
            if ((std::fabs((yub - ylb) / (xub - xlb)) < 1e-12) && ((xub - xlb) > 10)) { info = -1; return; }
            if (yub < yd) { ylb = yub; xlb = xub; stepSize *= 2.0; }
            else break;
        }
        if (i >= maxIts) info = -2;
    }
}

static double findXITP(double xlb, double xub, double /*yd*/, double ylb, double yub, double k1, double k2,
                       double nhalf, double n0, int it, double xtol) {
    double xb = 0.5 * (xub + xlb);
    double xf = (xub * ylb - xlb * yub) / (ylb - yub);
    double sigma = ((xb - xf) > 0) ? 1.0 : -1.0;
    double delta = std::fmin(k1 * std::pow((xub - xlb), k2), std::fabs(xb - xf));
    xf += delta * sigma;
    double rho = std::fmin(xtol * std::pow(2.0, nhalf + n0 - it) - 0.5 * (xub - xlb), std::fabs(xf - xb));
    double xc = xb - sigma * rho;
    return xc;
}

template <class F>
static double inverseSingleBracket(double yd, F& f, double x0, const double xtol, const double ftol, int& info) {
    const unsigned maxIts = 10000;
    double xlb, xub, ylb, yub, xc, yc;
    info = 0;
    xlb = xub = x0;
    ylb = yub = f(xlb);
    int binfo = 0;
    findBracket(f, xlb, ylb, xub, yub, yd, binfo);
    if ((binfo < 0) || (((ylb > yd) || (yub < yd)))) {
        info = -2;
        return std::numeric_limits<double>::quiet_NaN();
    }
    const double k1 = 0.1, k2 = 2.0;
    const double nhalf = std::ceil(std::log2(0.5 * (xub - xlb) / xtol));
    const double n0 = 1.0;
    unsigned it;
    for (it = 0; it < maxIts; ++it) {
        xc = findXITP(xlb, xub, yd, ylb, yub, k1, k2, nhalf, n0, it, xtol);
        yc = f(xc);
        if (std::fabs(yc - yd) < ftol) return xc;
        else if (yc > yd) { std::swap(xc, xub); std::swap(yc, yub); }
        else { std::swap(xc, xlb); std::swap(yc, ylb); }
        if (((xub - xlb) < xtol) || ((yub - ylb) < ftol)) break;
    }
    if (it > maxIts) info = -1;
    return 0.5 * (xub + xlb);
}

// ----------------------------------------------------------------------------
// MonotoneComponent (MParT/MonotoneComponent.h).  One object per component;
// every entry point loops over points with OpenMP, one point per iteration
// (the Kokkos one-thread-per-point model).
// ----------------------------------------------------------------------------
struct Component {
    bool contDeriv = true;  // MapOptions::contDeriv
    Expansion ex;
    ACC quad;
    int pos = kSoftPlus;
    double nugget = 0.0;
    int nthreads = 1;

    unsigned D() const { return ex.D; }
    unsigned T() const { return ex.numTerms(); }
};

// Column accessor for a D x N point matrix with strides.
struct View2 {
    const double* p;
    long rs, cs;
    double at(long r, long c) const { return p[r * rs + c * cs]; }
};

#define ORC_PARALLEL_FOR _Pragma("omp parallel for schedule(dynamic, 16)")

// EvaluateSingle (MonotoneComponent.h:992-1017).  Its nugget argument
// defaults to 0: EvaluateImpl calls it without one (MonotoneComponent.h:290),
// so Evaluate ignores MapOptions::nugget, while Inverse passes the
// component's (SingleEvaluator, :434, :1085-1088).
static double evaluateSingle(const Component& C, double* cache, double* ws, double xd, const double* coeffs, long* nev,
                             int* inf, double nugget = 0.0) {
    Integrand ig{&C.ex, cache, xd, coeffs, dNone, nugget, C.pos};
    double out = 0.0;
    C.quad.integrate(ws, ig, 1, 0, 1, &out);
    C.ex.fillCache2(cache, 0.0, dNone);
    out += C.ex.evaluate(cache, coeffs);
    if (nev) *nev += ig.nevals;
    if (inf && ig.infFlag) *inf = ig.infFlag;
    return out;
}

static void setThreads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // namespace orc

using namespace orc;

// ============================================================================
// C interface for the Python test harness (ctypes).  Matrices are given as
// (pointer, row stride, column stride); points are D x N, one column per point.
// Status codes: 0 ok; per-point status 1 = integrand g(df) was infinite.
// ============================================================================
extern "C" {

int orc_total_order_size(unsigned dim, unsigned order, unsigned* nterms, unsigned* nnz) {
    MultiSet ms = totalOrder(dim, order);
    *nterms = ms.size();
    *nnz = (unsigned)ms.dims.size();
    return 0;
}
int orc_total_order_fill(unsigned dim, unsigned order, unsigned* starts, unsigned* dims, unsigned* orders) {
    MultiSet ms = totalOrder(dim, order);
    std::copy(ms.starts.begin(), ms.starts.end(), starts);
    std::copy(ms.dims.begin(), ms.dims.end(), dims);
    std::copy(ms.orders.begin(), ms.orders.end(), orders);
    return 0;
}

void* orc_component_new(unsigned dim, unsigned nterms, const unsigned* starts, const unsigned* dims,
                        const unsigned* orders, int basis, int normalize, int pos, double absTol, double relTol,
                        unsigned maxSub, unsigned minSub, unsigned quadPts, double nugget, int quadType) {
    Component* C = new Component();
    C->ex.ms.dim = dim;
    C->ex.ms.starts.assign(starts, starts + nterms + 1);
    unsigned nnz = starts[nterms];
    C->ex.ms.dims.assign(dims, dims + nnz);
    C->ex.ms.orders.assign(orders, orders + nnz);
    C->ex.ms.calcMaxDegrees();
    C->ex.basis.kind = basis;
    C->ex.basis.prob.normalize = normalize != 0;
    C->ex.setup();
    // MapFactoryImpl4.cpp:18 -- level = (unsigned) log2(quadPts - 2)
    unsigned level = (unsigned)std::log2(quadPts - 2);
    C->quad.init(level, maxSub, absTol, relTol, minSub);
    C->quad.kind = quadType;
    if (quadType == 0) {
        C->quad.ruleP.resize(quadPts);
        C->quad.ruleW.resize(quadPts);
        ccRule(quadPts, C->quad.ruleW.data(), C->quad.ruleP.data());
    }
    C->pos = pos;
    C->nugget = nugget;
    return C;
}
void orc_component_free(void* h) { delete (Component*)h; }
void orc_set_threads(int n) { setThreads(n); }
unsigned orc_cache_size(void* h) { return ((Component*)h)->ex.cacheSize; }

// EvaluateImpl (MonotoneComponent.h:255-299).  nevals (optional) receives the
// integrand evaluation count per point; status (optional) the per-point flag.
int orc_evaluate(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out,
                 long* nevals, int* status) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(1)), pt(C.D());
        for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        long nev = 0;
        int inf = 0;
        out[i] = evaluateSingle(C, cache.data(), ws.data(), pt[C.D() - 1], coeffs, &nev, &inf);
        if (nevals) nevals[i] = nev;
        if (status) status[i] = inf;
    }
    return 0;
}

// ContinuousDerivative (MonotoneComponent.h:487-531).
int orc_cont_derivative(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), pt(C.D());
        for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        C.ex.fillCache2(cache.data(), pt[C.D() - 1], dDiagonal);
        double v = C.ex.diagonalDerivative(cache.data(), coeffs, 1);
        out[i] = posEval(C.pos, v);
    }
    return 0;
}

// LogDeterminantImpl with contDeriv=true (MonotoneComponent.h:105-125).
// DiscreteDerivative (MonotoneComponent.h:585-638): the Diagonal integrand
// integrated with the value, i.e. the x_D-derivative of the quadrature
// approximation of T.
int orc_discrete_derivative(void* h, const double* coeffs, const double* pts, long N, long rs, long cs,
                            double* out) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(2)), pt(C.D());
        for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        Integrand ig{&C.ex, cache.data(), pt[C.D() - 1], coeffs, dDiagonal, C.nugget, C.pos};
        double both[2];
        C.quad.integrate(ws.data(), ig, 2, 0, 1, both);
        out[i] = both[1];
    }
    return 0;
}

void orc_set_cont_deriv(void* h, int on) { ((Component*)h)->contDeriv = on != 0; }

int orc_logdet(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out) {
    if (((Component*)h)->contDeriv) orc_cont_derivative(h, coeffs, pts, N, rs, cs, out);
    else orc_discrete_derivative(h, coeffs, pts, N, rs, cs, out);
    for (long i = 0; i < N; ++i) out[i] = (out[i] <= 0) ? -std::numeric_limits<double>::infinity() : std::log(out[i]);
    return 0;
}

// CoeffJacobian (MonotoneComponent.h:684-741).  jac is T x N with strides.
int orc_coeff_jacobian(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* evals,
                       double* jac, long jrs, long jcs, int* status) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    const unsigned T = C.T();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(T + 1)), integral(T + 1), pt(C.D());
        for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        Integrand ig{&C.ex, cache.data(), pt[C.D() - 1], coeffs, dParameters, C.nugget, C.pos};
        C.quad.integrate(ws.data(), ig, T + 1, 0, 1, integral.data());
        double ev = integral[0];
        C.ex.fillCache2(cache.data(), 0.0, dNone);
        double* jcol = jac + i * jcs;
        ev += C.ex.coeffDerivative(cache.data(), coeffs, jcol, jrs);
        for (unsigned t = 0; t < T; ++t) jcol[t * jrs] += integral[t + 1];
        if (evals) evals[i] = ev;
        if (status) status[i] = ig.infFlag;
    }
    return 0;
}

// CoeffGradImpl (MonotoneComponent.h:166-182): CoeffJacobian scaled by sens.
int orc_coeff_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, const double* sens,
                   long sstride, double* out, long ors, long ocs) {
    Component& C = *(Component*)h;
    orc_coeff_jacobian(h, coeffs, pts, N, rs, cs, nullptr, out, ors, ocs, nullptr);
    const unsigned T = C.T();
    for (long i = 0; i < N; ++i)
        for (unsigned t = 0; t < T; ++t) out[t * ors + i * ocs] *= sens[i * sstride];
    return 0;
}

// InputJacobian (MonotoneComponent.h:757-818).  jac is D x N.
int orc_input_jacobian(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* evals,
                       double* jac, long jrs, long jcs) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    const unsigned D = C.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(D + 1)), integral(D + 1), pt(D);
        for (unsigned d = 0; d < D; ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dInput);
        Integrand ig{&C.ex, cache.data(), pt[D - 1], coeffs, dInput, C.nugget, C.pos};
        C.quad.integrate(ws.data(), ig, D + 1, 0, 1, integral.data());
        double ev = integral[0];
        C.ex.fillCache2(cache.data(), 0.0, dInput);
        double* jcol = jac + i * jcs;
        ev += C.ex.inputDerivative(cache.data(), coeffs, jcol, jrs);
        for (unsigned d = 0; d + 1 < D; ++d) jcol[d * jrs] += integral[d + 1];
        jcol[(D - 1) * jrs] = integral[D];
        if (evals) evals[i] = ev;
    }
    return 0;
}

// GradientImpl (MonotoneComponent.h:148-164).
int orc_gradient(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, const double* sens,
                 long sstride, double* out, long ors, long ocs) {
    Component& C = *(Component*)h;
    orc_input_jacobian(h, coeffs, pts, N, rs, cs, nullptr, out, ors, ocs);
    for (long i = 0; i < N; ++i)
        for (unsigned d = 0; d < C.D(); ++d) out[d * ors + i * ocs] *= sens[i * sstride];
    return 0;
}

// ContinuousMixedJacobian (MonotoneComponent.h:824-874).
int orc_cont_mixed_jacobian(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* jac,
                            long jrs, long jcs) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    const unsigned T = C.T();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), pt(C.D());
        for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        C.ex.fillCache2(cache.data(), pt[C.D() - 1], dDiagonal);
        double* jcol = jac + i * jcs;
        double df = C.ex.mixedCoeffDerivative(cache.data(), coeffs, 1, jcol, jrs);
        double dgdf = posDeriv(C.pos, df);
        for (unsigned t = 0; t < T; ++t) jcol[t * jrs] *= dgdf;
    }
    return 0;
}

// LogDeterminantCoeffGradImpl (MonotoneComponent.h:185-206).
int orc_logdet_coeff_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out,
                          long ors, long ocs) {
    Component& C = *(Component*)h;
    std::vector<double> derivs(N);
    if (C.contDeriv) {
        orc_cont_mixed_jacobian(h, coeffs, pts, N, rs, cs, out, ors, ocs);
        orc_cont_derivative(h, coeffs, pts, N, rs, cs, derivs.data());
    } else {
        // DiscreteMixedJacobian (MonotoneComponent.h:928-980): the MixedCoeff integrand.
        View2 P{pts, rs, cs};
        const unsigned T = C.T();
        ORC_PARALLEL_FOR
        for (long i = 0; i < N; ++i) {
            std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(T + 1)), integral(T + 1), work(T),
                pt(C.D());
            for (unsigned d = 0; d < C.D(); ++d) pt[d] = P.at(d, i);
            C.ex.fillCache1(cache.data(), pt.data(), dNone);
            Integrand ig{&C.ex, cache.data(), pt[C.D() - 1], coeffs, dMixedCoeff, C.nugget, C.pos, work.data()};
            C.quad.integrate(ws.data(), ig, T + 1, 0, 1, integral.data());
            for (unsigned t = 0; t < T; ++t) out[t * ors + i * ocs] = integral[t + 1];
        }
        orc_discrete_derivative(h, coeffs, pts, N, rs, cs, derivs.data());
    }
    for (long i = 0; i < N; ++i)
        for (unsigned t = 0; t < C.T(); ++t) out[t * ors + i * ocs] *= 1.0 / derivs[i];
    return 0;
}

// ContinuousMixedInputJacobian (MonotoneComponent.h:876-926).
int orc_cont_mixed_input_jacobian(void* h, const double* coeffs, const double* pts, long N, long rs, long cs,
                                  double* jac, long jrs, long jcs) {
    Component& C = *(Component*)h;
    View2 P{pts, rs, cs};
    const unsigned D = C.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(C.ex.cacheSize), pt(D);
        for (unsigned d = 0; d < D; ++d) pt[d] = P.at(d, i);
        C.ex.fillCache1(cache.data(), pt.data(), dMixedInput);
        C.ex.fillCache2(cache.data(), pt[D - 1], dMixedInput);
        double* jcol = jac + i * jcs;
        double df = C.ex.mixedInputDerivative(cache.data(), coeffs, jcol, jrs);
        double dgdf = posDeriv(C.pos, df);
        for (unsigned d = 0; d < D; ++d) jcol[d * jrs] *= dgdf;
    }
    return 0;
}

// LogDeterminantInputGradImpl (MonotoneComponent.h:208-232).
int orc_logdet_input_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out,
                          long ors, long ocs) {
    Component& C = *(Component*)h;
    // The reference throws std::invalid_argument here ("Discrete derivative
    // version is not implemented yet", MonotoneComponent.h:216-222).
    if (!C.contDeriv) return -1;
    orc_cont_mixed_input_jacobian(h, coeffs, pts, N, rs, cs, out, ors, ocs);
    std::vector<double> derivs(N);
    orc_cont_derivative(h, coeffs, pts, N, rs, cs, derivs.data());
    for (long i = 0; i < N; ++i)
        for (unsigned d = 0; d < C.D(); ++d) out[d * ors + i * ocs] *= 1.0 / derivs[i];
    return 0;
}

// InverseImpl (MonotoneComponent.h:330-443).  xs is D x numXs (numXs 1 or N);
// its last row is the initial guess.  info (optional) receives the root
// finder's status, which the reference discards.
int orc_inverse(void* h, const double* coeffs, const double* xs, long numXs, long rs, long cs, const double* ys,
                long ystride, long N, double xtol, double ytol, double* out, long ostride, int* info) {
    Component& C = *(Component*)h;
    if ((numXs != 1) && (numXs != N)) return -1;
    View2 P{xs, rs, cs};
    const unsigned D = C.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        long xi = (numXs == 1) ? 0 : i;
        std::vector<double> pt(D);
        bool hasNan = false;
        for (unsigned d = 0; d < D; ++d) {
            pt[d] = P.at(d, xi);
            if (std::isnan(pt[d])) hasNan = true;
        }
        if (hasNan) {
            out[i * ostride] = std::numeric_limits<double>::quiet_NaN();
            if (info) info[i] = 0;
            continue;
        }
        std::vector<double> cache(C.ex.cacheSize), ws(C.quad.wsSize(1));
        C.ex.fillCache1(cache.data(), pt.data(), dNone);
        auto f = [&](double x) { return evaluateSingle(C, cache.data(), ws.data(), x, coeffs, nullptr, nullptr, C.nugget); };
        int inf = 0;
        out[i * ostride] = inverseSingleBracket(ys[i * ystride], f, pt[D - 1], xtol, ytol, inf);
        if (info) info[i] = inf;
    }
    return 0;
}

// ----------------------------------------------------------------------------
// Sigmoid expansions: RectifiedMultivariateExpansion
// (MParT/RectifiedMultivariateExpansion.h:40-405) and, for one input,
// UnivariateExpansion<Sigmoid1d> (MParT/UnivariateExpansion.h:47-297).  The
// worker is the Expansion above with the sigmoid basis in the last input and
// the rectifier on the leading-input products.  No quadrature.
// ----------------------------------------------------------------------------
struct RectComponent {
    Sigmoid1d sig;
    Expansion ex;
    bool univariate = false;
    unsigned D() const { return ex.D; }
    unsigned T() const { return ex.numTerms(); }
};

// CreateSigmoid's parameters for a vector of centers (0 ok, -1 invalid).
// outStarts has room for nCenters entries; *nStarts receives their count.
int orc_sigmoid_from_centers(unsigned n, const double* centers, double edgeShape, int sumType, double* outCenters,
                             double* outWidths, double* outWeights, unsigned* outStarts, unsigned* nStarts) {
    Sigmoid1d S;
    if (!sigmoidFromCenters(centers, n, edgeShape, sumType, S)) return -1;
    std::copy(S.centers.begin(), S.centers.end(), outCenters);
    std::copy(S.widths.begin(), S.widths.end(), outWidths);
    std::copy(S.weights.begin(), S.weights.end(), outWeights);
    std::copy(S.starts.begin(), S.starts.end(), outStarts);
    *nStarts = (unsigned)S.starts.size();
    return 0;
}

static bool makeSigmoid(unsigned n, const double* c, const double* w, const double* wt, unsigned ns,
                        const unsigned* st, Sigmoid1d& S) {
    S.centers.assign(c, c + n);
    S.widths.assign(w, w + n);
    S.weights.assign(wt, wt + n);
    S.starts.assign(st, st + ns);
    return S.validate();
}

// Sigmoid1d::EvaluateAll / EvaluateDerivatives / EvaluateSecondDerivatives
// (which = 0, 1, 2).  -1: invalid parameters or maxOrder above the order.
int orc_sigmoid_eval(unsigned n, const double* c, const double* w, const double* wt, unsigned ns, const unsigned* st,
                     int which, unsigned maxOrder, double x, double* v, double* d1, double* d2) {
    Sigmoid1d S;
    if (!makeSigmoid(n, c, w, wt, ns, st, S)) return -1;
    if ((int)maxOrder > S.order) return -1;
    if (which == 0) S.evalAll(v, maxOrder, x);
    else if (which == 1) S.evalDerivs(v, d1, maxOrder, x);
    else S.evalSecond(v, d1, d2, maxOrder, x);
    return S.order;
}

// rect: -1 Identity, else the positive bijector kind.  nC == 0 puts the
// leading-input basis in the last input as well (the unrectified test case).
void* orc_rect_new(unsigned dim, unsigned nterms, const unsigned* starts, const unsigned* dims,
                   const unsigned* orders, int basis, int normalize, int rect, unsigned nC, const double* centers,
                   const double* widths, const double* weights, unsigned nStarts, const unsigned* sstarts,
                   int univariate) {
    RectComponent* R = new RectComponent();
    R->ex.ms.dim = dim;
    R->ex.ms.starts.assign(starts, starts + nterms + 1);
    unsigned nnz = starts[nterms];
    R->ex.ms.dims.assign(dims, dims + nnz);
    R->ex.ms.orders.assign(orders, orders + nnz);
    R->ex.ms.calcMaxDegrees();
    R->ex.basis.kind = basis;
    R->ex.basis.prob.normalize = normalize != 0;
    R->univariate = univariate != 0;
    R->ex.rect = R->univariate ? -1 : rect;
    if (nC) {
        if (!makeSigmoid(nC, centers, widths, weights, nStarts, sstarts, R->sig) ||
            (int)R->ex.ms.maxDeg[dim - 1] > R->sig.order) {
            delete R;
            return nullptr;
        }
        R->ex.diag = &R->sig;
    }
    R->ex.setup();
    return R;
}
void orc_rect_free(void* h) { delete (RectComponent*)h; }

// EvaluateImpl (RectifiedMultivariateExpansion.h:40-75; UnivariateExpansion.h:47-75).
int orc_rect_evaluate(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(R.D());
        for (unsigned d = 0; d < R.D(); ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dNone);
        R.ex.fillCache2(cache.data(), pt[R.D() - 1], dNone);
        out[i] = R.ex.evaluate(cache.data(), coeffs);
    }
    return 0;
}

// GradientImpl (:77-139): sens(i) * grad_x T(x_i), D x N.
int orc_rect_gradient(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, const double* sens,
                      double* out, long ors, long ocs) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    const unsigned D = R.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(D), g(D);
        for (unsigned d = 0; d < D; ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dInput);
        R.ex.fillCache2(cache.data(), pt[D - 1], dInput);
        R.ex.inputDerivative(cache.data(), coeffs, g.data(), 1);
        for (unsigned d = 0; d < D; ++d) out[d * ors + i * ocs] = g[d] * sens[i];
    }
    return 0;
}

// CoeffGradImpl (:141-190): sens(i) * dT/dc, T x N (row stride N).
int orc_rect_coeff_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs,
                        const double* sens, double* out) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    const unsigned T = R.T();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(R.D());
        for (unsigned d = 0; d < R.D(); ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dParameters);
        R.ex.fillCache2(cache.data(), pt[R.D() - 1], dParameters);
        R.ex.coeffDerivative(cache.data(), coeffs, out + i, N);
        for (unsigned t = 0; t < T; ++t) out[t * N + i] *= sens[i];
    }
    return 0;
}

// LogDeterminantImpl (:192-225): log of the diagonal derivative.
int orc_rect_logdet(void* h, const double* coeffs, const double* pts, long N, long rs, long cs, double* out) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(R.D());
        for (unsigned d = 0; d < R.D(); ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dNone);
        R.ex.fillCache2(cache.data(), pt[R.D() - 1], dDiagonal);
        out[i] = std::log(R.ex.diagonalDerivative(cache.data(), coeffs, 1));
    }
    return 0;
}

// LogDeterminantInputGradImpl (:279-325): [grad_x d_D T, d_D^2 T] / d_D T.
int orc_rect_logdet_input_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs,
                               double* out, long ors, long ocs) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    const unsigned D = R.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(D), g(D);
        for (unsigned d = 0; d < D; ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dMixedInput);
        R.ex.fillCache2(cache.data(), pt[D - 1], dMixedInput);
        R.ex.mixedInputDerivative(cache.data(), coeffs, g.data(), 1);
        R.ex.fillCache1(cache.data(), pt.data(), dDiagonal);
        R.ex.fillCache2(cache.data(), pt[D - 1], dDiagonal);
        double dd = R.ex.diagonalDerivative(cache.data(), coeffs, 1);
        for (unsigned d = 0; d < D; ++d) out[d * ors + i * ocs] = g[d] / dd;
    }
    return 0;
}

// LogDeterminantCoeffGradImpl (:327-370): d_c d_D T / d_D T, T x N.
int orc_rect_logdet_coeff_grad(void* h, const double* coeffs, const double* pts, long N, long rs, long cs,
                               double* out) {
    RectComponent& R = *(RectComponent*)h;
    View2 P{pts, rs, cs};
    const unsigned T = R.T();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        std::vector<double> cache(R.ex.cacheSize), pt(R.D());
        for (unsigned d = 0; d < R.D(); ++d) pt[d] = P.at(d, i);
        R.ex.fillCache1(cache.data(), pt.data(), dMixedCoeff);
        R.ex.fillCache2(cache.data(), pt[R.D() - 1], dMixedCoeff);
        R.ex.mixedCoeffDerivative(cache.data(), coeffs, 1, out + i, N);
        R.ex.fillCache1(cache.data(), pt.data(), dDiagonal);
        R.ex.fillCache2(cache.data(), pt[R.D() - 1], dDiagonal);
        double dd = R.ex.diagonalDerivative(cache.data(), coeffs, 1);
        for (unsigned t = 0; t < T; ++t) out[t * N + i] /= dd;
    }
    return 0;
}

// InverseImpl (:227-277; UnivariateExpansion.h:213-250): bracketed ITP root
// of T(x_<D, .) = r from x0 = the point's last entry (0 for one input).
int orc_rect_inverse(void* h, const double* coeffs, const double* xs, long numXs, long rs, long cs, const double* ys,
                     long ystride, long N, double xtol, double ytol, double* out, long ostride, int* info) {
    RectComponent& R = *(RectComponent*)h;
    if ((numXs != 1) && (numXs != N)) return -1;
    View2 P{xs, rs, cs};
    const unsigned D = R.D();
    ORC_PARALLEL_FOR
    for (long i = 0; i < N; ++i) {
        long xi = (numXs == 1) ? 0 : i;
        std::vector<double> pt(D);
        bool hasNan = std::isnan(ys[i * ystride]) && R.univariate;
        for (unsigned d = 0; d < D; ++d) {
            pt[d] = R.univariate ? 0.0 : P.at(d, xi);
            if (std::isnan(pt[d])) hasNan = true;
        }
        if (hasNan) {
            out[i * ostride] = std::numeric_limits<double>::quiet_NaN();
            if (info) info[i] = 0;
            continue;
        }
        std::vector<double> cache(R.ex.cacheSize);
        R.ex.fillCache1(cache.data(), pt.data(), dNone);
        auto f = [&](double x) {
            R.ex.fillCache2(cache.data(), x, dNone);
            return R.ex.evaluate(cache.data(), coeffs);
        };
        int inf = 0;
        out[i * ostride] = inverseSingleBracket(ys[i * ystride], f, pt[D - 1], xtol, ytol, inf);
        if (info) info[i] = inf;
    }
    return 0;
}

// ----------------------------------------------------------------------------
// Known-answer helpers for the pin tests.
// ----------------------------------------------------------------------------
// which: 0 EvaluateAll, 1 EvaluateDerivatives, 2 EvaluateSecondDerivatives.
// kind: 0 probabilist Hermite, 1 physicist Hermite, 2 Hermite functions.
int orc_basis(int kind, int normalize, int which, unsigned maxOrder, double x, double* v, double* d1, double* d2) {
    if (kind == 2) {
        HermiteFn hf;
        if (which == 0) hf.evalAll(v, maxOrder, x);
        else if (which == 1) hf.evalDerivs(v, d1, maxOrder, x);
        else hf.evalSecond(v, d1, d2, maxOrder, x);
        return 0;
    }
    Poly p{kind == 1, normalize != 0};
    if (which == 0) p.evalAll(v, maxOrder, x);
    else if (which == 1) p.evalDerivs(v, d1, maxOrder, x);
    else p.evalSecond(v, d1, d2, maxOrder, x);
    return 0;
}

double orc_posfunc(int kind, int which, double x) { return which == 0 ? posEval(kind, x) : posDeriv(kind, x); }

int orc_cc_rule(unsigned n, double* wts, double* pts) { ccRule(n, wts, pts); return 0; }

// Scalar or 2-vector test integrands from tests/Test_Quadrature.cpp:
// id 0: exp(x); id 1: exp(x) for x<0.5 else 1+exp(x); id 2: [exp(x), 2 exp(x)].
int orc_acc_test(int id, unsigned level, unsigned maxSub, double absTol, double relTol, unsigned minSub, double lb,
                 double ub, double* res, long* nevals) {
    ACC q;
    q.init(level, maxSub, absTol, relTol, minSub);
    unsigned fdim = (id == 2) ? 2 : 1;
    long n = 0;
    auto f = [&](double x, double* o) {
        n++;
        if (id == 0) o[0] = std::exp(x);
        else if (id == 1) o[0] = (x < 0.5) ? std::exp(x) : 1.0 + std::exp(x);
        else { o[0] = std::exp(x); o[1] = 2.0 * std::exp(x); }
    };
    struct Wrap {
        decltype(f)& g;
        void operator()(double x, double* o) const { g(x, o); }
        int failed() const { return 0; }
    } w{f};
    std::vector<double> ws(ACC::workspaceSize(maxSub, fdim));
    q.integrate(ws.data(), w, fdim, lb, ub, res);
    if (nevals) *nevals = n;
    return 0;
}

// Same test integrands through any quadrature kind (0 ClenshawCurtis with
// `n` points, 1 AdaptiveSimpson, 2 AdaptiveClenshawCurtis of level `n`).
int orc_quad_test(int kind, int id, unsigned n, unsigned maxSub, double absTol, double relTol, unsigned minSub,
                  double lb, double ub, double* res, long* nevals) {
    ACC q;
    q.init(kind == 2 ? n : 1, maxSub, absTol, relTol, minSub);
    q.kind = kind;
    if (kind == 0) {
        q.ruleP.resize(n);
        q.ruleW.resize(n);
        ccRule(n, q.ruleW.data(), q.ruleP.data());
    }
    unsigned fdim = (id == 2) ? 2 : 1;
    long cnt = 0;
    auto f = [&](double x, double* o) {
        cnt++;
        if (id == 0) o[0] = std::exp(x);
        else if (id == 1) o[0] = (x < 0.5) ? std::exp(x) : 1.0 + std::exp(x);
        else { o[0] = std::exp(x); o[1] = 2.0 * std::exp(x); }
    };
    struct Wrap {
        decltype(f)& g;
        void operator()(double x, double* o) const { g(x, o); }
        int failed() const { return 0; }
    } w{f};
    std::vector<double> ws(q.wsSize(fdim));
    q.integrate(ws.data(), w, fdim, lb, ub, res);
    if (nevals) *nevals = cnt;
    return 0;
}

// Root-finding test functions from tests/Test_RootFinding.cpp:
// id 0 identity, 1 sigmoid, 2 sigmoid combo, 3 flat (-1).
static double rfTest(int id, double x) {
    auto sig = [](double z) { return 1. / (std::exp(-z) + 1); };
    if (id == 0) return x;
    if (id == 1) return sig(x);
    if (id == 2) return sig(2 * (x - 1)) + 3 * sig(x * 0.5) + 0.5 * sig(1.5 * (x + 1));
    return -1.0;
}
double orc_rootfind_test(int id, double yd, double x0, double xtol, double ftol, int* info) {
    auto f = [&](double x) { return rfTest(id, x); };
    return inverseSingleBracket(yd, f, x0, xtol, ftol, *info);
}
int orc_findbracket_test(int id, double* xlb, double* ylb, double* xub, double* yub, double yd) {
    auto f = [&](double x) { return rfTest(id, x); };
    int info = 0;
    findBracket(f, *xlb, *ylb, *xub, *yub, yd, info);
    return info;
}

// Integrand values at a single node for one point (for KATs of
// MonotoneIntegrand, tests/Test_MonotoneComponent.cpp:22-356).  mode: 0 None,
// 1 Diagonal, 2 Parameters, 3 Input.  out must hold the mode's fdim.
int orc_integrand(void* h, const double* coeffs, const double* pt, double t, int mode, double* out) {
    Component& C = *(Component*)h;
    std::vector<double> cache(C.ex.cacheSize);
    DerivType dts[4] = {dNone, dDiagonal, dParameters, dInput};
    DerivType dt = dts[mode];
    C.ex.fillCache1(cache.data(), pt, dt == dInput ? dInput : dNone);
    Integrand ig{&C.ex, cache.data(), pt[C.D() - 1], coeffs, dt, C.nugget, C.pos};
    ig(t, out);
    return 0;
}

}  // extern "C"
