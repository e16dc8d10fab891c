// Map training: standard-normal reverse KL of a triangular map, minimised
// component by component as TrainMap does for a KLObjective with a
// standard-normal density (src/TrainMap.cpp:144-164, :166-216).  The
// reference hands each component to NLopt in turn; here every component's
// optimiser runs in lockstep and one batched launch (optionally replayed from
// a CUDA graph) evaluates all of their requests at once.  NLopt itself is not
// available; two optimisers of this library's own stand in for its algorithms:
// the iteration of SLSQP (the reference's default, LD_SLSQP) for a problem
// without constraints, and a limited-memory BFGS (LD_LBFGS), both with
// NLopt's stopping rules.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "../../include/mpart_gb300.hpp"
#include "mpgb_launch.h"
#include "mpgb_program.h"

namespace mpgb {

namespace {

#define TR_CUDA(call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA error in trainer: ") +      \
                                                        cudaGetErrorString(e_));                     \
    } while (0)

struct TrainOpts {
    int maxIters = 100;
    int maxEvals = 1000;
    double ftolRel = 0.0, ftolAbs = 0.0, xtolRel = 0.0, xtolAbs = 0.0, gtol = 0.0;
    int memory = 10;
    int algorithm = MPGB_OPT_SLSQP;
    bool precondition = false;  // L-BFGS: diagonal initial inverse Hessian from the squared per-point gradients
};

// NLopt's stopping test on one value: the change is below the absolute
// tolerance or below the relative tolerance times the mean magnitude.
bool relStop(double vold, double vnew, double reltol, double abstol) {
    if (std::isinf(vold)) return false;
    const double d = std::fabs(vnew - vold);
    return d < abstol || d < reltol * 0.5 * (std::fabs(vnew) + std::fabs(vold)) || (reltol > 0 && vnew == vold);
}

// Reverse-communication optimiser of one component's coefficients: the
// caller evaluates the objective and gradient at request() and passes them
// to tell() until done().
class Optimizer {
public:
    virtual ~Optimizer() = default;
    const std::vector<double>& request() const { return trial_; }
    bool done() const { return done_; }
    int iterations() const { return iters_; }
    int evaluations() const { return evals_; }
    double f() const { return f_; }
    const std::vector<double>& x() const { return x_; }
    double gradNorm() const {
        double s = 0;
        for (double v : g_) s += v * v;
        return std::sqrt(s);
    }
    virtual void tell(double f, const double* g) = 0;

protected:
    Optimizer(const double* x0, int n, const TrainOpts& o) : n_(n), o_(o), x_(x0, x0 + n), trial_(x0, x0 + n) {}
    static double dot(const std::vector<double>& a, const std::vector<double>& b) {
        double s = 0;
        for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
        return s;
    }
    bool converged0() const { return o_.gtol > 0 && gradNorm() <= o_.gtol; }
    // NLopt's tests between two iterates (and this library's iteration and
    // gradient-norm limits).
    bool stopAfter(double fOld, const std::vector<double>& xOld) const {
        if (iters_ >= o_.maxIters || evals_ >= o_.maxEvals || converged0()) return true;
        if (relStop(fOld, f_, o_.ftolRel, o_.ftolAbs)) return true;
        bool allX = true;
        for (int i = 0; i < n_ && allX; ++i) allX = relStop(xOld[i], x_[i], o_.xtolRel, o_.xtolAbs);
        return allX;
    }
    int n_;
    TrainOpts o_;
    std::vector<double> x_, trial_, g_;
    double f_ = 0;
    bool done_ = false;
    int iters_ = 0, evals_ = 0;
};

// The iteration of SLSQP (D. Kraft, "A software package for sequential
// quadratic programming", DFVLR-FB 88-28, 1988) for a problem without
// constraints or bounds, where its quadratic subproblem is min_d g'd +
// d'Bd/2: a quasi-Newton method whose matrix B starts as the identity and
// takes Powell's damped BFGS update (with s'u raised to 0.2 s'Bs where it is
// smaller), and whose line search starts from the full step, accepts when the
// decrease is at least a tenth of the linear prediction (or after ten
// reductions), and otherwise shrinks the step by the minimiser of the
// quadratic through the two values and the slope, at least to a tenth.
// B^-1 is kept and updated directly (the inverse form of the same update:
// with d = -B^-1 g exactly, B s = -alpha g), O(n^2) per iteration.  A
// non-finite trial value shrinks the step by a tenth and is never accepted.
class SLSQPU : public Optimizer {
public:
    SLSQPU(const double* x0, int n, const TrainOpts& o) : Optimizer(x0, n, o), H_((size_t)n * n, 0.0) {
        for (int i = 0; i < n; ++i) H_[(size_t)i * n + i] = 1.0;
    }
    void tell(double f, const double* g) override {
        ++evals_;
        if (first_) {
            first_ = false;
            f_ = f;
            g_.assign(g, g + n_);
            if (!std::isfinite(f) || converged0()) { done_ = true; return; }
            direction();
            return;
        }
        const double h1 = f - f_;
        const bool finite = std::isfinite(f);
        if (finite && (h1 <= 0.1 * h3_ || line_ > 10)) {
            const double fOld = f_;
            const std::vector<double> xOld = x_, gOld = g_;
            x_ = trial_;
            f_ = f;
            g_.assign(g, g + n_);
            ++iters_;
            update(gOld);
            if (stopAfter(fOld, xOld)) { done_ = true; trial_ = x_; return; }
            direction();
            return;
        }
        if (evals_ >= o_.maxEvals || line_ > 40) { done_ = true; trial_ = x_; return; }
        double a = finite ? h3_ / (2.0 * (h3_ - h1)) : 0.1;
        if (!(a > 0.1)) a = 0.1;
        alpha_ *= a;
        h3_ *= a;
        for (int i = 0; i < n_; ++i) { s_[i] *= a; trial_[i] = x_[i] + s_[i]; }
        ++line_;
    }

private:
    void direction() {
        s_.assign(n_, 0.0);
        for (int i = 0; i < n_; ++i) {
            double v = 0;
            const double* row = &H_[(size_t)i * n_];
            for (int j = 0; j < n_; ++j) v += row[j] * g_[j];
            s_[i] = -v;
        }
        h3_ = dot(g_, s_);
        if (!(h3_ < 0)) {  // not a descent direction: back to the identity
            std::fill(H_.begin(), H_.end(), 0.0);
            for (int i = 0; i < n_; ++i) { H_[(size_t)i * n_ + i] = 1.0; s_[i] = -g_[i]; }
            h3_ = dot(g_, s_);
        }
        alpha_ = 1.0;
        line_ = 1;
        for (int i = 0; i < n_; ++i) trial_[i] = x_[i] + s_[i];
    }
    void update(const std::vector<double>& gOld) {
        // s_ is the step taken; B s = -alpha g_old.
        std::vector<double> u(n_), v(n_);
        for (int i = 0; i < n_; ++i) {
            u[i] = g_[i] - gOld[i];
            v[i] = -alpha_ * gOld[i];
        }
        double h1 = dot(s_, u);
        const double h2 = dot(s_, v);
        if (!(h2 > 0)) return;
        const double h3 = 0.2 * h2;
        if (h1 < h3) {
            const double t = (h2 - h3) / (h2 - h1);
            for (int i = 0; i < n_; ++i) u[i] = t * u[i] + (1.0 - t) * v[i];
            h1 = h3;
        }
        // H <- (I - r s u') H (I - r u s') + r s s', r = 1 / s'u.
        const double r = 1.0 / h1;
        std::vector<double> Hu(n_);
        for (int i = 0; i < n_; ++i) {
            double w = 0;
            const double* row = &H_[(size_t)i * n_];
            for (int j = 0; j < n_; ++j) w += row[j] * u[j];
            Hu[i] = w;
        }
        const double c = r * r * dot(u, Hu) + r;
        for (int i = 0; i < n_; ++i) {
            double* row = &H_[(size_t)i * n_];
            for (int j = 0; j < n_; ++j) row[j] += c * s_[i] * s_[j] - r * (s_[i] * Hu[j] + Hu[i] * s_[j]);
        }
    }
    std::vector<double> H_, s_;
    double h3_ = 0, alpha_ = 1;
    int line_ = 0;
    bool first_ = true;
};

// Limited-memory BFGS (two-loop recursion, Nocedal & Wright Alg. 7.4 / 7.5)
// with a backtracking Armijo line search.
class LBFGS : public Optimizer {
public:
    // dinv (optional, n entries): the diagonal of the initial inverse
    // Hessian, scaled at every iteration by s'y / y'Dy of the newest pair.
    LBFGS(const double* x0, int n, const TrainOpts& o, const double* dinv = nullptr)
        : Optimizer(x0, n, o), dinv_(dinv ? std::vector<double>(dinv, dinv + n) : std::vector<double>()) {}

    void tell(double f, const double* g) override {
        ++evals_;
        if (first_) {
            first_ = false;
            f_ = f;
            g_.assign(g, g + n_);
            if (!std::isfinite(f) || converged0()) { done_ = true; return; }
            newDirection(true);
            return;
        }
        // line search
        const double gd = dot(gPrevDir_, d_);
        if (std::isfinite(f) && f <= f_ + 1e-4 * alpha_ * gd) {
            // accept
            std::vector<double> s(n_), y(n_);
            for (int i = 0; i < n_; ++i) {
                s[i] = trial_[i] - x_[i];
                y[i] = g[i] - g_[i];
            }
            const double sy = dot(s, y);
            if (sy > 1e-12 * std::sqrt(dot(s, s) * dot(y, y))) {
                S_.push_back(s);
                Y_.push_back(y);
                rho_.push_back(1.0 / sy);
                if ((int)S_.size() > o_.memory) {
                    S_.erase(S_.begin());
                    Y_.erase(Y_.begin());
                    rho_.erase(rho_.begin());
                }
            }
            const double fOld = f_;
            const std::vector<double> xOld = x_;
            x_ = trial_;
            f_ = f;
            g_.assign(g, g + n_);
            ++iters_;
            if (stopAfter(fOld, xOld)) {
                done_ = true;
                trial_ = x_;
                return;
            }
            newDirection(false);
            return;
        }
        // backtrack (quadratic interpolation, safeguarded to [0.1, 0.5] of the step)
        if (evals_ >= o_.maxEvals || ++backtracks_ > 40) {
            done_ = true;
            trial_ = x_;
            return;
        }
        double a = alpha_;
        double an = -gd * a * a / (2.0 * (f - f_ - gd * a));
        if (!std::isfinite(an)) an = 0.5 * a;
        an = std::min(std::max(an, 0.1 * a), 0.5 * a);
        alpha_ = an;
        for (int i = 0; i < n_; ++i) trial_[i] = x_[i] + alpha_ * d_[i];
    }

private:
    void newDirection(bool first) {
        // Two-loop recursion: d = -H g.
        std::vector<double> q = g_;
        const int m = (int)S_.size();
        std::vector<double> a(m);
        for (int i = m - 1; i >= 0; --i) {
            a[i] = rho_[i] * dot(S_[i], q);
            for (int j = 0; j < n_; ++j) q[j] -= a[i] * Y_[i][j];
        }
        if (dinv_.empty()) {
            double gamma = 1.0;
            if (m > 0) gamma = dot(S_[m - 1], Y_[m - 1]) / dot(Y_[m - 1], Y_[m - 1]);
            for (int j = 0; j < n_; ++j) q[j] *= gamma;
        } else {
            double gamma = 1.0;
            if (m > 0) {
                double yDy = 0;
                for (int j = 0; j < n_; ++j) yDy += Y_[m - 1][j] * dinv_[j] * Y_[m - 1][j];
                gamma = dot(S_[m - 1], Y_[m - 1]) / yDy;
            }
            for (int j = 0; j < n_; ++j) q[j] *= gamma * dinv_[j];
        }
        for (int i = 0; i < m; ++i) {
            const double b = rho_[i] * dot(Y_[i], q);
            for (int j = 0; j < n_; ++j) q[j] += S_[i][j] * (a[i] - b);
        }
        d_.resize(n_);
        for (int j = 0; j < n_; ++j) d_[j] = -q[j];
        if (dot(d_, g_) >= 0) {  // not a descent direction: restart from the (scaled) steepest descent
            S_.clear(); Y_.clear(); rho_.clear();
            for (int j = 0; j < n_; ++j) d_[j] = -g_[j] * (dinv_.empty() ? 1.0 : dinv_[j]);
        }
        alpha_ = 1.0;
        if (first || S_.empty()) {
            // no curvature pair yet: no coefficient moves by more than 1
            double dn = 0;
            for (double v : d_) dn = std::max(dn, std::fabs(v));
            alpha_ = dn > 0 ? std::min(1.0, 1.0 / dn) : 1.0;
        }
        gPrevDir_ = g_;
        backtracks_ = 0;
        for (int i = 0; i < n_; ++i) trial_[i] = x_[i] + alpha_ * d_[i];
    }

    std::vector<double> d_, gPrevDir_, dinv_;
    double alpha_ = 1;
    std::vector<std::vector<double>> S_, Y_;
    std::vector<double> rho_;
    bool first_ = true;
    int backtracks_ = 0;
};

std::unique_ptr<Optimizer> makeOptimizer(const double* x0, int n, const TrainOpts& o, const double* dinv) {
    if (o.algorithm == MPGB_OPT_LBFGS) return std::unique_ptr<Optimizer>(new LBFGS(x0, n, o, dinv));
    if (o.algorithm == MPGB_OPT_SLSQP) return std::unique_ptr<Optimizer>(new SLSQPU(x0, n, o));
    throw std::invalid_argument("TrainMap: unknown optimisation algorithm.");
}

struct Pinned {
    double* p = nullptr;
    explicit Pinned(size_t n) { TR_CUDA(cudaMallocHost(&p, std::max<size_t>(1, n) * sizeof(double))); }
    ~Pinned() { if (p) cudaFreeHost(p); }
};
struct Dev {
    double* p = nullptr;
    explicit Dev(size_t n) { TR_CUDA(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(double))); }
    ~Dev() { if (p) cudaFree(p); }
};

// One KL evaluation of all components: coefficients in, losses and gradients out.
struct KLStep {
    MonotoneMapBase& map;
    StridedMatrix pts;
    cudaStream_t s;
    // 0 batched (graph), 1 batched (direct launches), 2 one fused launch set per
    // component, 3 per component the reference objective's call sequence
    // (Evaluate, LogDeterminant, CoeffGrad with sens = T and
    // LogDeterminantCoeffGrad into dense outputs, then reductions).
    int mode;
    double* dCoef;
    Pinned hCoef, hLoss, hGrad;
    Dev dLoss, dGrad;
    std::unique_ptr<Dev> dT, dLd, dDenseT, dDenseL;  // mode 3 buffers
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graphKernels = 0;  // kernel nodes of the captured step
    unsigned nc, no;

    // The step runs on a private non-blocking stream (a graph cannot be
    // captured on the legacy default stream); the caller's stream is
    // synchronised first.
    KLStep(MonotoneMapBase& m, StridedMatrix const& p, cudaStream_t user, int md)
        : map(m), pts(p), s(nullptr), mode(md), dCoef(m.Coeffs()), hCoef(m.numCoeffs), hLoss(m.outputDim),
          hGrad(m.numCoeffs), dLoss(m.outputDim), dGrad(m.numCoeffs), nc(m.numCoeffs), no(m.outputDim) {
        TR_CUDA(cudaStreamSynchronize(user));
        TR_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        // Every run starts from the |x_D| order of the samples, whatever
        // earlier calls left, so that runs in different launch modes process
        // the samples in the same orders (bitwise-equal trajectories).
        map.ResetKLOrder();
        // Every step uploads hCoef: start from the map's current coefficients.
        TR_CUDA(cudaMemcpy(hCoef.p, dCoef, nc * sizeof(double), cudaMemcpyDefault));
        if (mode == 3) {
            size_t maxTerms = 1;
            for (auto& p : map.Parts()) {
                if (!dynamic_cast<MonotoneMapBase*>(p.owner) || p.owner->numCoeffs != (unsigned)p.prog->numTerms)
                    throw std::invalid_argument("KL mode 3 needs a map made of monotone components.");
                maxTerms = std::max<size_t>(maxTerms, p.prog->numTerms);
            }
            const size_t n = (size_t)pts.cols;
            dT.reset(new Dev(n));
            dLd.reset(new Dev(n));
            dDenseT.reset(new Dev(maxTerms * n));
            dDenseL.reset(new Dev(maxTerms * n));
            run();
            return;
        }
        // Warm-up (builds launch tables, sets kernel attributes) outside any capture.
        map.KLObjective(pts, dLoss.p, dGrad.p, mode == 2 ? 0 : -1, s);
        if (mode == 2)
            for (unsigned c = 1; c < map.NumMonotoneComponents(); ++c) map.KLObjective(pts, dLoss.p, dGrad.p, (int)c, s);
        TR_CUDA(cudaStreamSynchronize(s));
        if (mode == 0) {
            const bool wasAsync = map.Async();
            map.SetAsync(true);
            TR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            enqueue();
            TR_CUDA(cudaStreamEndCapture(s, &graph));
            map.SetAsync(wasAsync);
            TR_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            size_t nNodes = 0;
            TR_CUDA(cudaGraphGetNodes(graph, nullptr, &nNodes));
            std::vector<cudaGraphNode_t> nodes(nNodes);
            if (nNodes) TR_CUDA(cudaGraphGetNodes(graph, nodes.data(), &nNodes));
            for (auto n : nodes) {
                cudaGraphNodeType t;
                TR_CUDA(cudaGraphNodeGetType(n, &t));
                if (t == cudaGraphNodeTypeKernel) ++graphKernels;
            }
        }
    }
    ~KLStep() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
    void enqueue() {
        TR_CUDA(cudaMemcpyAsync(dCoef, hCoef.p, nc * sizeof(double), cudaMemcpyHostToDevice, s));
        if (mode == 3) {
            // (an overflowing trial shows as a non-finite objective; run()
            // clears the status)
            map.KLObjectiveCalls(pts, dLoss.p, dGrad.p, -1, dT->p, dLd->p, dDenseT->p, dDenseL->p, s);
        } else if (mode == 2) {
            for (unsigned c = 0; c < map.NumMonotoneComponents(); ++c) map.KLObjective(pts, dLoss.p, dGrad.p, (int)c, s);
        } else {
            map.KLObjective(pts, dLoss.p, dGrad.p, -1, s);
        }
        TR_CUDA(cudaMemcpyAsync(hLoss.p, dLoss.p, no * sizeof(double), cudaMemcpyDeviceToHost, s));
        TR_CUDA(cudaMemcpyAsync(hGrad.p, dGrad.p, nc * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    void run() {
        if (mode == 0) {
            TR_CUDA(cudaGraphLaunch(exec, s));
            countLaunches(s, graphKernels);
        } else {
            const bool wasAsync = map.Async();
            map.SetAsync(true);
            enqueue();
            map.SetAsync(wasAsync);
        }
        TR_CUDA(cudaStreamSynchronize(s));
        if (mode == 3)
            for (auto& p : map.Parts()) dynamic_cast<MonotoneMapBase*>(p.owner)->CheckStatus(s);
    }
};

}  // namespace
}  // namespace mpgb

namespace mpgb {

// The inverse of the mean squared per-point KL gradient of every coefficient
// at the map's coefficients, 1 / (mean_i (d l_i / d c_j)^2 + eps), eps a
// 1e-10 fraction of the component's largest mean: a diagonal scaling that
// puts coefficients whose terms differ in magnitude by orders of magnitude
// (high-order Hermite terms) on one footing for L-BFGS.  One pass of the
// reference objective's call sequence with dense outputs per component.
std::vector<double> inverseFisherDiagonal(MonotoneMapBase& map, StridedMatrix const& pts, cudaStream_t s) {
    size_t maxTerms = 1;
    for (auto& p : map.Parts()) {
        if (!dynamic_cast<MonotoneMapBase*>(p.owner) || p.owner->numCoeffs != (unsigned)p.prog->numTerms)
            throw std::invalid_argument("TrainMap: preconditioning needs a map made of monotone components.");
        maxTerms = std::max<size_t>(maxTerms, p.prog->numTerms);
    }
    const size_t n = (size_t)pts.cols;
    Dev T(n), Ld(n), DT(maxTerms * n), DL(maxTerms * n), loss(map.outputDim), grad(map.numCoeffs), sq(map.numCoeffs);
    const auto& parts = map.Parts();
    for (size_t c = 0; c < parts.size(); ++c) {
        map.KLObjectiveCalls(pts, loss.p, grad.p, (int)c, T.p, Ld.p, DT.p, DL.p, s);
        TR_CUDA(launchDenseKLSquares(DT.p, DL.p, parts[c].prog->numTerms, (long long)n, sq.p + parts[c].mapCoeffOffset,
                                     s));
    }
    std::vector<double> d(map.numCoeffs);
    TR_CUDA(cudaMemcpyAsync(d.data(), sq.p, d.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    TR_CUDA(cudaStreamSynchronize(s));
    map.CheckStatus(s);
    for (size_t c = 0; c < parts.size(); ++c) {
        const size_t off = parts[c].mapCoeffOffset, nt = parts[c].prog->numTerms;
        double mx = 0;
        for (size_t j = off; j < off + nt; ++j) mx = std::max(mx, d[j]);
        const double eps = mx > 0 ? 1e-10 * mx : 1.0;
        for (size_t j = off; j < off + nt; ++j) d[j] = 1.0 / (d[j] + eps);
    }
    return d;
}

// Standard-normal KL training of every component (src/TrainMap.cpp:144-164):
// lockstep optimisers, one per component, over one batched objective step
// per iteration.  Throws; sets the map's coefficients to the result.
void trainKL(MonotoneMapBase& map, StridedMatrix const& pts, TrainOpts const& o, int mode, cudaStream_t s,
             double* loss_per_comp, mpgb_train_result* res) {
    // A map without coefficients starts from ones (src/TrainMap.cpp:168-176).
    if (!map.CheckCoefficients()) {
        std::vector<double> ones(map.numCoeffs, 1.0);
        map.SetCoeffs(ones.data(), map.numCoeffs, true, s);
    }
    const auto& parts = map.Parts();
    std::vector<double> x0 = map.CoeffMap();
    std::vector<double> dinv;
    if (o.precondition && o.algorithm == MPGB_OPT_LBFGS) dinv = inverseFisherDiagonal(map, pts, s);
    KLStep step(map, pts, s, mode);
    std::vector<std::unique_ptr<Optimizer>> opt;
    for (auto& p : parts)
        opt.push_back(makeOptimizer(x0.data() + p.mapCoeffOffset,
                                    (int)((&p == &parts.back() ? map.numCoeffs : (&p + 1)->mapCoeffOffset) -
                                          p.mapCoeffOffset),
                                    o, dinv.empty() ? nullptr : dinv.data() + p.mapCoeffOffset));
    int steps = 0;
    double stepMs = 0.0;
    EventPair ev;
    const auto t0 = std::chrono::steady_clock::now();
    while (true) {
        bool any = false;
        for (size_t c = 0; c < opt.size(); ++c) {
            const auto& r = opt[c]->request();
            std::memcpy(step.hCoef.p + parts[c].mapCoeffOffset, r.data(), r.size() * sizeof(double));
            any |= !opt[c]->done();
        }
        if (!any) break;
        TR_CUDA(cudaEventRecord(ev.a, step.s));
        step.run();
        TR_CUDA(cudaEventRecord(ev.b, step.s));
        TR_CUDA(cudaEventSynchronize(ev.b));
        stepMs += ev.ms();
        ++steps;
        // A trial point whose integrand overflows gives its component a
        // non-finite objective, which the line search rejects (it steps
        // back); only an overflow at the starting point is an error.
        map.CheckStatus(step.s);
        for (size_t c = 0; c < opt.size(); ++c)
            if (!opt[c]->done()) opt[c]->tell(step.hLoss.p[c], step.hGrad.p + parts[c].mapCoeffOffset);
    }
    const double totalMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (size_t c = 0; c < opt.size(); ++c)
        if (!std::isfinite(opt[c]->f()))
            throw IntegrandError("TrainMap: MonotoneIntegrand: the objective is not finite at the starting "
                                 "coefficients (g(df) overflowed).");
    std::vector<double> xf(map.numCoeffs);
    double total = 0, gn2 = 0;
    int iters = 0, evals = 0;
    for (size_t c = 0; c < opt.size(); ++c) {
        gn2 += opt[c]->gradNorm() * opt[c]->gradNorm();
        std::memcpy(xf.data() + parts[c].mapCoeffOffset, opt[c]->x().data(), opt[c]->x().size() * sizeof(double));
        if (loss_per_comp) loss_per_comp[c] = opt[c]->f();
        total += opt[c]->f();
        iters = std::max(iters, opt[c]->iterations());
        evals = std::max(evals, opt[c]->evaluations());
    }
    map.SetCoeffs(xf.data(), map.numCoeffs, true, s);
    if (res) {
        res->total_loss = total;
        res->iterations = iters;
        res->evaluations = evals;
        res->steps = steps;
        res->ms_per_step = steps ? stepMs / steps : 0.0;
        res->total_ms = totalMs;
        res->grad_norm = std::sqrt(gn2);
    }
}

TrainOpts trainOptsFromC(const mpgb_train_options* opts) {
    TrainOpts o;
    o.maxIters = opts->max_iters;
    o.maxEvals = opts->max_evals;
    o.ftolRel = opts->ftol_rel;
    o.ftolAbs = opts->ftol_abs;
    o.xtolRel = opts->xtol_rel;
    o.xtolAbs = opts->xtol_abs;
    o.gtol = opts->gtol;
    o.memory = opts->memory > 0 ? opts->memory : 10;
    o.algorithm = opts->algorithm;
    o.precondition = opts->precondition != 0;
    if (o.algorithm != MPGB_OPT_SLSQP && o.algorithm != MPGB_OPT_LBFGS)
        throw std::invalid_argument("TrainOptions: algorithm must be MPGB_OPT_SLSQP or MPGB_OPT_LBFGS.");
    return o;
}

namespace {
MonotoneMapBase& monotoneMap(std::shared_ptr<ConditionalMapBase> const& map) {
    auto* m = dynamic_cast<MonotoneMapBase*>(map.get());
    if (!m) throw std::invalid_argument("KLObjective: the map must be a monotone component or a TriangularMap of them.");
    return *m;
}
double klError(MonotoneMapBase& m, StridedMatrix const& pts, cudaStream_t s) {
    if (pts.rows < m.inputDim) throw std::invalid_argument("KLObjective: the samples have fewer rows than inputDim.");
    StridedMatrix p(pts.data, m.inputDim, pts.cols, pts.rowStride, pts.colStride);
    Dev loss(m.outputDim), g(m.numCoeffs);
    m.KLObjective(p, loss.p, g.p, s);
    std::vector<double> lh(m.outputDim);
    TR_CUDA(cudaMemcpyAsync(lh.data(), loss.p, lh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    TR_CUDA(cudaStreamSynchronize(s));
    double v = 0.5 * m.outputDim * std::log(2.0 * 3.14159265358979323846);
    for (double l : lh) v += l;
    return v;
}
}  // namespace

double KLObjective::TrainError(std::shared_ptr<ConditionalMapBase> const& map, cudaStream_t stream) const {
    return klError(monotoneMap(map), train_, stream);
}

double KLObjective::TestError(std::shared_ptr<ConditionalMapBase> const& map, cudaStream_t stream) const {
    if (test_.empty()) throw std::invalid_argument("KLObjective::TestError: no test samples.");
    return klError(monotoneMap(map), test_, stream);
}

double TrainMap(std::shared_ptr<ConditionalMapBase> const& map, KLObjective const& objective,
                TrainOptions const& options, cudaStream_t stream) {
    MonotoneMapBase& m = monotoneMap(map);
    TrainOpts o;
    if (options.opt_alg == "LD_SLSQP") o.algorithm = MPGB_OPT_SLSQP;
    else if (options.opt_alg == "LD_LBFGS") o.algorithm = MPGB_OPT_LBFGS;
    else throw std::invalid_argument("TrainOptions: opt_alg " + options.opt_alg + " is not provided (LD_SLSQP, LD_LBFGS).");
    o.maxIters = o.maxEvals = options.opt_maxeval;
    o.ftolRel = options.opt_ftol_rel;
    o.ftolAbs = options.opt_ftol_abs;
    o.xtolRel = options.opt_xtol_rel;
    o.xtolAbs = options.opt_xtol_abs;
    StridedMatrix const& t = objective.Train();
    if (t.rows < m.inputDim) throw std::invalid_argument("TrainMap: the samples have fewer rows than inputDim.");
    StridedMatrix p(t.data, m.inputDim, t.cols, t.rowStride, t.colStride);
    trainKL(m, p, o, 0, stream, nullptr, nullptr);
    return objective.TrainError(map, stream);
}

int trainMapImpl(void* mapObj, mpgb_matrix samples, const mpgb_train_options* opts, double* loss_per_comp,
                 mpgb_train_result* res, void* stream, char* err, int errLen) {
    try {
        auto* map = static_cast<MonotoneMapBase*>(mapObj);
        if (!map || !opts) throw std::invalid_argument("null argument");
        StridedMatrix pts(samples.data, samples.rows, samples.cols, samples.row_stride, samples.col_stride);
        trainKL(*map, pts, trainOptsFromC(opts), opts->mode, (cudaStream_t)stream, loss_per_comp, res);
        return MPGB_OK;
    } catch (IntegrandError const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_INTEGRAND;
    } catch (std::invalid_argument const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_RUNTIME;
    }
}

int klStepTimeImpl(void* mapObj, mpgb_matrix samples, int mode, int steps, double* ms_per_step, double* loss,
                   double* grad, void* stream, char* err, int errLen) {
    try {
        auto* map = static_cast<MonotoneMapBase*>(mapObj);
        if (!map || steps <= 0) throw std::invalid_argument("bad argument");
        cudaStream_t s = (cudaStream_t)stream;
        StridedMatrix pts(samples.data, samples.rows, samples.cols, samples.row_stride, samples.col_stride);
        KLStep step(*map, pts, s, mode);
        std::vector<double> x0 = map->CoeffMap();
        std::memcpy(step.hCoef.p, x0.data(), x0.size() * sizeof(double));
        for (int i = 0; i < 3; ++i) step.run();
        EventPair ev;
        double tot = 0;
        for (int i = 0; i < steps; ++i) {
            TR_CUDA(cudaEventRecord(ev.a, step.s));
            step.run();
            TR_CUDA(cudaEventRecord(ev.b, step.s));
            TR_CUDA(cudaEventSynchronize(ev.b));
            tot += ev.ms();
        }
        *ms_per_step = tot / steps;
        if (loss) std::memcpy(loss, step.hLoss.p, map->outputDim * sizeof(double));
        if (grad) std::memcpy(grad, step.hGrad.p, map->numCoeffs * sizeof(double));
        return MPGB_OK;
    } catch (std::exception const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_RUNTIME;
    }
}

// ---------------------------------------------------------------------------
// Adaptive transport map (src/TrainMapAdaptive.cpp:44-271; Baptista et al.
// 2022): grow each component's multi-index set one term at a time, choosing
// the reduced-margin term whose coefficient has the largest KL gradient, and
// keep the sets with the best test objective.
// ---------------------------------------------------------------------------

// Multi-index set with the bookkeeping of the reference's MultiIndexSet
// (src/MultiIndices/MultiIndexSet.cpp), which fixes the order in which the
// adaptive loop meets its candidates: every multi-index the set has seen gets
// a global number in order of first appearance; activating one adds its
// forward neighbours m + e_d (d = 0..dim-1) and backward neighbours m - e_d
// as inactive entries where they are new, and records the edges between
// entries that exist (a sorted set of global numbers per entry and
// direction).  Active terms keep their order of activation (the term and
// coefficient order).  No limiter: every multi-index is allowed.  A set given
// as a list of terms is rebuilt by activating them in order, which is how the
// reference's total-order construction, += and Expand build theirs.
struct AdaptiveSet {
    unsigned dim = 0;
    std::vector<std::vector<unsigned>> terms;  // active terms, in activation order
    std::vector<std::vector<unsigned>> all;    // every entry, by global number
    std::map<std::vector<unsigned>, int> global;
    std::vector<int> activeOf;                 // global number -> active index or -1
    std::vector<int> globalOf;                 // active index -> global number
    std::vector<std::set<int>> inE, outE;      // backward / forward edges by global number

    bool has(const std::vector<unsigned>& m) const {
        auto it = global.find(m);
        return it != global.end() && activeOf[it->second] >= 0;
    }
    // Activates m (a new entry if needed): MultiIndexSet::AddActive.
    void add(const std::vector<unsigned>& m) {
        if (m.size() != dim) throw std::invalid_argument("multi-index of the wrong length");
        auto it = global.find(m);
        activate(it != global.end() ? it->second : newEntry(m));
    }
    // Active terms not yet expanded are given their forward neighbours that
    // are admissible (every backward neighbour active), in the reference's
    // order: the frontier's terms in activation order, each one's forward
    // entries by global number (MultiIndexSet::Expand).  Returns the active
    // indices of the new terms in that order, a term reached from several
    // frontier terms once for each, as the reference's does.
    std::vector<int> expand() {
        std::vector<int> pending;
        for (size_t a = 0; a < globalOf.size(); ++a) {
            const int g = globalOf[a];
            bool expandable = false;
            for (int f : outE[g])
                if (activeOf[f] < 0 && admissible(f)) { expandable = true; break; }
            if (!expandable) continue;
            for (int f : outE[g])
                if (activeOf[f] < 0 && admissible(f)) pending.push_back(f);
        }
        std::vector<int> out;
        for (int f : pending) {
            activate(f);
            out.push_back(activeOf[f]);
        }
        return out;
    }
    // Inactive entries whose existing backward neighbours are all active, by
    // global number (MultiIndexSet::ReducedMargin).
    std::vector<std::vector<unsigned>> reducedMargin() const {
        std::vector<std::vector<unsigned>> out;
        for (size_t g = 0; g < all.size(); ++g) {
            if (activeOf[g] >= 0) continue;
            bool ok = true;
            for (int b : inE[g]) ok = ok && activeOf[b] >= 0;
            if (ok) out.push_back(all[g]);
        }
        return out;
    }
    FixedMultiIndexSet fix() const { return fixTerms(dim, terms); }
    // Compressed fixed set of the given terms, in their order (MultiIndexSet::Fix(true)).
    static FixedMultiIndexSet fixTerms(unsigned dim, const std::vector<std::vector<unsigned>>& ts) {
        std::vector<unsigned> s{0}, d, o;
        for (const auto& t : ts) {
            for (unsigned e = 0; e < dim; ++e)
                if (t[e]) {
                    d.push_back(e);
                    o.push_back(t[e]);
                }
            s.push_back((unsigned)d.size());
        }
        return FixedMultiIndexSet(dim, s, d, o);
    }

private:
    static unsigned nnz(const std::vector<unsigned>& m) {
        unsigned n = 0;
        for (unsigned v : m) n += v != 0;
        return n;
    }
    bool admissible(int g) const {
        if (activeOf[g] >= 0) return true;
        unsigned n = 0;
        for (int b : inE[g]) n += activeOf[b] >= 0;
        return n == nnz(all[g]);
    }
    int newEntry(const std::vector<unsigned>& m) {
        const int g = (int)all.size();
        all.push_back(m);
        global[m] = g;
        activeOf.push_back(-1);
        inE.emplace_back();
        outE.emplace_back();
        link(g, false);
        return g;
    }
    // Edges between g and its existing neighbours; with grow, missing
    // neighbours become new inactive entries (which link themselves).
    void link(int g, bool grow) {
        for (unsigned d = 0; d < dim; ++d) {
            std::vector<unsigned> f = all[g];
            ++f[d];
            auto it = global.find(f);
            if (it != global.end()) {
                inE[it->second].insert(g);
                outE[g].insert(it->second);
            } else if (grow) {
                newEntry(f);
            }
        }
        for (unsigned d = 0; d < dim; ++d) {
            if (all[g][d] == 0) continue;
            std::vector<unsigned> b = all[g];
            --b[d];
            auto it = global.find(b);
            if (it != global.end()) {
                outE[it->second].insert(g);
                inE[g].insert(it->second);
            } else if (grow) {
                newEntry(b);
            }
        }
    }
    void activate(int g) {
        if (activeOf[g] >= 0) return;
        activeOf[g] = (int)globalOf.size();
        globalOf.push_back(g);
        terms.push_back(all[g]);
        link(g, true);
    }
};

struct ATMOpts {
    MapOptions map;
    TrainOpts train;
    int mode = 0;
    unsigned maxPatience = 10, maxSize = 0x7fffffff;
    std::vector<unsigned> maxDegrees;
    int verbose = 0;
};

namespace {

std::shared_ptr<ConditionalMapBase> atmComponent(const FixedMultiIndexSet& set, const MapOptions& o,
                                                 const std::vector<double>& coeffs) {
    auto c = MapFactory::CreateComponent(set, o);
    if (!coeffs.empty()) c->SetCoeffs(coeffs.data(), (unsigned)coeffs.size(), true);
    return c;
}

// KLObjective value (src/MapObjective.cpp:54-91): the components' reverse-KL
// losses plus (M/2) log 2 pi; and the coefficient gradient.
double atmObjective(MonotoneMapBase& map, StridedMatrix const& pts, std::vector<double>* grad, cudaStream_t s) {
    Dev loss(map.outputDim), g(map.numCoeffs);
    map.KLObjective(pts, loss.p, g.p, s);
    std::vector<double> lh(map.outputDim);
    TR_CUDA(cudaMemcpyAsync(lh.data(), loss.p, lh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (grad) {
        grad->resize(map.numCoeffs);
        TR_CUDA(cudaMemcpyAsync(grad->data(), g.p, grad->size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    TR_CUDA(cudaStreamSynchronize(s));
    double v = 0.5 * map.outputDim * std::log(2.0 * 3.14159265358979323846);
    for (double l : lh) v += l;
    return v;
}

}  // namespace

std::shared_ptr<ConditionalMapBase> trainMapAdaptive(std::vector<AdaptiveSet>& mset0, StridedMatrix const& train,
                                                     StridedMatrix const& test, ATMOpts const& o, cudaStream_t s,
                                                     mpgb_atm_result* res) {
    const auto t0 = std::chrono::steady_clock::now();
    const unsigned nOut = (unsigned)mset0.size();
    if (nOut == 0) throw std::invalid_argument("TrainMapAdaptive: no multi-index sets.");
    const unsigned inDim = (unsigned)train.rows;
    for (unsigned j = 0; j < nOut; ++j)
        if (mset0[j].dim != inDim - nOut + j + 1) {
            std::ostringstream os;
            os << "TrainMapAdaptive: multi-index set " << j << " has length " << mset0[j].dim << ", expected "
               << inDim - nOut + j + 1 << ".";
            throw std::invalid_argument(os.str());
        }
    if (test.rows != train.rows || test.cols == 0) throw std::invalid_argument("TrainMapAdaptive: bad test samples.");
    if (!o.maxDegrees.empty() && o.maxDegrees.size() != inDim)
        throw std::invalid_argument("TrainMapAdaptive: maxDegrees must have inputDim entries or none.");

    auto build = [&](std::vector<std::shared_ptr<ConditionalMapBase>> const& comps) {
        return std::make_shared<TriangularMap>(comps, true);
    };
    auto split = [&](TriangularMap& map) {
        std::vector<std::vector<double>> out(nOut);
        const std::vector<double> all = map.CoeffMap();
        unsigned off = 0;
        for (unsigned j = 0; j < nOut; ++j) {
            const unsigned n = (unsigned)mset0[j].terms.size();
            out[j].assign(all.begin() + off, all.begin() + off + n);
            off += n;
        }
        return out;
    };

    std::vector<std::shared_ptr<ConditionalMapBase>> comps(nOut);
    std::vector<std::vector<double>> coeffs(nOut);
    unsigned size = 0;
    for (unsigned j = 0; j < nOut; ++j) {
        coeffs[j].assign(mset0[j].terms.size(), 0.0);
        comps[j] = atmComponent(mset0[j].fix(), o.map, coeffs[j]);
        size += (unsigned)mset0[j].terms.size();
    }
    auto map = build(comps);
    trainKL(*map, train, o.train, o.mode, s, nullptr, nullptr);
    coeffs = split(*map);
    double best = atmObjective(*map, test, nullptr, s);
    if (o.verbose) std::printf("TrainMapAdaptive: initial size %u, test objective %.10g\n", size, best);
    std::vector<AdaptiveSet> bestSets = mset0;
    unsigned patience = 0, iterations = 0;
    double trainErr = 0.0;

    while (size < o.maxSize && patience < o.maxPatience) {
        // Every component with its set expanded (MultiIndexSet::Expand): the
        // new terms with zero coefficients, the others with their trained
        // ones.  Terms beyond the largest last-input order the kernels are
        // built for (kMaxLastOrder) cannot be represented: such candidates
        // are left out of the expanded component and of the choice.
        std::vector<AdaptiveSet> expanded(nOut);
        std::vector<std::vector<int>> cand(nOut);  // Expand's active indices, in its order
        std::vector<std::vector<int>> pos(nOut);   // active index -> coefficient of the expanded component
        std::vector<std::shared_ptr<ConditionalMapBase>> tmp(nOut);
        for (unsigned j = 0; j < nOut; ++j) {
            expanded[j] = mset0[j];
            cand[j] = expanded[j].expand();
            const auto& ts = expanded[j].terms;
            std::vector<std::vector<unsigned>> kept;
            std::vector<double> c;
            pos[j].assign(ts.size(), -1);
            for (size_t t = 0; t < ts.size(); ++t) {
                if (ts[t][expanded[j].dim - 1] > (unsigned)kMaxLastOrder) continue;
                pos[j][t] = (int)kept.size();
                kept.push_back(ts[t]);
                c.push_back(t < coeffs[j].size() ? coeffs[j][t] : 0.0);
            }
            tmp[j] = atmComponent(AdaptiveSet::fixTerms(expanded[j].dim, kept), o.map, c);
        }
        auto mapTmp = build(tmp);
        std::vector<double> grad;
        atmObjective(*mapTmp, train, &grad, s);
        // Largest |gradient| over the candidates below maxDegrees, scanned in
        // Expand's order with the first of equal values winning (findMaxGrad
        // and maxDegreeRMFilter, src/TrainMapAdaptive.cpp:6-42).
        int bestBlock = -1, bestTerm = -1;
        double bestVal = 0.0;
        unsigned off = 0;
        for (unsigned j = 0; j < nOut; ++j) {
            for (int k : cand[j]) {
                if (pos[j][k] < 0) continue;
                const auto& t = expanded[j].terms[k];
                bool bounded = false;
                for (unsigned d = 0; d < mset0[j].dim && !o.maxDegrees.empty(); ++d)
                    bounded |= t[d] >= o.maxDegrees[d];
                if (bounded) continue;
                const double v = std::fabs(grad[off + pos[j][k]]);
                if (v > bestVal) {
                    bestVal = v;
                    bestBlock = (int)j;
                    bestTerm = k;
                }
            }
            off += tmp[j]->numCoeffs;
        }
        if (bestBlock < 0) break;  // nothing left to add
        mset0[bestBlock].add(expanded[bestBlock].terms[bestTerm]);
        // The grown component starts again from zero coefficients (a new
        // component from the factory, src/TrainMapAdaptive.cpp:217-226); the
        // others keep their trained ones.
        coeffs[bestBlock].assign(mset0[bestBlock].terms.size(), 0.0);
        for (unsigned j = 0; j < nOut; ++j) comps[j] = atmComponent(mset0[j].fix(), o.map, coeffs[j]);
        ++size;
        map = build(comps);
        mpgb_train_result tr{};
        trainKL(*map, train, o.train, o.mode, s, nullptr, &tr);
        coeffs = split(*map);
        trainErr = tr.total_loss + 0.5 * nOut * std::log(2.0 * 3.14159265358979323846);
        const double testErr = atmObjective(*map, test, nullptr, s);
        ++iterations;
        ++patience;
        if (testErr < best) {
            best = testErr;
            bestSets = mset0;
            patience = 0;
        }
        if (o.verbose)
            std::printf("TrainMapAdaptive: size %u (component %d), train %.10g, test %.10g\n", size, bestBlock,
                        trainErr, testErr);
    }

    // The best sets, trained from zero coefficients (src/TrainMapAdaptive.cpp:243-254).
    mset0 = bestSets;
    for (unsigned j = 0; j < nOut; ++j)
        comps[j] = atmComponent(mset0[j].fix(), o.map, std::vector<double>(mset0[j].terms.size(), 0.0));
    map = build(comps);
    mpgb_train_result tr{};
    trainKL(*map, train, o.train, o.mode, s, nullptr, &tr);
    if (res) {
        unsigned n = 0;
        for (auto& m : mset0) n += (unsigned)m.terms.size();
        res->size = n;
        res->iterations = iterations;
        res->best_test_error = best;
        res->final_train_error = tr.total_loss + 0.5 * nOut * std::log(2.0 * 3.14159265358979323846);
        res->final_test_error = atmObjective(*map, test, nullptr, s);
        res->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return map;
}

// The C++ TrainMapAdaptive: the sets' terms in order go to the adaptive loop
// (which rebuilds the reference's bookkeeping from them), and the selected
// sets come back as MultiIndexSets of those terms.
std::shared_ptr<ConditionalMapBase> TrainMapAdaptive(std::vector<MultiIndexSet>& mset0, KLObjective const& objective,
                                                     ATMOptions const& options, cudaStream_t stream) {
    std::vector<AdaptiveSet> sets(mset0.size());
    for (size_t j = 0; j < mset0.size(); ++j) {
        if (mset0[j].HasLimiter())
            throw std::invalid_argument("TrainMapAdaptive: limiters on the initial multi-index sets are not "
                                        "supported; bound the degrees with ATMOptions::maxDegrees.");
        sets[j].dim = mset0[j].Length();
        for (unsigned int k = 0; k < mset0[j].Size(); ++k) sets[j].add(mset0[j].IndexToMulti(k).Vector());
        if (sets[j].terms.empty()) throw std::invalid_argument("TrainMapAdaptive: empty multi-index set.");
    }
    ATMOpts o;
    o.map = options;
    if (options.opt_alg == "LD_SLSQP") o.train.algorithm = MPGB_OPT_SLSQP;
    else if (options.opt_alg == "LD_LBFGS") o.train.algorithm = MPGB_OPT_LBFGS;
    else throw std::invalid_argument("TrainOptions: opt_alg " + options.opt_alg + " is not provided (LD_SLSQP, LD_LBFGS).");
    o.train.maxIters = o.train.maxEvals = options.opt_maxeval;
    o.train.ftolRel = options.opt_ftol_rel;
    o.train.ftolAbs = options.opt_ftol_abs;
    o.train.xtolRel = options.opt_xtol_rel;
    o.train.xtolAbs = options.opt_xtol_abs;
    o.maxPatience = options.maxPatience;
    o.maxSize = options.maxSize;
    o.maxDegrees = options.maxDegrees.Vector();
    o.verbose = options.verbose;
    StridedMatrix const& train = objective.Train();
    StridedMatrix const& test = objective.Test().empty() ? train : objective.Test();
    auto map = trainMapAdaptive(sets, train, test, o, stream, nullptr);
    for (size_t j = 0; j < mset0.size(); ++j) {
        MultiIndexSet s(sets[j].dim);
        for (auto const& t : sets[j].terms) s += MultiIndex(t);
        mset0[j] = s;
    }
    return map;
}

int trainMapAdaptiveImpl(unsigned int n_sets, const unsigned int* num_terms, const unsigned int* multis,
                         mpgb_matrix train, mpgb_matrix test, const mpgb_atm_options* opts, mpgb_map** out,
                         mpgb_atm_result* result, unsigned int* final_num_terms, void* stream, char* err, int errLen) {
    try {
        if (!num_terms || !multis || !opts || !out) throw std::invalid_argument("null argument");
        StridedMatrix tr(train.data, train.rows, train.cols, train.row_stride, train.col_stride);
        StridedMatrix te(test.data, test.rows, test.cols, test.row_stride, test.col_stride);
        const unsigned inDim = (unsigned)train.rows;
        if (n_sets == 0 || n_sets > inDim) throw std::invalid_argument("TrainMapAdaptive: bad number of sets.");
        std::vector<AdaptiveSet> sets(n_sets);
        size_t off = 0;
        for (unsigned j = 0; j < n_sets; ++j) {
            sets[j].dim = inDim - n_sets + j + 1;
            for (unsigned t = 0; t < num_terms[j]; ++t) {
                std::vector<unsigned> m(multis + off, multis + off + sets[j].dim);
                off += sets[j].dim;
                sets[j].add(m);
            }
            if (sets[j].terms.empty()) throw std::invalid_argument("TrainMapAdaptive: empty multi-index set.");
        }
        ATMOpts o;
        o.map = mapOptionsFromC(&opts->map);
        o.train = trainOptsFromC(&opts->train);
        o.mode = opts->train.mode;
        o.maxPatience = opts->max_patience;
        o.maxSize = opts->max_size;
        if (opts->max_degrees) o.maxDegrees.assign(opts->max_degrees, opts->max_degrees + inDim);
        o.verbose = opts->verbose;
        auto map = trainMapAdaptive(sets, tr, te, o, (cudaStream_t)stream, result);
        if (final_num_terms)
            for (unsigned j = 0; j < n_sets; ++j) final_num_terms[j] = (unsigned)sets[j].terms.size();
        *out = new mpgb_map{map};
        return MPGB_OK;
    } catch (IntegrandError const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_INTEGRAND;
    } catch (std::invalid_argument const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        if (err) { std::strncpy(err, e.what(), errLen - 1); err[errLen - 1] = 0; }
        return MPGB_ERR_RUNTIME;
    }
}

int reducedMarginImpl(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_out,
                      unsigned int* out, unsigned int cap_rows) {
    AdaptiveSet s;
    s.dim = dim;
    for (unsigned t = 0; t < n; ++t) s.add(std::vector<unsigned>(multis + (size_t)t * dim, multis + (size_t)(t + 1) * dim));
    const auto rm = s.reducedMargin();
    if (n_out) *n_out = (unsigned)rm.size();
    if (out) {
        if (cap_rows < rm.size()) throw std::invalid_argument("reduced margin: output too small");
        for (size_t k = 0; k < rm.size(); ++k) std::memcpy(out + k * dim, rm[k].data(), dim * sizeof(unsigned));
    }
    return MPGB_OK;
}

// The optimisers on host test functions: 0 the extended Rosenbrock function
// sum_i 100 (x_{2i+1} - x_{2i}^2)^2 + (1 - x_{2i})^2 from (-1.2, 1, ...),
// 1 the quadratic sum_i 10^(4 i / (n - 1)) (x_i - 1)^2 / 2 from 0 (condition
// number 10^4).  Returns the final point, objective and counts.
int optimizerSelfTestImpl(int algorithm, int which, int n, int maxIters, const double* dinv, double* xOut,
                          double* fOut, int* itersOut, int* evalsOut) {
    if (n < 2 || (which == 0 && n % 2) || which < 0 || which > 1) throw std::invalid_argument("bad test problem");
    TrainOpts o;
    o.algorithm = algorithm;
    o.maxIters = maxIters;
    o.maxEvals = 20 * maxIters;
    o.gtol = 1e-10;
    std::vector<double> x0(n);
    for (int i = 0; i < n; ++i) x0[i] = which == 0 ? ((i % 2) ? 1.0 : -1.2) : 0.0;
    auto opt = makeOptimizer(x0.data(), n, o, dinv);
    std::vector<double> g(n);
    while (!opt->done()) {
        const auto& x = opt->request();
        double f = 0;
        std::fill(g.begin(), g.end(), 0.0);
        if (which == 0) {
            for (int i = 0; i < n; i += 2) {
                const double a = x[i + 1] - x[i] * x[i], b = 1.0 - x[i];
                f += 100.0 * a * a + b * b;
                g[i] += -400.0 * a * x[i] - 2.0 * b;
                g[i + 1] += 200.0 * a;
            }
        } else {
            for (int i = 0; i < n; ++i) {
                const double w = std::pow(10.0, 4.0 * i / (n - 1)), d = x[i] - 1.0;
                f += 0.5 * w * d * d;
                g[i] = w * d;
            }
        }
        opt->tell(f, g.data());
    }
    std::memcpy(xOut, opt->x().data(), n * sizeof(double));
    *fOut = opt->f();
    *itersOut = opt->iterations();
    *evalsOut = opt->evaluations();
    return MPGB_OK;
}

int expandImpl(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_terms_out,
               unsigned int* terms_out, unsigned int* n_idx_out, unsigned int* idx_out, unsigned int cap) {
    AdaptiveSet s;
    s.dim = dim;
    for (unsigned t = 0; t < n; ++t) s.add(std::vector<unsigned>(multis + (size_t)t * dim, multis + (size_t)(t + 1) * dim));
    const size_t n0 = s.terms.size();
    const auto idx = s.expand();
    const size_t nNew = s.terms.size() - n0;
    if (n_terms_out) *n_terms_out = (unsigned)nNew;
    if (n_idx_out) *n_idx_out = (unsigned)idx.size();
    if (terms_out || idx_out) {
        if (cap < nNew || cap < idx.size()) throw std::invalid_argument("Expand: output too small");
        if (terms_out)
            for (size_t k = 0; k < nNew; ++k) std::memcpy(terms_out + k * dim, s.terms[n0 + k].data(), dim * sizeof(unsigned));
        if (idx_out)
            for (size_t k = 0; k < idx.size(); ++k) idx_out[k] = (unsigned)idx[k];
    }
    return MPGB_OK;
}

}  // namespace mpgb

