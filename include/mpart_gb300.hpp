// C++ API of the GB300 monotone-component path.  Mirrors the reference's
// host classes (MParT/ParameterizedFunctionBase.h, MParT/ConditionalMapBase.h,
// MParT/TriangularMap.h, MParT/MapFactory.h, MParT/MapOptions.h,
// MParT/MultiIndices/FixedMultiIndexSet.h, MultiIndex.h, MultiIndexLimiter.h,
// MultiIndexSet.h, MParT/MapObjective.h, MParT/TrainMap.h,
// MParT/TrainMapAdaptive.h) with device pointers in place of Kokkos device
// views.  Every *Impl call takes caller-allocated outputs, like
// the reference's virtual *Impl methods; calls are stream ordered and, unless
// the object is put in asynchronous mode, synchronous from the host's view.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <initializer_list>
#include <iosfwd>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace mpgb {

enum class BasisTypes { ProbabilistHermite, PhysicistHermite, HermiteFunctions };
enum class PosFuncTypes { Exp, SoftPlus };
enum class QuadTypes { ClenshawCurtis, AdaptiveSimpson, AdaptiveClenshawCurtis };
// MParT/MapOptions.h:31-39 and MParT/Sigmoid.h:45-48.
enum class SigmoidTypes { Logistic };
enum class EdgeTypes { SoftPlus };
enum class SigmoidSumSizeType { Linear, Constant };

// MParT/MapOptions.h:58-123 (the fields this path reads; same defaults).
struct MapOptions {
    BasisTypes basisType = BasisTypes::ProbabilistHermite;
    PosFuncTypes posFuncType = PosFuncTypes::SoftPlus;
    QuadTypes quadType = QuadTypes::AdaptiveSimpson;
    double quadAbsTol = 1e-6;
    double quadRelTol = 1e-6;
    unsigned int quadMaxSub = 30;
    unsigned int quadMinSub = 0;
    unsigned int quadPts = 5;
    bool contDeriv = true;
    bool basisNorm = true;
    double nugget = 0.0;
    // Sigmoid expansions (MParT/MapOptions.h:64-73).
    SigmoidTypes sigmoidType = SigmoidTypes::Logistic;
    EdgeTypes edgeType = EdgeTypes::SoftPlus;
    double edgeShape = 1.5;
    SigmoidSumSizeType sigmoidBasisSumType = SigmoidSumSizeType::Linear;
};

// A strided 2-D array (the reference's StridedMatrix = View<T**, LayoutStride>,
// MParT/Utilities/ArrayConversions.h:17).  Points are rows x cols with one
// column per point.  data may be device memory, or host memory for the
// host-staging overloads.
struct StridedMatrix {
    double* data = nullptr;
    int64_t rows = 0, cols = 0;
    int64_t rowStride = 0, colStride = 0;
    StridedMatrix() = default;
    StridedMatrix(double* d, int64_t r, int64_t c, int64_t rs, int64_t cs)
        : data(d), rows(r), cols(c), rowStride(rs), colStride(cs) {}
    static StridedMatrix RowMajor(double* d, int64_t r, int64_t c) { return StridedMatrix(d, r, c, c, 1); }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
};

// Compressed multi-index set (MParT/MultiIndices/FixedMultiIndexSet.h).
class FixedMultiIndexSet {
public:
    // Total-order set (src/MultiIndices/FixedMultiIndexSet.cpp:208-233).
    FixedMultiIndexSet(unsigned int dim, unsigned int maxOrder, unsigned int minOrder = 0);
    // Compressed form; each term's nonzero dims are sorted increasingly.
    FixedMultiIndexSet(unsigned int dim, std::vector<unsigned int> nzStarts, std::vector<unsigned int> nzDims,
                       std::vector<unsigned int> nzOrders);
    unsigned int Length() const { return dim_; }
    unsigned int Size() const { return (unsigned int)nzStarts.size() - 1; }
    std::vector<unsigned int> MaxDegrees() const { return maxDegrees; }
    std::vector<unsigned int> IndexToMulti(unsigned int index) const;
    int MultiToIndex(std::vector<unsigned int> const& multi) const;
    std::vector<unsigned int> NonzeroDiagonalEntries() const;
    // Terms (i, j) with i of this set outermost, the other set's dimensions
    // after this set's (src/MultiIndices/FixedMultiIndexSet.cpp:356-397).
    FixedMultiIndexSet Cartesian(FixedMultiIndexSet const& other) const;
    // This set's terms followed by the other's (FixedMultiIndexSet.cpp:400-431).
    FixedMultiIndexSet Concatenate(FixedMultiIndexSet const& other) const;

    std::vector<unsigned int> nzStarts, nzDims, nzOrders, maxDegrees;

private:
    unsigned int dim_;
    void CalculateMaxDegrees();
};

// MParT/MultiIndices/MultiIndex.h: a multi-index (stored densely).
class MultiIndex {
public:
    MultiIndex() = default;
    explicit MultiIndex(unsigned int length, unsigned int val = 0) : v_(length, val) {}
    MultiIndex(std::vector<unsigned int> const& v) : v_(v) {}
    MultiIndex(std::initializer_list<unsigned int> v) : v_(v) {}
    // A copy, as the reference's MultiIndex::Vector returns (safe on temporaries).
    std::vector<unsigned int> Vector() const { return v_; }
    unsigned int Length() const { return (unsigned int)v_.size(); }
    unsigned int Sum() const;
    unsigned int Max() const;
    unsigned int NumNz() const;
    bool HasNonzeroEnd() const { return !v_.empty() && v_.back() != 0; }
    // Get(Length()) reads 0; larger indices throw std::out_of_range (MultiIndex::Get).
    unsigned int Get(unsigned int i) const;
    // Sets entry i; returns whether it was nonzero (MultiIndex::Set).
    bool Set(unsigned int i, unsigned int val);
    std::string String() const;  // entries separated by spaces
    bool operator==(MultiIndex const& b) const { return v_ == b.v_; }
    bool operator!=(MultiIndex const& b) const { return v_ != b.v_; }
    // MultiIndex::operator<: length, total order, maximum, then entry by entry.
    bool operator<(MultiIndex const& b) const;
    bool operator>(MultiIndex const& b) const { return b < *this; }
    bool operator<=(MultiIndex const& b) const { return !(*this > b); }
    bool operator>=(MultiIndex const& b) const { return !(*this < b); }

private:
    std::vector<unsigned int> v_;
};

using LimiterType = std::function<bool(MultiIndex const&)>;

// MParT/MultiIndices/MultiIndexLimiter.h.
namespace MultiIndexLimiter {
struct TotalOrder {
    explicit TotalOrder(unsigned int totalOrder) : totalOrder(totalOrder) {}
    bool operator()(MultiIndex const& m) const { return m.Sum() <= totalOrder; }
    unsigned int totalOrder;
};
// Nonzero entries only in [lowerDim, lowerDim + length).
struct Dimension {
    Dimension(unsigned int lowerDim, unsigned int length) : lowerDim(lowerDim), length(length) {}
    bool operator()(MultiIndex const& m) const;
    unsigned int lowerDim, length;
};
// prod_i weights[i]^m[i] >= epsilon; weights in [0, 1], epsilon in (0, 1).
struct Anisotropic {
    Anisotropic(std::vector<double> const& weights, double epsilon);
    bool operator()(MultiIndex const& m) const;
    std::vector<double> weights;
    double epsilon;
};
struct MaxDegree {
    MaxDegree(unsigned int maxDegree, unsigned int length) : maxDegrees(length, maxDegree) {}
    explicit MaxDegree(std::vector<unsigned int> const& maxDegrees) : maxDegrees(maxDegrees) {}
    bool operator()(MultiIndex const& m) const;
    std::vector<unsigned int> maxDegrees;
};
struct None {
    bool operator()(MultiIndex const&) const { return true; }
};
// No cross terms with the last input.
struct Separable {
    bool operator()(MultiIndex const& m) const {
        return !m.HasNonzeroEnd() || m.Sum() == m.Get(m.Length() - 1);
    }
};
struct NonzeroDiag {
    bool operator()(MultiIndex const& m) const { return m.HasNonzeroEnd(); }
};
struct And {
    And(LimiterType a, LimiterType b) : a(std::move(a)), b(std::move(b)) {}
    bool operator()(MultiIndex const& m) const { return a(m) && b(m); }
    LimiterType a, b;
};
struct Or {
    Or(LimiterType a, LimiterType b) : a(std::move(a)), b(std::move(b)) {}
    bool operator()(MultiIndex const& m) const { return a(m) || b(m); }
    LimiterType a, b;
};
struct Xor {
    Xor(LimiterType a, LimiterType b) : a(std::move(a)), b(std::move(b)) {}
    bool operator()(MultiIndex const& m) const { return a(m) != b(m); }
    LimiterType a, b;
};
}  // namespace MultiIndexLimiter

// MParT/MultiIndices/MultiIndexSet.h (src/MultiIndices/MultiIndexSet.cpp):
// the active terms in activation order and the reference's bookkeeping that
// orders every query -- each multi-index seen gets a global number in order
// of first appearance, activating one adds the forward and backward
// neighbours the limiter allows as inactive entries, and edges are ordered
// sets of global numbers.
class MultiIndexSet {
public:
    explicit MultiIndexSet(unsigned int length, LimiterType const& limiter = MultiIndexLimiter::None());
    static MultiIndexSet CreateTotalOrder(unsigned int length, unsigned int maxOrder,
                                          LimiterType const& limiter = MultiIndexLimiter::None());
    static MultiIndexSet CreateTensorProduct(unsigned int length, unsigned int maxDegree,
                                             LimiterType const& limiter = MultiIndexLimiter::None());
    // The active terms, in order (the compressed form either way).
    FixedMultiIndexSet Fix(bool compress = true) const;

    void SetLimiter(LimiterType const& limiter);
    LimiterType GetLimiter() const { return limiter_; }
    // Whether a limiter was given (at construction or by SetLimiter).
    bool HasLimiter() const { return hasLimiter_; }

    unsigned int Length() const { return length_; }
    unsigned int Size() const { return (unsigned int)a2g_.size(); }
    std::vector<unsigned int> const& MaxOrders() const { return maxOrders_; }
    MultiIndex IndexToMulti(unsigned int activeIndex) const { return all_.at(a2g_.at(activeIndex)); }
    MultiIndex at(int activeIndex) const { return IndexToMulti((unsigned int)activeIndex); }
    MultiIndex const& operator[](int activeIndex) const { return all_[a2g_[activeIndex]]; }
    int MultiToIndex(MultiIndex const& m) const;  // active index, or -1
    std::vector<unsigned int> NonzeroDiagonalEntries() const;

    int AddActive(MultiIndex const& m);  // active index, or -1 when the limiter refuses it
    MultiIndexSet& operator+=(MultiIndex const& m) {
        AddActive(m);
        return *this;
    }
    MultiIndexSet& operator+=(MultiIndexSet const& rhs) {
        Union(rhs);
        return *this;
    }
    unsigned int Union(MultiIndexSet const& rhs);  // number of terms that became active
    void Activate(MultiIndex const& m);           // an admissible entry of the set

    bool IsActive(MultiIndex const& m) const;
    bool IsAdmissible(MultiIndex const& m) const;
    bool IsExpandable(unsigned int activeIndex) const;
    unsigned int NumActiveForward(unsigned int activeIndex) const;
    unsigned int NumForward(unsigned int activeIndex) const;
    std::vector<unsigned int> Frontier() const;
    std::vector<unsigned int> StrictFrontier() const;
    std::vector<MultiIndex> Margin() const;
    std::vector<MultiIndex> ReducedMargin() const;
    std::vector<MultiIndex> ReducedMarginDim(unsigned int dim) const;
    std::vector<unsigned int> Expand(unsigned int activeIndex);
    std::vector<unsigned int> Expand();

private:
    int addMulti(MultiIndex const& m);
    int addInactive(MultiIndex const& m);
    void addForward(int g, bool addInactive);
    void addBackward(int g, bool addInactive);
    void activate(int g);
    bool active(int g) const { return g2a_[g] >= 0; }
    bool admissible(int g) const;

    unsigned int length_;
    LimiterType limiter_;
    bool hasLimiter_ = false;
    std::vector<MultiIndex> all_;
    std::map<std::vector<unsigned int>, int> global_;
    std::vector<int> g2a_, a2g_;
    std::vector<std::set<int>> in_, out_;
    std::vector<unsigned int> maxOrders_;
};

struct ComponentProgram;
struct MapWorkspace;
class ConditionalMapBase;

// MParT/ParameterizedFunctionBase.h
class ParameterizedFunctionBase {
public:
    ParameterizedFunctionBase(unsigned int inDim, unsigned int outDim, unsigned int nCoeffs)
        : inputDim(inDim), outputDim(outDim), numCoeffs(nCoeffs) {}
    virtual ~ParameterizedFunctionBase();

    // Deep copy into coefficient storage owned by (or already wrapped by) this object
    // (src/ParameterizedFunctionBase.cpp:185-207).  host = true for a host pointer.
    virtual void SetCoeffs(const double* coeffs, unsigned int n, bool host = false, cudaStream_t stream = 0);
    // Alias caller-owned device memory (src/ParameterizedFunctionBase.cpp:219-228).
    virtual void WrapCoeffs(double* deviceCoeffs, unsigned int n) { WrapCoeffsLabeled(deviceCoeffs, n, std::string()); }
    double* Coeffs() const { return coeffs_; }
    // ParameterizedFunctionBase::Save / Load (MParT/ParameterizedFunctionBase.h:197-215):
    // the whole map in the reference's archive (what its ToBytes / pickle
    // write), for monotone components and triangular maps of them.
    void Save(std::ostream& os) const;
    static std::shared_ptr<ConditionalMapBase> Load(std::istream& is);
    // Label of the coefficient view the reference would hold after the same
    // calls, as its map archive records it: "ParameterizedFunctionBase<MemorySpace>
    // Coefficients" for storage SetCoeffs allocated, "coeffs" for a
    // TriangularMap built with moveCoeffs, "" for wrapped caller memory (an
    // unmanaged view); a triangular map's components carry the map's label
    // (src/ParameterizedFunctionBase.cpp:185-228, src/TriangularMap.cpp:38-98).
    std::string const& CoeffLabel() const { return coeffLabel_; }
    bool CheckCoefficients() const { return coeffs_ != nullptr; }
    void CheckCoefficients(std::string const& functionName) const;
    std::vector<double> CoeffMap() const;  // host copy

    virtual void EvaluateImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream = 0) = 0;
    virtual void GradientImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                              cudaStream_t stream = 0) = 0;
    virtual void CoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                               cudaStream_t stream = 0) = 0;

    const unsigned int inputDim, outputDim, numCoeffs;

    // Asynchronous mode: calls neither synchronise nor read the status word;
    // CheckStatus() does both later.  Needed for CUDA-graph capture.
    void SetAsync(bool async) { async_ = async; }
    bool Async() const { return async_; }

protected:
    virtual void OnCoeffsChanged() {}
    // WrapCoeffs with the label of the wrapped view.
    virtual void WrapCoeffsLabeled(double* deviceCoeffs, unsigned int n, std::string const& label);
    friend class TriangularMap;
    std::string coeffLabel_;
    double* coeffs_ = nullptr;
    double* owned_ = nullptr;
    bool async_ = false;
};

class MonotoneMapBase;

// MParT/ConditionalMapBase.h
class ConditionalMapBase : public ParameterizedFunctionBase {
public:
    using ParameterizedFunctionBase::ParameterizedFunctionBase;
    virtual void LogDeterminantImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream = 0) = 0;
    virtual void InverseImpl(StridedMatrix const& x1, StridedMatrix const& r, StridedMatrix const& output,
                             cudaStream_t stream = 0) = 0;
    virtual void LogDeterminantCoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                             cudaStream_t stream = 0) = 0;
    virtual void LogDeterminantInputGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                             cudaStream_t stream = 0) = 0;
    // Bounds on the coefficients (host arrays of numCoeffs): -inf / +inf
    // unless a subclass restricts them (ConditionalMapBase::CoeffBounds,
    // src/ConditionalMapBase.cpp:297-312).
    virtual void FillCoeffBoundsImpl(double* lb, double* ub) const;
};

// Parameters of a Sigmoid1d basis (MParT/Sigmoid.h:87-446): centers, widths
// and weights of the two edge terms and the sigmoids, and the first index of
// each sigmoid term (startInds, CSR style).
struct Sigmoid1dParams {
    std::vector<double> centers, widths, weights;
    std::vector<unsigned int> startInds;
    // Highest basis order: affine part, two edge terms, one per sigmoid term.
    int Order() const { return (int)startInds.size() + 3; }
    // Throws std::invalid_argument when the arrays do not form a basis (Sigmoid.h:386-431).
    void Validate() const;
    // ConstructStartInds (Sigmoid.h:95-130).
    static std::vector<unsigned int> ConstructStartInds(unsigned int numCenters, SigmoidSumSizeType sumType);
    static int ComputeNumSigmoids(unsigned int numCenters, SigmoidSumSizeType sumType);
    // CreateSigmoid (src/MapFactory.cpp:181-254): widths and weights from the
    // centers by the factory's rule of thumb.
    static Sigmoid1dParams FromCenters(std::vector<double> const& centers, double edgeShape,
                                       SigmoidSumSizeType sumType);
};

// Inverse solver options (MonotoneComponent.h:353-396).  method 0 is the
// reference's "Bracket" method (FindBracket + ITP, RootFinding.h:20-178);
// method 1 closes the same bracket by safeguarded Newton steps with the exact
// slope, to the same tolerances, in fewer evaluations (not the ITP iterate).
struct InverseOptions {
    double xtol = 1e-6;
    double ytol = 1e-6;
    int method = 0;
};

// Maps made of monotone components (a single MonotoneComponent or a
// TriangularMap of them) share one execution engine.
class MonotoneMapBase : public ConditionalMapBase {
public:
    MonotoneMapBase(unsigned int inDim, unsigned int outDim, unsigned int nCoeffs, MapOptions const& opts);
    ~MonotoneMapBase() override;

    void EvaluateImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream = 0) override;
    void GradientImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                      cudaStream_t stream = 0) override;
    void CoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                       cudaStream_t stream = 0) override;
    void LogDeterminantImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream = 0) override;
    void InverseImpl(StridedMatrix const& x1, StridedMatrix const& r, StridedMatrix const& output,
                     cudaStream_t stream = 0) override;
    void InverseImpl(StridedMatrix const& x1, StridedMatrix const& r, StridedMatrix const& output,
                     InverseOptions const& opts, int* deviceInfo, cudaStream_t stream);
    void LogDeterminantCoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                     cudaStream_t stream = 0) override;
    void LogDeterminantInputGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                     cudaStream_t stream = 0) override;

    // Fused forward + adjoint in one pass over the points.  Any output may be
    // empty.  coeffGrad (device, numCoeffs) receives
    //   sum_i [ sens(c,i) dT_c(x_i)/dc + logdetSens(i) d logdet(x_i)/dc ]
    // and inputGrad (inputDim x N) the same combination of input gradients.
    // logdetSens may be empty, in which case logdetSensScale is used for all points.
    void FusedForwardAdjoint(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& logdetSens,
                             double logdetSensScale, StridedMatrix const& outEval, StridedMatrix const& outLogDet,
                             double* coeffGrad, StridedMatrix const& inputGrad, cudaStream_t stream = 0);

    // Implicit-function adjoint of the inverse (no counterpart in the
    // reference, which does not differentiate Inverse).  pts = [x1; x]
    // (inputDim x N) with x = Inverse(x1, r); w (outputDim x N) holds the
    // weights of the functional L = sum_{k,i} w(k,i) x(k,i).  With
    // (dT/dx)^T lambda = w solved per point by back-substitution over the
    // components (last first), coeffGrad (device, numCoeffs; may be null)
    // receives dL/dc = -sum_i lambda_i^T dT/dc(x_i), and ptsGrad (inputDim x N;
    // may be empty) receives [dL/dx1; dL/dr] = [-lambda^T dT/dx1; lambda].
    // One launch per component; dT/dx_D is taken as g(df(x)) + nugget.
    void InverseCoeffGrad(StridedMatrix const& pts, StridedMatrix const& w, double* coeffGrad,
                          StridedMatrix const& ptsGrad, cudaStream_t stream = 0);

    // Standard-normal reverse KL of every component at once
    // (FastGaussianReverseKLObjective, src/MapObjective.cpp:93-234): per component
    // loss_c = mean(0.5 T_c^2 - logdet_c) and its coefficient gradient.
    // lossPerComp (device, outputDim) and grad (device, numCoeffs) are written.
    void KLObjective(StridedMatrix const& pts, double* lossPerComp, double* grad, cudaStream_t stream = 0);
    // Same for one component only (onlyComp >= 0), or all (onlyComp = -1).
    void KLObjective(StridedMatrix const& pts, double* lossPerComp, double* grad, int onlyComp, cudaStream_t stream);
    // The same objective through the reference objective's own call sequence,
    // per component: Evaluate, LogDeterminant, CoeffGrad with sens = T and
    // LogDeterminantCoeffGrad into dense numTerms x N scratch, then the
    // reductions (FastGaussianReverseKLObjective::CommonEval,
    // src/MapObjective.cpp:185-234).  T and Ld (N doubles each), DT and DL
    // (largest numTerms x N doubles each) are device scratch.  KLObjective
    // takes this route when the nugget is nonzero: Evaluate then integrates
    // without it and CoeffGrad with it, two quadrature trees.
    void KLObjectiveCalls(StridedMatrix const& pts, double* lossPerComp, double* grad, int onlyComp, double* T,
                          double* Ld, double* DT, double* DL, cudaStream_t stream);

    int CheckStatus(cudaStream_t stream = 0);  // synchronise, read and clear the status word
    // Process points grouped by |x_D| (default on); results do not depend on it
    // beyond summation order.
    void SetPointOrdering(bool on);
    // The next KLObjective call orders the samples by |x_D| again (later
    // calls order them by the interval counts of the call before).
    void ResetKLOrder();
    // Grow-only device buffer `slot` (0..7) of at least `bytes`, for host staging.
    double* StagingBuffer(int slot, size_t bytes, cudaStream_t stream);
    MapOptions const& Options() const { return opts_; }
    unsigned int NumMonotoneComponents() const { return (unsigned int)parts_.size(); }

    struct Part;
    std::vector<Part> const& Parts() const { return parts_; }

    struct Part {
        std::shared_ptr<ComponentProgram> prog;
        ParameterizedFunctionBase* owner;  // object holding the coefficients of this part
        unsigned int coeffOffset;          // offset inside the owner's coefficients
        unsigned int mapCoeffOffset;       // offset inside this map's coefficient vector
        unsigned int outRow;
    };

protected:
    MapOptions opts_;
    std::vector<Part> parts_;
    std::unique_ptr<MapWorkspace> ws_;
    void Prepare(cudaStream_t stream);
    void Finish(cudaStream_t stream, const char* fn);
};

// MParT/MonotoneComponent.h, constructed through MapFactory::CreateComponent.
class MonotoneComponent : public MonotoneMapBase {
public:
    MonotoneComponent(FixedMultiIndexSet const& mset, MapOptions const& opts);
    FixedMultiIndexSet const& GetMultiIndexSet() const { return mset_; }
    std::vector<unsigned int> DiagonalCoeffIndices() const { return mset_.NonzeroDiagonalEntries(); }

private:
    FixedMultiIndexSet mset_;
};

// Sigmoid expansions, constructed through MapFactory::CreateSigmoidComponent:
// MParT/RectifiedMultivariateExpansion.h for two or more inputs (Hermite
// functions in the leading inputs, the Sigmoid1d basis in the last one, the
// positive bijector as rectifier of the leading product of every term with a
// last-input factor) and MParT/UnivariateExpansion.h for one input.  The
// expansion is monotone in the last input when the coefficients of those
// terms are non-negative (the lower bounds of CoeffBounds).  Same engine as
// the monotone components, without quadrature.
class SigmoidComponent : public MonotoneMapBase {
public:
    SigmoidComponent(FixedMultiIndexSet const& mset, Sigmoid1dParams const& sigmoid, MapOptions const& opts);
    FixedMultiIndexSet const& GetMultiIndexSet() const { return mset_; }
    Sigmoid1dParams const& GetSigmoid() const { return sig_; }
    bool IsUnivariate() const { return mset_.Length() == 1; }
    // Terms that depend on the last input (all terms for one input).
    std::vector<unsigned int> DiagonalCoeffIndices() const;
    // 0 for DiagonalCoeffIndices (except the constant of a univariate
    // expansion), -inf elsewhere; +inf above (RectifiedMultivariateExpansion.h:374-390,
    // UnivariateExpansion.h:28-35).
    void FillCoeffBoundsImpl(double* lb, double* ub) const override;

private:
    FixedMultiIndexSet mset_;
    Sigmoid1dParams sig_;
};

// MParT/TriangularMap.h
class TriangularMap : public MonotoneMapBase {
public:
    TriangularMap(std::vector<std::shared_ptr<ConditionalMapBase>> const& components, bool moveCoeffs = false);
    void SetCoeffs(const double* coeffs, unsigned int n, bool host = false, cudaStream_t stream = 0) override;
    std::shared_ptr<ConditionalMapBase> GetComponent(unsigned int i) { return comps_.at(i); }
    unsigned int NumComponents() const { return (unsigned int)comps_.size(); }
    void FillCoeffBoundsImpl(double* lb, double* ub) const override;  // src/TriangularMap.cpp:313-325

protected:
    void WrapCoeffsLabeled(double* deviceCoeffs, unsigned int n, std::string const& label) override;

private:
    std::vector<std::shared_ptr<ConditionalMapBase>> comps_;
};

namespace MapFactory {
// src/MapFactory.cpp:22-27 and :105-124.
std::shared_ptr<ConditionalMapBase> CreateComponent(FixedMultiIndexSet const& mset, MapOptions opts);
std::shared_ptr<ConditionalMapBase> CreateTriangular(unsigned int inputDim, unsigned int outputDim,
                                                     unsigned int totalOrder, MapOptions options = MapOptions());
// MParT/MapFactory.h:138-213 and src/MapFactory.cpp:256-407.
std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(unsigned int inputDim, unsigned int offDiagOrder,
                                                           unsigned int crossOrder, std::vector<double> const& centers,
                                                           MapOptions opts);
std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(unsigned int inputDim, unsigned int totalOrder,
                                                           std::vector<double> const& centers, MapOptions opts);
std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(FixedMultiIndexSet const& mset,
                                                           std::vector<double> const& centers, MapOptions opts);
std::shared_ptr<ConditionalMapBase> CreateSigmoidTriangular(unsigned int inputDim, unsigned int outputDim,
                                                            unsigned int totalOrder,
                                                            std::vector<std::vector<double>> const& centers,
                                                            MapOptions opts);
}  // namespace MapFactory

// Thrown when the rectified integrand overflows (the reference throws from
// MonotoneIntegrand.h:183-190).
struct IntegrandError : public std::runtime_error {
    using std::runtime_error::runtime_error;
};

// MParT/TrainMap.h:19-58, same field names and defaults.  opt_alg "LD_SLSQP"
// (SLSQP's iteration for an unconstrained problem) or "LD_LBFGS"
// (limited-memory BFGS); NLopt is not used, so other names throw
// std::invalid_argument.  The tolerances are NLopt's stopping rules;
// opt_stopval and opt_maxtime are not used.
struct TrainOptions {
    std::string opt_alg = "LD_SLSQP";
    double opt_stopval = -std::numeric_limits<double>::infinity();
    double opt_ftol_rel = 1e-3;
    double opt_ftol_abs = 1e-3;
    double opt_xtol_rel = 1e-4;
    double opt_xtol_abs = 1e-4;
    int opt_maxeval = 1000;
    double opt_maxtime = std::numeric_limits<double>::infinity();
    int verbose = 0;
};

// KLObjective with the standard Gaussian reference density
// (MParT/MapObjective.h, ObjectiveFactory::CreateGaussianKLObjective,
// src/MapObjective.cpp:54-91): train and test are inputDim x N device
// matrices that stay owned by the caller.
class KLObjective {
public:
    KLObjective(StridedMatrix const& train, StridedMatrix const& test = StridedMatrix()) : train_(train), test_(test) {}
    // -mean(log N(T(x)) + log det dT/dx) over the training / test samples: the
    // components' reverse-KL losses plus (M/2) log 2 pi.
    double TrainError(std::shared_ptr<ConditionalMapBase> const& map, cudaStream_t stream = 0) const;
    double TestError(std::shared_ptr<ConditionalMapBase> const& map, cudaStream_t stream = 0) const;
    StridedMatrix const& Train() const { return train_; }
    StridedMatrix const& Test() const { return test_; }

private:
    StridedMatrix train_, test_;
};

// TrainMap(map, objective, options) (src/TrainMap.cpp:166-216) for a
// standard-Gaussian KLObjective on a map of monotone components: every
// component minimises its reverse KL (src/TrainMap.cpp:144-164), all of them
// in lockstep over one batched GPU step per iteration.  A map whose
// coefficients were never set starts from ones.  Returns the training error
// (TrainError at the result).
double TrainMap(std::shared_ptr<ConditionalMapBase> const& map, KLObjective const& objective,
                TrainOptions const& options, cudaStream_t stream = 0);

// MParT/TrainMapAdaptive.h:19-47: map and training options, maxPatience,
// maxSize and maxDegrees (a multi-index of inputDim entries, or empty).
struct ATMOptions : public MapOptions, public TrainOptions {
    unsigned int maxPatience = 10;
    unsigned int maxSize = std::numeric_limits<int>::max();
    MultiIndex maxDegrees;
};

// TrainMapAdaptive (src/TrainMapAdaptive.cpp:44-271): grows each output's
// set one reduced-margin term at a time and returns the triangular map of
// the best sets, which replace mset0.  The sets grow from their terms in
// order without a limiter: sets that carry one are refused
// (std::invalid_argument); maxDegrees bounds the degrees.
std::shared_ptr<ConditionalMapBase> TrainMapAdaptive(std::vector<MultiIndexSet>& mset0, KLObjective const& objective,
                                                     ATMOptions const& options, cudaStream_t stream = 0);

}  // namespace mpgb
