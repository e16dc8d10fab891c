// Host side of the GB300 monotone-component path: multi-index sets, the
// prefix-tree planner, the map classes of include/mpart_gb300.hpp and the C
// ABI of include/mpart_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "../../include/mpart_gb300.hpp"
#include "mpgb_launch.h"
#include "mpgb_types.h"
#include "mpgb_program.h"

namespace mpgb {

static const double kPiHost = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// FixedMultiIndexSet
// ---------------------------------------------------------------------------
static void fillTotalOrder(unsigned dim, unsigned maxOrder, unsigned minOrder, std::vector<unsigned>& work,
                           unsigned currDim, std::vector<unsigned>& starts, std::vector<unsigned>& dims,
                           std::vector<unsigned>& orders) {
    // Recursive enumeration of FixedMultiIndexSet::FillTotalOrder
    // (src/MultiIndices/FixedMultiIndexSet.cpp:508-549): dimension 0 outermost,
    // the last dimension fastest; nonzeros listed in increasing dimension.
    if (currDim + 1 < dim) {
        for (unsigned p = 0; p <= maxOrder; ++p) {
            work[currDim] = p;
            fillTotalOrder(dim, maxOrder - p, minOrder, work, currDim + 1, starts, dims, orders);
        }
    } else {
        for (unsigned p = 0; p <= maxOrder; ++p) {
            work[currDim] = p;
            unsigned tot = 0;
            for (unsigned i = 0; i <= currDim; ++i) tot += work[i];
            if (tot >= minOrder) {
                starts.push_back((unsigned)dims.size());
                for (unsigned i = 0; i < dim; ++i)
                    if (work[i] > 0) {
                        dims.push_back(i);
                        orders.push_back(work[i]);
                    }
            }
        }
    }
}

FixedMultiIndexSet::FixedMultiIndexSet(unsigned int dim, unsigned int maxOrder, unsigned int minOrder) : dim_(dim) {
    if (dim == 0) throw std::invalid_argument("FixedMultiIndexSet: dimension must be positive.");
    std::vector<unsigned> work(dim, 0);
    fillTotalOrder(dim, maxOrder, minOrder, work, 0, nzStarts, nzDims, nzOrders);
    nzStarts.push_back((unsigned)nzDims.size());
    CalculateMaxDegrees();
}

FixedMultiIndexSet::FixedMultiIndexSet(unsigned int dim, std::vector<unsigned int> starts,
                                       std::vector<unsigned int> dims, std::vector<unsigned int> orders)
    : nzStarts(std::move(starts)), nzDims(std::move(dims)), nzOrders(std::move(orders)), dim_(dim) {
    if (dim == 0) throw std::invalid_argument("FixedMultiIndexSet: dimension must be positive.");
    if (nzStarts.empty() || nzStarts.front() != 0 || nzStarts.back() != nzDims.size() ||
        nzDims.size() != nzOrders.size())
        throw std::invalid_argument("FixedMultiIndexSet: inconsistent compressed arrays.");
    for (size_t t = 0; t + 1 < nzStarts.size(); ++t) {
        if (nzStarts[t + 1] < nzStarts[t]) throw std::invalid_argument("FixedMultiIndexSet: nzStarts must increase.");
        // Sort each term's nonzeros by dimension (FixedMultiIndexSet.h:36-41).
        std::vector<std::pair<unsigned, unsigned>> nz;
        for (unsigned i = nzStarts[t]; i < nzStarts[t + 1]; ++i) {
            if (nzDims[i] >= dim) throw std::invalid_argument("FixedMultiIndexSet: dimension index out of range.");
            if (nzOrders[i] == 0) throw std::invalid_argument("FixedMultiIndexSet: stored orders must be nonzero.");
            nz.push_back({nzDims[i], nzOrders[i]});
        }
        std::sort(nz.begin(), nz.end());
        for (size_t j = 1; j < nz.size(); ++j)
            if (nz[j].first == nz[j - 1].first)
                throw std::invalid_argument("FixedMultiIndexSet: repeated dimension within a term.");
        for (size_t j = 0; j < nz.size(); ++j) {
            nzDims[nzStarts[t] + j] = nz[j].first;
            nzOrders[nzStarts[t] + j] = nz[j].second;
        }
    }
    CalculateMaxDegrees();
}

void FixedMultiIndexSet::CalculateMaxDegrees() {
    maxDegrees.assign(dim_, 0);
    for (size_t i = 0; i < nzOrders.size(); ++i) maxDegrees[nzDims[i]] = std::max(maxDegrees[nzDims[i]], nzOrders[i]);
}

std::vector<unsigned int> FixedMultiIndexSet::IndexToMulti(unsigned int index) const {
    if (index >= Size()) throw std::out_of_range("FixedMultiIndexSet::IndexToMulti: index out of range.");
    std::vector<unsigned int> m(dim_, 0);
    for (unsigned i = nzStarts[index]; i < nzStarts[index + 1]; ++i) m[nzDims[i]] = nzOrders[i];
    return m;
}

int FixedMultiIndexSet::MultiToIndex(std::vector<unsigned int> const& multi) const {
    for (unsigned t = 0; t < Size(); ++t)
        if (IndexToMulti(t) == multi) return (int)t;
    return -1;
}

std::vector<unsigned int> FixedMultiIndexSet::NonzeroDiagonalEntries() const {
    std::vector<unsigned int> out;
    for (unsigned t = 0; t < Size(); ++t)
        if (nzStarts[t + 1] > nzStarts[t] && nzDims[nzStarts[t + 1] - 1] == dim_ - 1) out.push_back(t);
    return out;
}

FixedMultiIndexSet FixedMultiIndexSet::Cartesian(FixedMultiIndexSet const& other) const {
    std::vector<unsigned> st{0}, dm, od;
    for (unsigned i = 0; i < Size(); ++i) {
        for (unsigned j = 0; j < other.Size(); ++j) {
            for (unsigned k = nzStarts[i]; k < nzStarts[i + 1]; ++k) {
                dm.push_back(nzDims[k]);
                od.push_back(nzOrders[k]);
            }
            for (unsigned k = other.nzStarts[j]; k < other.nzStarts[j + 1]; ++k) {
                dm.push_back(dim_ + other.nzDims[k]);
                od.push_back(other.nzOrders[k]);
            }
            st.push_back((unsigned)dm.size());
        }
    }
    return FixedMultiIndexSet(dim_ + other.Length(), st, dm, od);
}

FixedMultiIndexSet FixedMultiIndexSet::Concatenate(FixedMultiIndexSet const& other) const {
    if (Length() != other.Length()) {
        std::ostringstream os;
        os << "Length of multiindices must be the same but first set has length " << Length()
           << " multis and second set has length " << other.Length() << " multis.";
        throw std::invalid_argument(os.str());
    }
    std::vector<unsigned> st(nzStarts.begin(), nzStarts.end() - 1), dm = nzDims, od = nzOrders;
    for (unsigned v : other.nzStarts) st.push_back((unsigned)nzDims.size() + v);
    dm.insert(dm.end(), other.nzDims.begin(), other.nzDims.end());
    od.insert(od.end(), other.nzOrders.begin(), other.nzOrders.end());
    return FixedMultiIndexSet(dim_, st, dm, od);
}

// ---------------------------------------------------------------------------
// Sigmoid1d parameters
// ---------------------------------------------------------------------------
int Sigmoid1dParams::ComputeNumSigmoids(unsigned int numCenters, SigmoidSumSizeType sumType) {
    if (sumType == SigmoidSumSizeType::Constant) return (int)numCenters - 2;
    if (numCenters < 2) return -1;
    return (int)((std::sqrt(1.0 + 8.0 * ((double)numCenters - 2.0)) - 1.0) / 2.0);
}

std::vector<unsigned int> Sigmoid1dParams::ConstructStartInds(unsigned int centerSize, SigmoidSumSizeType sumType) {
    std::vector<unsigned int> out;
    if (centerSize <= 2) return out;
    int numTerms = ComputeNumSigmoids(centerSize, sumType);
    if (sumType == SigmoidSumSizeType::Linear) {
        if ((int)(centerSize - 2) != numTerms * (numTerms + 1) / 2)
            throw std::invalid_argument(
                "Sigmoid: Could not construct starting indices.  The size of the centers array cannot be used with "
                "the Linear sum type.");
        out.resize(numTerms);
        out[0] = 2;
        for (int i = 1; i < numTerms; ++i) out[i] = out[i - 1] + i;
    } else {
        numTerms = (int)centerSize - 2;
        out.resize(numTerms);
        out[0] = 2;
        for (int i = 1; i < numTerms; ++i) out[i] = out[i - 1] + 1;
    }
    return out;
}

void Sigmoid1dParams::Validate() const {
    if (centers.size() != widths.size() || centers.size() != weights.size() || centers.size() < startInds.size()) {
        std::ostringstream os;
        os << "Sigmoid: incompatible dims of centers and widths.\ncenters: " << centers.size()
           << ", \nwidths: " << widths.size() << ",\nweights: " << weights.size() << "\n";
        throw std::invalid_argument(os.str());
    }
    if (centers.size() < 2)
        throw std::invalid_argument(
            "Sigmoid: centers/widths/weights too short.\nLength should be of form 2+(1+2+3+...+n) for some order n>=0");
    if (!startInds.empty()) {
        if (startInds[0] != 2) {
            std::ostringstream os;
            os << "Sigmoid: First term must start at index 2, but has startInds(0)=" << startInds[0];
            throw std::invalid_argument(os.str());
        }
        for (size_t i = 1; i < startInds.size(); ++i) {
            if (startInds[i] <= startInds[i - 1])
                throw std::invalid_argument("Sigmoid: Starting indices must be strictly increasing.");
            if (startInds[i] >= centers.size()) {
                std::ostringstream os;
                os << "Sigmoid: All starting indices must be smaller than the number of sigmoid centers but startInds("
                   << i << ")=" << startInds[i] << " and centers.extent(0)=" << centers.size() << ".";
                throw std::invalid_argument(os.str());
            }
        }
    }
    if (Order() > kMaxLastOrder) {
        std::ostringstream os;
        os << "Sigmoid: " << startInds.size() << " sigmoid terms give order " << Order()
           << ", above the supported maximum " << kMaxLastOrder << ".";
        throw std::invalid_argument(os.str());
    }
}

Sigmoid1dParams Sigmoid1dParams::FromCenters(std::vector<double> const& c, double edgeShape,
                                             SigmoidSumSizeType sumType) {
    const unsigned n = (unsigned)c.size();
    if (n < 2)
        throw std::invalid_argument(
            "Sigmoid: centers/widths/weights too short.\nLength should be of form 2+(1+2+3+...+n) for some order n>=0");
    const int numSig = ComputeNumSigmoids(n, sumType);
    Sigmoid1dParams S;
    S.centers = c;
    S.widths.assign(n, 0.0);
    S.weights.assign(n, 1.0);
    S.widths[0] = edgeShape;
    S.weights[0] = 1.0 / edgeShape;
    S.widths[1] = edgeShape;
    S.weights[1] = 1.0 / edgeShape;
    if (sumType == SigmoidSumSizeType::Linear) {
        // Term i has i + 1 sigmoids; the first i get widths from the spacing of
        // their neighbours (the edge centers at the ends), the last keeps 0.
        for (int i = 0; i < numSig; i++) {
            const int start = 2 + (i * (i + 1)) / 2;
            for (int j = 0; j < i; j++) {
                const double prev = (j == 0 || i == 0) ? c[0] : c[start + j - 1];
                const double next = (j == i - 1 || i == 0) ? c[1] : c[start + j];
                S.widths[start + j] = 2 / (next - prev);
                S.weights[start + j] = 1.;
            }
        }
    } else if (numSig > 0) {
        std::sort(S.centers.begin() + 2, S.centers.end());
        const std::vector<double>& h = S.centers;
        S.widths[2] = (numSig > 1) ? 4.0 / (h[3] - h[2]) : 8.0 / std::abs(h[1] - h[0]);
        for (int i = 1; i < numSig - 1; i++) S.widths[2 + i] = 8.0 / (h[3 + i] - h[1 + i]);
        if (numSig > 1) S.widths[2 + numSig - 1] = 4.0 / (h[2 + numSig - 1] - h[2 + numSig - 2]);
    }
    S.startInds = ConstructStartInds(n, sumType);
    S.Validate();
    return S;
}

// ---------------------------------------------------------------------------
// Per-map device workspace (grow-only buffers).
// ---------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t b, cudaStream_t s) {
        if (b <= bytes) return;
        if (p) {
            MPGB_CUDA(cudaStreamSynchronize(s));
            MPGB_CUDA(cudaFree(p));
            p = nullptr;
        }
        size_t nb = std::max<size_t>(b, 256);
        MPGB_CUDA(cudaMalloc(&p, nb));
        bytes = nb;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    template <class T>
    T* as() const { return (T*)p; }
};

struct GatherDescHost {
    const double* src;
    const int32_t* slotTerm;
    int slotOffset;
    int nSlots;
};

// Launch tables of a KL step, cached per (N, component subset) so that a
// step issues only kernel launches (capturable in a CUDA graph).
struct KLPlan {
    long long N = -1;
    int onlyComp = -2;
    int nItems = 0;
    std::vector<std::vector<int>> itemsOf;
    std::vector<int> rowOff;   // first row of each component in rowBase
    std::vector<int> lossOff;  // first entry of each component in lossSlots
    DevBuf items, rowBase, lossSlots;
    size_t partialDoubles = 0;
    // The step's reductions (one launch for all components).
    DevBuf reduceDesc;
    int nReduce = 0, maxTerms = 0;
    // Processing order of the samples: sorted once per sample array (the
    // points of a training run do not change between steps).  Any
    // permutation gives the same results up to summation order, so a stale
    // order after the caller rewrites the array in place costs only speed.
    DevBuf perm;
    const double* permPts = nullptr;
    long long permRs = 0, permCs = 0;
    // Each call records every sample's quadrature interval count per
    // component (costKey) and sorts by it, so the next call -- the next step
    // of a training run, at nearby coefficients -- groups samples of similar
    // cost in a warp; the first call sorts by |x_D|.  The order depends only
    // on the samples and the coefficient history, so launch modes at the same
    // history process the samples in the same order (bitwise-equal results).
    DevBuf costKey;
    long long rcTotal = 0;  // rectifier cache of sigmoid expansions (doubles)
};

struct MapWorkspace {
    DevBuf comps, cm, gather, items, partials, rowBase, lossPart, lossSlots, logdetRows, status, reduceDesc;
    DevBuf stage[8];
    std::vector<CompDesc> hostComps;
    std::vector<GatherDescHost> hostGather;
    int totalSlots = 0;
    int numSMs = 0;
    QuadParams quad{};
    BasisConsts bc{};
    int pmax = 1, dmax = 1, nBmax = 0, depthMax = 0;
    int stageNeed = 0;  // doubles of the largest phase-A staging among the monotone components (<= kStageCap)
    int smemPerSM = 0;
    int basis = 0;  // kernel family: the options' basis, or kBasisSigmoid
    bool built = false;
    std::vector<std::unique_ptr<KLPlan>> klPlans;
    DevBuf perm, sortHist;
    DevBuf implicitAcc;  // back-substitution sums when the caller wants no input gradient
    DevBuf rcache;       // rectifier cache of sigmoid expansions (reduced adjoints)
    DevBuf inverseDefer; // two-pass inverse: number of deferred points
    DevBuf inverseKey;   // inverse processing order: per-target sort keys
    DevBuf inverseA;     // inverse: a_k of the component being solved, (pmax + 1) x N
    DevBuf inverseList;  // inverse: points left to the warp pass
    DevBuf inverseStack; // inverse: the warp pass's interval stacks
    DevBuf inverseState; // inverse: solver states of the points left to the warp pass
    DevBuf klT, klLd, klDT, klDL;  // KLObjectiveCalls scratch (nonzero nugget)
    bool ordering = true;
};

}  // namespace mpgb

// Coefficient gather over several components (separate translation unit needs no kernel here).
namespace mpgb {
__global__ void gatherMultiKernel(const GatherDescHost* descs, int nComps, double* cm) {
    const int c = blockIdx.y;
    if (c >= nComps) return;
    const GatherDescHost g = descs[c];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < g.nSlots; s += gridDim.x * blockDim.x) {
        const int t = g.slotTerm[s];
        cm[g.slotOffset + s] = (t >= 0) ? g.src[t] : 0.0;
    }
}

__global__ void sumRowsKernel(const double* rows, int nRows, long long N, double* out, long long outStride) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double s = 0.0;
    for (int r = 0; r < nRows; ++r) s += rows[(long long)r * N + i];
    out[i * outStride] = s;
}
}  // namespace mpgb

namespace mpgb {

// ---------------------------------------------------------------------------
// ParameterizedFunctionBase
// ---------------------------------------------------------------------------
ParameterizedFunctionBase::~ParameterizedFunctionBase() {
    if (owned_) cudaFree(owned_);
}

void ParameterizedFunctionBase::SetCoeffs(const double* coeffs, unsigned int n, bool host, cudaStream_t stream) {
    if (n != numCoeffs) {
        std::ostringstream os;
        os << "Error in ParameterizedFunctionBase<MemorySpace>::SetCoeffs.  Expected coefficient vector with size "
           << numCoeffs << ", but new coefficients have size " << n << ".";
        throw std::invalid_argument(os.str());
    }
    if (!coeffs_) {
        if (!owned_ && numCoeffs > 0) MPGB_CUDA(cudaMalloc(&owned_, numCoeffs * sizeof(double)));
        coeffs_ = owned_;
        coeffLabel_ = "ParameterizedFunctionBase<MemorySpace> Coefficients";
    }
    if (numCoeffs > 0) {
        if (host) {
            MPGB_CUDA(cudaMemcpyAsync(coeffs_, coeffs, n * sizeof(double), cudaMemcpyHostToDevice, stream));
            MPGB_CUDA(cudaStreamSynchronize(stream));
        } else {
            MPGB_CUDA(cudaMemcpyAsync(coeffs_, coeffs, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
        }
    }
    OnCoeffsChanged();
}

void ParameterizedFunctionBase::WrapCoeffsLabeled(double* deviceCoeffs, unsigned int n, std::string const& label) {
    if (n != numCoeffs) {
        std::ostringstream os;
        os << "Error in ParameterizedFunctionBase<MemorySpace>::WrapCoeffs.  Expected coefficient vector with size "
           << numCoeffs << ", but new coefficients have size " << n << ".";
        throw std::invalid_argument(os.str());
    }
    coeffs_ = deviceCoeffs;
    coeffLabel_ = label;
    OnCoeffsChanged();
}

void ParameterizedFunctionBase::CheckCoefficients(std::string const& functionName) const {
    if (!CheckCoefficients()) {
        std::ostringstream os;
        os << "Error in \"" << functionName
           << "\", the coefficients have not been set yet.  Make sure to call SetCoeffs() before calling this function.";
        throw std::runtime_error(os.str());
    }
}

std::vector<double> ParameterizedFunctionBase::CoeffMap() const {
    CheckCoefficients("CoeffMap");
    std::vector<double> h(numCoeffs);
    if (numCoeffs) MPGB_CUDA(cudaMemcpy(h.data(), coeffs_, numCoeffs * sizeof(double), cudaMemcpyDeviceToHost));
    return h;
}

// ---------------------------------------------------------------------------
// MonotoneMapBase
// ---------------------------------------------------------------------------
void ccRule(unsigned numPts, double* wts, double* pts) {
    // Clenshaw-Curtis points and weights on [-1,1] (Quadrature.h:212-258).
    if (numPts == 1) { pts[0] = 0.0; wts[0] = 2.0; return; }
    for (unsigned i = 0; i < numPts; ++i) pts[i] = std::cos((numPts - (i + 1)) * kPiHost / (numPts - 1));
    pts[0] = -1.0;
    if (numPts % 2 == 1) pts[(numPts - 1) / 2] = 0.0;
    pts[numPts - 1] = 1.0;
    for (unsigned i = 0; i < numPts; ++i) {
        wts[i] = 1.0;
        const double theta = i * kPiHost / (numPts - 1);
        for (unsigned j = 0; j < (numPts - 1) / 2; ++j) {
            const double b = (2 * (j + 1) == (numPts - 1)) ? 1.0 : 2.0;
            wts[i] = wts[i] - b * std::cos(2.0 * (j + 1) * theta) / (4 * (j + 1) * (j + 1) - 1);
        }
    }
    wts[0] = wts[0] / (numPts - 1.0);
    for (unsigned i = 1; i < numPts - 1; ++i) wts[i] = 2.0 * wts[i] / (numPts - 1.0);
    wts[numPts - 1] = wts[numPts - 1] / (numPts - 1.0);
}

static unsigned factorialU(unsigned d) {
    unsigned out = 1;
    for (unsigned i = 2; i <= d; ++i) out *= i;
    return out;
}

MapOptions mapOptionsFromC(const mpgb_map_options* o) {
    MapOptions m;
    if (!o) return m;
    if (o->basis_type < 0 || o->basis_type > 2) throw std::invalid_argument("invalid basis_type");
    if (o->pos_func_type < 0 || o->pos_func_type > 1) throw std::invalid_argument("invalid pos_func_type");
    if (o->quad_type < 0 || o->quad_type > 2) throw std::invalid_argument("invalid quad_type");
    m.basisType = (BasisTypes)o->basis_type;
    m.posFuncType = (PosFuncTypes)o->pos_func_type;
    m.quadType = (QuadTypes)o->quad_type;
    m.quadAbsTol = o->quad_abs_tol;
    m.quadRelTol = o->quad_rel_tol;
    m.quadMaxSub = o->quad_max_sub;
    m.quadMinSub = o->quad_min_sub;
    m.quadPts = o->quad_pts;
    m.contDeriv = o->cont_deriv != 0;
    m.basisNorm = o->basis_norm != 0;
    m.nugget = o->nugget;
    if (o->sigmoid_type != 0 || o->edge_type != 0 || o->sigmoid_sum_type < 0 || o->sigmoid_sum_type > 1)
        throw std::invalid_argument("invalid sigmoid enum value in options");
    m.sigmoidType = SigmoidTypes::Logistic;
    m.edgeType = EdgeTypes::SoftPlus;
    m.edgeShape = o->edge_shape;
    m.sigmoidBasisSumType = (SigmoidSumSizeType)o->sigmoid_sum_type;
    return m;
}

static void validateOptions(MapOptions const& o) {
    if (o.basisType == BasisTypes::PhysicistHermite)
        throw std::invalid_argument("MapOptions: basisType must be ProbabilistHermite or HermiteFunctions.");
    if (o.quadMaxSub < 1 || o.quadMaxSub > (unsigned)kMaxSubCap)
        throw std::invalid_argument("MapOptions: quadMaxSub must be in [1, 32].");
    if (o.quadMinSub >= o.quadMaxSub) throw std::invalid_argument("MapOptions: quadMinSub must be below quadMaxSub.");
    if (o.quadType == QuadTypes::AdaptiveClenshawCurtis && o.quadPts < 3)
        throw std::invalid_argument("MapOptions: quadPts must be at least 3.");
    if (o.quadType == QuadTypes::ClenshawCurtis && (o.quadPts < 1 || o.quadPts > (unsigned)kMaxRulePts))
        throw std::invalid_argument("MapOptions: ClenshawCurtis quadPts must be in [1, 33].");
    if (!(o.quadAbsTol >= 0) || !(o.quadRelTol >= 0)) throw std::invalid_argument("MapOptions: negative tolerance.");
    if (!(o.nugget >= 0)) throw std::invalid_argument("MapOptions: nugget must be non-negative.");
}

MonotoneMapBase::MonotoneMapBase(unsigned int inDim, unsigned int outDim, unsigned int nCoeffs, MapOptions const& opts)
    : ConditionalMapBase(inDim, outDim, nCoeffs), opts_(opts), ws_(new MapWorkspace()) {}

MonotoneMapBase::~MonotoneMapBase() = default;

// Builds the launch tables on first use.
// Quadrature rules and basis constants of a launch (both engines).
void buildLaunchConstants(const MapOptions& o, QuadParams& q, BasisConsts& b) {
    if (o.quadType == QuadTypes::AdaptiveClenshawCurtis) {
        // Quadrature rule: level = (unsigned) log2(quadPts - 2) (src/MapFactoryImpl4.cpp:18).
        const unsigned level = (unsigned)std::log2((double)(o.quadPts - 2));
        if (level < 1 || (int)level > kMaxQuadLevel)
            throw std::invalid_argument("MapOptions: quadPts gives an unsupported Clenshaw-Curtis level.");
        q.kind = kQuadACC;
        q.nCoarse = (1 << level) + 1;
        q.nFine = (1 << (level + 1)) + 1;
        ccRule(q.nCoarse, q.cWts, q.cPts);
        ccRule(q.nFine, q.fWts, q.fPts);
    } else if (o.quadType == QuadTypes::AdaptiveSimpson) {
        // Simpson on [-1, 1] and composite Simpson on its halves.
        q.kind = kQuadSimpson;
        q.nCoarse = 3;
        q.nFine = 5;
        const double cp[3] = {-1.0, 0.0, 1.0}, cw[3] = {1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0};
        const double fp[5] = {-1.0, -0.5, 0.0, 0.5, 1.0}, fw[5] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 6.0};
        for (int i = 0; i < 3; ++i) { q.cPts[i] = cp[i]; q.cWts[i] = cw[i]; }
        for (int i = 0; i < 5; ++i) { q.fPts[i] = fp[i]; q.fWts[i] = fw[i]; }
    } else {
        // ClenshawCurtis with quadPts points (ClenshawCurtisQuadrature::GetRule).
        if (o.quadPts < 1 || o.quadPts > (unsigned)kMaxRulePts)
            throw std::invalid_argument("MapOptions: ClenshawCurtis quadPts must be in [1, 33].");
        q.kind = kQuadFixedCC;
        q.nCoarse = 0;
        q.nFine = (int)o.quadPts;
        ccRule(q.nFine, q.fWts, q.fPts);
    }
    q.maxSub = (int)o.quadMaxSub;
    q.minSub = (int)o.quadMinSub;
    q.absTol = o.quadAbsTol;
    q.relTol = o.quadRelTol;
    q.maxIntervals = 1LL << 24;

    const bool norm = o.basisNorm;
    for (int k = 0; k <= kMaxLastOrder; ++k) {
        b.invNorm[k] = norm ? 1.0 / std::sqrt(std::sqrt(2.0 * kPiHost) * factorialU(k)) : 1.0;
        double fact = 1.0;
        for (int i = 2; i <= k; ++i) fact *= i;
        b.hfScale[k] = std::pow(kPiHost, -0.25) * std::pow(std::pow(2.0, k) * fact, -0.5);
    }
    for (int i = 0; i < kMaxLastOrder + 8; ++i) {
        b.hfR1[i] = std::sqrt(0.5 * (i - 1.0 > 0 ? i - 1.0 : 0.0));
        b.hfR2[i] = i > 0 ? 1.0 / std::sqrt(0.5 * i) : 0.0;
    }
    b.piQuarter = std::pow(kPiHost, -0.25);
    b.leadDR[0] = 0.0;
    b.leadDR[1] = b.invNorm[1];
    for (int k = 2; k <= kMaxLastOrder; ++k) b.leadDR[k] = k * b.invNorm[k] / b.invNorm[k - 1];
    for (int j = 0; j < kMaxLastOrder + 8; ++j) b.hfSq2j[j] = std::sqrt(2.0 * j);
    // phit_k(0).
    {
        double he[kMaxLastOrder + 1], H[kMaxLastOrder + 1];
        he[0] = 1.0; he[1] = 0.0;
        H[0] = 1.0; H[1] = 0.0;
        for (int k = 2; k <= kMaxLastOrder; ++k) {
            he[k] = -(k - 1.0) * he[k - 2];
            H[k] = -2.0 * (k - 1.0) * H[k - 2];
        }
        b.v0[0] = 1.0;
        for (int k = 1; k <= kMaxLastOrder; ++k) {
            if (o.basisType == BasisTypes::HermiteFunctions)
                b.v0[k] = (k == 1) ? 0.0 : b.hfScale[k - 2] * H[k - 2];
            else
                b.v0[k] = he[k] * b.invNorm[k];
        }
    }
}

void MonotoneMapBase::Prepare(cudaStream_t stream) {
    MapWorkspace& W = *ws_;
    if (!W.built) {
        int dev = 0;
        MPGB_CUDA(cudaGetDevice(&dev));
        MPGB_CUDA(cudaDeviceGetAttribute(&W.numSMs, cudaDevAttrMultiProcessorCount, dev));
        buildLaunchConstants(opts_, W.quad, W.bc);
        // Component descriptors.
        W.hostComps.clear();
        W.hostGather.clear();
        int slotOff = 0, pm = 1;
        W.dmax = 1; W.nBmax = 0; W.depthMax = 0;
        for (auto& pt : parts_) {
            const ComponentProgram& p = *pt.prog;
            CompDesc c{};
            c.D = p.D; c.P = p.P; c.nB = p.nB; c.nNodes = p.nNodes; c.nSlots = p.nSlots; c.nCNodes = p.nCNodes;
            c.maxDepth = p.maxDepth; c.numTerms = p.numTerms; c.outRow = (int)pt.outRow;
            c.coeffOffset = (int)pt.mapCoeffOffset; c.slotOffset = slotOff; c.cSegs = p.cSegs;
            c.nodeA = p.dNodeA; c.nodeSlot = p.dNodeSlot; c.nodeC = p.dNodeC; c.nodeCRows = p.dNodeCRows;
            c.slotTerm = p.dSlotTerm; c.leadDeg = p.dLeadDeg; c.rowOff = p.dRowOff;
            c.sigC = p.dSigC; c.sigW = p.dSigW; c.sigWt = p.dSigWt; c.sigStart = p.dSigStart;
            c.sigN = (int)p.sigC.size(); c.sigNStarts = (int)p.sigStart.size(); c.rectify = p.kind == 1 ? 1 : 0;
            c.nodeCIdx = p.dNodeCIdx;
            W.hostComps.push_back(c);
            slotOff += p.nSlots;
            pm = std::max(pm, p.P);
            W.dmax = std::max(W.dmax, p.D);
            W.nBmax = std::max(W.nBmax, p.nB);
            W.depthMax = std::max(W.depthMax, p.maxDepth);
            if (p.kind == 0 && p.nSlots + p.nNodes <= kStageCap) W.stageNeed = std::max(W.stageNeed, p.nSlots + p.nNodes);
        }
        MPGB_CUDA(cudaDeviceGetAttribute(&W.smemPerSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        W.totalSlots = slotOff;
        W.pmax = instantiatedPmax(pm);
        bool anySig = false, anyMono = false;
        for (auto& pt : parts_) (pt.prog->kind ? anySig : anyMono) = true;
        if (anySig && anyMono)
            throw std::invalid_argument(
                "TriangularMap: sigmoid expansions and monotone components cannot share one map on this path.");
        W.basis = anySig ? kBasisSigmoid
                         : (opts_.basisType == BasisTypes::HermiteFunctions ? kBasisHermiteFunctions : kBasisProbHermite);
        W.comps.ensure(W.hostComps.size() * sizeof(CompDesc), stream);
        MPGB_CUDA(cudaMemcpy(W.comps.p, W.hostComps.data(), W.hostComps.size() * sizeof(CompDesc),
                             cudaMemcpyHostToDevice));
        W.cm.ensure(std::max(1, W.totalSlots) * sizeof(double), stream);
        W.status.ensure(sizeof(int) * 4, stream);
        MPGB_CUDA(cudaMemset(W.status.p, 0, sizeof(int) * 4));
        W.built = true;
    }
    // Coefficient sources: each part reads its owner's current pointer.
    std::vector<GatherDescHost> g;
    int off = 0;
    for (auto& pt : parts_) {
        pt.owner->CheckCoefficients("MonotoneComponent");
        g.push_back({pt.owner->Coeffs() + pt.coeffOffset, pt.prog->dSlotTerm, off, pt.prog->nSlots});
        off += pt.prog->nSlots;
    }
    bool same = g.size() == W.hostGather.size();
    for (size_t i = 0; same && i < g.size(); ++i) same = g[i].src == W.hostGather[i].src;
    if (!same) {
        W.gather.ensure(g.size() * sizeof(GatherDescHost), stream);
        MPGB_CUDA(cudaMemcpyAsync(W.gather.p, g.data(), g.size() * sizeof(GatherDescHost), cudaMemcpyHostToDevice,
                                  stream));
        MPGB_CUDA(cudaStreamSynchronize(stream));
        W.hostGather = g;
    }
    int maxSlots = 1;
    for (auto& x : g) maxSlots = std::max(maxSlots, x.nSlots);
    dim3 grid((maxSlots + 255) / 256, (unsigned)g.size());
    gatherMultiKernel<<<grid, 256, 0, stream>>>(W.gather.as<GatherDescHost>(), (int)g.size(), W.cm.as<double>());
    MPGB_CUDA(cudaGetLastError());
    countLaunches(stream, 1);
}

void MonotoneMapBase::Finish(cudaStream_t stream, const char* fn) {
    if (async_) return;
    int st = CheckStatus(stream);
    if (st & kStatusInf) {
        std::ostringstream os;
        os << fn << ": MonotoneIntegrand: nan was encountered in value of g(df(...)).";
        throw IntegrandError(os.str());
    }
    if (st & kStatusBudget) {
        std::ostringstream os;
        os << fn << ": adaptive quadrature exceeded its interval budget.";
        throw std::runtime_error(os.str());
    }
}

void MonotoneMapBase::SetPointOrdering(bool on) { ws_->ordering = on; }

void MonotoneMapBase::ResetKLOrder() {
    for (auto& p : ws_->klPlans) p->permPts = nullptr;
}

double* MonotoneMapBase::StagingBuffer(int slot, size_t bytes, cudaStream_t stream) {
    if (slot < 0 || slot >= 8) throw std::invalid_argument("StagingBuffer: slot out of range.");
    ws_->stage[slot].ensure(bytes, stream);
    return ws_->stage[slot].as<double>();
}

int MonotoneMapBase::CheckStatus(cudaStream_t stream) {
    MapWorkspace& W = *ws_;
    if (!W.status.p) return 0;
    int st = 0;
    MPGB_CUDA(cudaMemcpyAsync(&st, W.status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    MPGB_CUDA(cudaStreamSynchronize(stream));
    MPGB_CUDA(cudaMemsetAsync(W.status.p, 0, sizeof(int), stream));
    return st;
}

namespace {

struct LaunchCommon {
    FusedParams prm{};
    int needJ = 0, needE = 0;
};

constexpr int kTpb = 128;
// Bracket-doubling steps per component in the inverse's first pass: roots
// within 7 of the initial guess are bracketed there, the rest wait for the
// second pass.
constexpr int kFirstPassBracketIts = 3;
// Inverse of monotone components: integrand nodes a point may take in the
// queue pass, and the width (intervals) of one of its quadratures, before the
// warp pass takes it over; the warp pass's grid
// (blocks of four warps per SM) and per-warp interval stack.
constexpr int kQueueNodeBudget = 16384;
// The width threshold balances the queue pass's tail (a few long serial
// solves, which dominate with few targets) against the warp pass's cost (a
// deferred point starts again, and narrow quadratures leave lanes idle),
// which weighs more with many: 48 intervals at 100k targets, growing as
// sqrt(N), at most 160 (measured on the 16-D inverse workload: ITP at 4M
// targets 11.9 s with 48, 9.4 s with 160; at 100k targets 0.52 s with 48,
// 0.79 s with 96).
inline int queueWideQuad(long long N) {
    const double w = 48.0 * std::sqrt((double)N / 1e5);
    return (int)std::min(160.0, std::max(48.0, w));
}
constexpr int kWarpPassBlocksPerSM = 2;
constexpr int kWarpStackCap = 512;

void checkMatrix(const StridedMatrix& m, int64_t rows, int64_t cols, const char* what, const char* fn) {
    if (m.rows != rows || m.cols != cols) {
        std::ostringstream os;
        os << fn << ": " << what << " has shape (" << m.rows << "," << m.cols << "), expected (" << rows << "," << cols
           << ").";
        throw std::invalid_argument(os.str());
    }
    if (rows > 0 && cols > 0 && m.data == nullptr) {
        std::ostringstream os;
        os << fn << ": " << what << " has no data.";
        throw std::invalid_argument(os.str());
    }
}

}  // namespace

// Fill the parameter fields common to every fused launch.
static void baseParams(MapWorkspace& W, const MapOptions& o, FusedParams& p, long long N) {
    p.comps = W.comps.as<CompDesc>();
    p.cm = W.cm.as<double>();
    p.N = N;
    p.tpb = kTpb;
    p.nugget = o.nugget;
    p.dmax = W.dmax;
    p.nBmax = W.nBmax;
    p.depthMax = W.depthMax;
    p.quad = W.quad;
    p.bc = W.bc;
    p.statusWord = W.status.as<int>();
}

static int posCode(const MapOptions& o) { return o.posFuncType == PosFuncTypes::Exp ? kPosExp : kPosSoftPlus; }

// Items of style "all components per tile" (per-point sums across components).
static std::vector<WorkItem> itemsAllComps(long long N, int nComps) {
    long long nTiles = (N + kTpb - 1) / kTpb;
    std::vector<WorkItem> v;
    v.reserve(nTiles);
    for (long long t = 0; t < nTiles; ++t) v.push_back({0, nComps, (int)t, 1, 0, 0, 1});
    return v;
}

// Items of style "one component, a set of tiles".  Heavier components first.
// With reduced outputs each component is cut into at most kFusedBlocksPerSM
// items per SM, independently of the other components of the launch, so a batched launch
// and per-component launches produce the same partial rows.  Item k of a
// component takes tiles k, k + nItems, k + 2 nItems, ...: points are processed
// in order of |x_D| (quadrature cost grows with it), and striding gives every
// item the same mix of cheap and expensive tiles.
static std::vector<WorkItem> itemsPerComp(const std::vector<MonotoneMapBase::Part>& parts, long long N, int numSMs,
                                          bool reduced, std::vector<long long>* rowBaseOut,
                                          std::vector<std::vector<int>>* itemsOfComp, int onlyComp = -1,
                                          long long* rcTotal = nullptr) {
    const int nComps = (int)parts.size();
    const long long nTiles = (N + kTpb - 1) / kTpb;
    std::vector<int> order;
    for (int c = 0; c < nComps; ++c)
        if (onlyComp < 0 || c == onlyComp) order.push_back(c);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return parts[a].prog->weight > parts[b].prog->weight; });
    std::vector<WorkItem> v;
    long long base = 0;
    if (itemsOfComp) itemsOfComp->assign(nComps, {});
    for (int c : order) {
        const long long nItemsC =
            reduced ? std::max<long long>(1, std::min<long long>(nTiles, (long long)numSMs * kFusedBlocksPerSM))
                    : nTiles;
        for (long long t = 0; t < nItemsC; ++t) {
            WorkItem w{c, c + 1, (int)t, (int)((nTiles - t + nItemsC - 1) / nItemsC), 0, 0, (int)nItemsC, 0};
            if (reduced) {
                w.partialBase = base;
                w.lossSlot = (int)v.size();
                if (rcTotal) {
                    w.rcBase = *rcTotal;
                    *rcTotal += (long long)parts[c].prog->nCNodes * kTpb;
                }
                for (int sg = 0; sg < parts[c].prog->cSegs; ++sg) {
                    if (rowBaseOut) rowBaseOut->push_back(base);
                    base += parts[c].prog->numTerms;
                }
            }
            if (itemsOfComp) (*itemsOfComp)[c].push_back((int)v.size());
            v.push_back(w);
        }
    }
    return v;
}

// The node cache of a reduced launch (rcTotal doubles, from itemsPerComp):
// phase A keeps per tile the rectified products of a sigmoid expansion, or
// the deeper prefix products of a monotone component, for the reduction.
// Above 2 GiB the reduction forms them again.
static double* rectCache(MapWorkspace& W, long long rcTotal, cudaStream_t stream) {
    if (rcTotal <= 0 || rcTotal > (2LL << 30) / (long long)sizeof(double)) return nullptr;
    W.rcache.ensure((size_t)rcTotal * sizeof(double), stream);
    return W.rcache.as<double>();
}

static void uploadItems(MapWorkspace& W, const std::vector<WorkItem>& items, cudaStream_t stream) {
    W.items.ensure(items.size() * sizeof(WorkItem), stream);
    MPGB_CUDA(cudaMemcpyAsync(W.items.p, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice,
                              stream));
}

// Processing order for per-component launches: each component's points
// sorted (stably) by |x_D| of its own last coordinate.
static void orderPoints(MapWorkspace& W, const std::vector<MonotoneMapBase::Part>& parts, StridedMatrix const& pts,
                        FusedParams& p, int onlyComp, cudaStream_t stream) {
    p.perm = nullptr;
    p.permStride = 0;
    const long long N = pts.cols;
    // (Sigmoid expansions have no quadrature: every point costs the same.)
    if (!W.ordering || N < 2 * kTpb || W.basis == kBasisSigmoid) return;
    const size_t nComps = parts.size();
    W.perm.ensure(nComps * (size_t)N * sizeof(int), stream);
    W.sortHist.ensure(sortScratchInts(N) * sizeof(int), stream);
    for (size_t c = 0; c < nComps; ++c) {
        if (onlyComp >= 0 && (int)c != onlyComp) continue;
        const double* xd = pts.data + (int64_t)(parts[c].prog->D - 1) * pts.rowStride;
        MPGB_CUDA(launchSortByLast(xd, pts.colStride, N, W.sortHist.as<int>(), W.perm.as<int>() + c * (size_t)N,
                                   stream));
    }
    p.perm = W.perm.as<int>();
    p.permStride = N;
}

// Phase A's inputs are staged in shared memory (FusedParams::stageDoubles)
// when the staging does not lower the number of blocks an SM holds.
static int stageDoubles(const MapWorkspace& W, const FusedParams& p, bool input) {
    if (W.stageNeed == 0 || W.smemPerSM <= 0) return 0;
    const size_t base = fusedSmemBytes(p.tpb, p.dmax, p.nBmax, p.depthMax, W.pmax, input) + 1024;
    const size_t with = base + (size_t)W.stageNeed * sizeof(double);
    auto blocks = [&](size_t b) { return std::min<size_t>(kFusedBlocksPerSM, (size_t)W.smemPerSM / b); };
    return (with <= 227 * 1024 && blocks(with) == blocks(base)) ? W.stageNeed : 0;
}

static void launch(MapWorkspace& W, const MapOptions& o, FusedParams& p, int nItems, int needJ, int needE,
                   cudaStream_t stream) {
    p.items = W.items.as<WorkItem>();
    if (nItems == 0) return;
    const size_t smem = fusedSmemBytes(p.tpb, p.dmax, p.nBmax, p.depthMax, W.pmax, (p.flags & kFlagInput) != 0);
    if (smem > 227 * 1024) throw std::invalid_argument("Component too large for the shared-memory tile.");
    p.stageDoubles = stageDoubles(W, p, (p.flags & kFlagInput) != 0);
    // contDeriv = false: log-determinants and their coefficient adjoints come
    // from the quadrature's x_D-derivative (the kernel variant NEEDE = 2).
    if (!o.contDeriv && ((p.flags & (kFlagLogDet | kFlagCoefDenseL | kFlagKL)) ||
                         ((p.flags & kFlagCoefReduced) && (p.lsens || p.lsensScale != 0.0)))) {
        needJ = 1;
        needE = 2;
    }
    MPGB_CUDA(launchFused(W.basis, posCode(o), W.pmax, p, nItems, needJ, needE, stream));
}

// The quadrature dimension each reference operation leaves on its components
// (ComponentProgram::quadDim): 1 after Evaluate and Inverse, 2 after the
// discrete-derivative LogDeterminant and LogDeterminantCoeffGrad, inputs + 1
// after Gradient, terms + 1 after CoeffGrad; the continuous-derivative
// operations integrate nothing and leave it.
enum class QuadDimRule { One, Two, InputsPlusOne, TermsPlusOne };

static void noteQuadDim(std::vector<MonotoneMapBase::Part> const& parts, QuadDimRule rule) {
    for (auto& pt : parts) {
        ComponentProgram& g = *pt.prog;
        g.quadDim = rule == QuadDimRule::One ? 1u
                    : rule == QuadDimRule::Two ? 2u
                    : rule == QuadDimRule::InputsPlusOne ? (unsigned)g.D + 1u
                                                         : (unsigned)g.numTerms + 1u;
    }
}

void MonotoneMapBase::EvaluateImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream) {
    CheckCoefficients("Evaluate");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "EvaluateImpl");
    checkMatrix(output, outputDim, N, "output", "EvaluateImpl");
    noteQuadDim(parts_, QuadDimRule::One);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsPerComp(parts_, N, W.numSMs, false, nullptr, nullptr);
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    // The reference's EvaluateImpl calls EvaluateSingle without the nugget
    // (MonotoneComponent.h:290): T integrates g(df) alone, whereas CoeffGrad,
    // Gradient and Inverse integrate g(df) + nugget (:434, :721, :794).
    p.nugget = 0.0;
    p.flags = kFlagEval;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.outEval = output.data; p.evalRs = output.rowStride; p.evalCs = output.colStride;
    orderPoints(W, parts_, pts, p, -1, stream);
    launch(W, opts_, p, (int)items.size(), 0, 0, stream);
    Finish(stream, "Evaluate");
}

void MonotoneMapBase::LogDeterminantImpl(StridedMatrix const& pts, StridedMatrix const& output, cudaStream_t stream) {
    CheckCoefficients("LogDeterminant");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "LogDeterminantImpl");
    if (output.rows * output.cols != N) throw std::invalid_argument("LogDeterminantImpl: output must hold N values.");
    if (!opts_.contDeriv) noteQuadDim(parts_, QuadDimRule::Two);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsAllComps(N, (int)parts_.size());
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagLogDet;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.outLogDet = output.data;
    p.logDetStride = (output.rows == 1) ? output.colStride : output.rowStride;
    launch(W, opts_, p, (int)items.size(), 0, 0, stream);
    Finish(stream, "LogDeterminant");
}

void MonotoneMapBase::CoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                                    cudaStream_t stream) {
    CheckCoefficients("CoeffGrad");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "CoeffGradImpl");
    checkMatrix(sens, outputDim, N, "sens", "CoeffGradImpl");
    checkMatrix(output, numCoeffs, N, "output", "CoeffGradImpl");
    noteQuadDim(parts_, QuadDimRule::TermsPlusOne);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsPerComp(parts_, N, W.numSMs, false, nullptr, nullptr);
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagCoefDenseT;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.sens = sens.data; p.sensRs = sens.rowStride; p.sensCs = sens.colStride;
    p.outDense = output.data; p.denseRs = output.rowStride; p.denseCs = output.colStride;
    orderPoints(W, parts_, pts, p, -1, stream);
    launch(W, opts_, p, (int)items.size(), 1, 0, stream);
    Finish(stream, "CoeffGrad");
}

void MonotoneMapBase::LogDeterminantCoeffGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                                  cudaStream_t stream) {
    CheckCoefficients("LogDeterminantCoeffGrad");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "LogDeterminantCoeffGradImpl");
    checkMatrix(output, numCoeffs, N, "output", "LogDeterminantCoeffGradImpl");
    if (!opts_.contDeriv) noteQuadDim(parts_, QuadDimRule::Two);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsPerComp(parts_, N, W.numSMs, false, nullptr, nullptr);
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagCoefDenseL;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.outDense = output.data; p.denseRs = output.rowStride; p.denseCs = output.colStride;
    launch(W, opts_, p, (int)items.size(), 0, 0, stream);
    Finish(stream, "LogDeterminantCoeffGrad");
}

void MonotoneMapBase::GradientImpl(StridedMatrix const& pts, StridedMatrix const& sens, StridedMatrix const& output,
                                   cudaStream_t stream) {
    CheckCoefficients("Gradient");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "GradientImpl");
    checkMatrix(sens, outputDim, N, "sens", "GradientImpl");
    checkMatrix(output, inputDim, N, "output", "GradientImpl");
    noteQuadDim(parts_, QuadDimRule::InputsPlusOne);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsAllComps(N, (int)parts_.size());
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagInput;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.sens = sens.data; p.sensRs = sens.rowStride; p.sensCs = sens.colStride;
    p.lsens = nullptr; p.lsensScale = 0.0;
    p.outInput = output.data; p.inputRs = output.rowStride; p.inputCs = output.colStride;
    launch(W, opts_, p, (int)items.size(), 1, 1, stream);
    Finish(stream, "Gradient");
}

void MonotoneMapBase::LogDeterminantInputGradImpl(StridedMatrix const& pts, StridedMatrix const& output,
                                                  cudaStream_t stream) {
    CheckCoefficients("LogDeterminantInputGrad");
    // MonotoneComponent.h:216-222 throws the same for contDeriv = false.
    if (!opts_.contDeriv) throw std::invalid_argument("Discrete derivative version is not implemented yet (To Do)");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "LogDeterminantInputGradImpl");
    checkMatrix(output, inputDim, N, "output", "LogDeterminantInputGradImpl");
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    auto items = itemsAllComps(N, (int)parts_.size());
    uploadItems(W, items, stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagInput;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.sens = nullptr;
    p.lsens = nullptr; p.lsensScale = 1.0;
    p.outInput = output.data; p.inputRs = output.rowStride; p.inputCs = output.colStride;
    launch(W, opts_, p, (int)items.size(), 0, 0, stream);
    Finish(stream, "LogDeterminantInputGrad");
}

void MonotoneMapBase::InverseImpl(StridedMatrix const& x1, StridedMatrix const& r, StridedMatrix const& output,
                                  cudaStream_t stream) {
    InverseImpl(x1, r, output, InverseOptions(), nullptr, stream);
}

void MonotoneMapBase::InverseImpl(StridedMatrix const& x1, StridedMatrix const& r, StridedMatrix const& output,
                                  InverseOptions const& io, int* deviceInfo, cudaStream_t stream) {
    CheckCoefficients("Inverse");
    if (io.xtol < 0 || io.ytol < 0) throw std::invalid_argument("Invalid tolerance given to MonotoneComponent::Inverse.");
    if (io.xtol <= std::numeric_limits<double>::epsilon() && io.ytol <= std::numeric_limits<double>::epsilon())
        throw std::invalid_argument(
            "Invalid tolerances given to MonotoneComponent::Inverse.  Either \"xtol\" or \"ytol\" must be nonzero.");
    if (io.method != kInverseITP && io.method != kInverseNewton)
        throw std::invalid_argument(
            "Invalid method given to MonotoneComponent::Inverse.  Valid options are 0 (\"Bracket\") and 1 (Newton).");
    const long long N = r.cols;
    if (r.rows != outputDim) throw std::invalid_argument("InverseImpl: r must have outputDim rows.");
    if (x1.cols != N && x1.cols != 1) {
        std::ostringstream os;
        os << "x1 and r have different numbers of columns.  x1.extent(1)=" << x1.cols << ", but r.extent(1)=" << N;
        throw std::invalid_argument(os.str());
    }
    if (x1.rows > inputDim) throw std::invalid_argument("InverseImpl: x1 has too many rows.");
    checkMatrix(output, outputDim, N, "output", "InverseImpl");
    noteQuadDim(parts_, QuadDimRule::One);
    if (N == 0) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    InverseParams p{};
    p.comps = W.comps.as<CompDesc>();
    p.nComps = (int)parts_.size();
    p.cm = W.cm.as<double>();
    p.N = N;
    p.tpb = kTpb;
    p.extra = (int)(inputDim - outputDim);
    p.x1 = x1.data; p.x1Rs = x1.rowStride; p.x1Cs = x1.colStride; p.x1Rows = (int)x1.rows; p.x1Cols = (int)x1.cols;
    p.r = r.data; p.rRs = r.rowStride; p.rCs = r.colStride;
    p.out = output.data; p.outRs = output.rowStride; p.outCs = output.colStride;
    p.info = deviceInfo; p.infoStride = N;
    p.statusWord = W.status.as<int>();
    p.xtol = io.xtol; p.ytol = io.ytol;
    p.method = io.method;
    p.nugget = opts_.nugget;
    p.dmax = W.dmax; p.nBmax = W.nBmax; p.depthMax = W.depthMax;
    p.quad = W.quad; p.bc = W.bc;
    const int nBlocks = (int)((N + kTpb - 1) / kTpb);
    if (N < 2 * kTpb) {
        // Few points: one launch solves every component in turn.
        p.bracketBudget = (int)kBracketIts;
        MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, p, nBlocks, stream));
        Finish(stream, "Inverse");
        return;
    }
    W.inverseDefer.ensure(4 * sizeof(int), stream);
    W.inverseKey.ensure((size_t)N * sizeof(double), stream);
    W.perm.ensure((size_t)N * sizeof(int), stream);
    W.sortHist.ensure(sortScratchInts(N) * sizeof(int), stream);
    int* deferCount = W.inverseDefer.as<int>();
    double* key = W.inverseKey.as<double>();
    int* perm = W.perm.as<int>();
    if (W.basis != kBasisSigmoid) {
        // Monotone components, one at a time: a key launch forms phase A of
        // every point (kept in inverseA for the solver) and a root estimate;
        // the points are sorted by |estimate| (the cost of a solver step grows
        // with the range [0, x] its quadrature covers); a persistent queue
        // launch solves them, expensive ones first, one integrand node per
        // lane and loop iteration (inverseQueueKernel).
        W.inverseA.ensure((size_t)(W.pmax + 1) * N * sizeof(double), stream);
        W.inverseList.ensure((size_t)N * sizeof(int), stream);
        const int warpBlocks = kWarpPassBlocksPerSM * W.numSMs;
        W.inverseStack.ensure((size_t)warpBlocks * (128 / kWarpGroup) * kWarpStackCap * sizeof(QEntry), stream);
        // Saved solver states for up to a quarter of the points (deferred
        // points beyond it start their solves again).
        const int stateCap = (int)std::min<long long>(N, N / 4 + 1024);
        W.inverseState.ensure((size_t)stateCap * kSolveStateDoubles * sizeof(double), stream);
        int* counters = W.inverseDefer.as<int>();  // [queue pass, deferred count, warp pass, queue drained]
        for (int c = 0; c < p.nComps; ++c) {
            InverseParams k = p;
            k.compBegin = c;
            k.compEnd = c + 1;
            k.keyPass = 1;
            k.acoef = W.inverseA.as<double>();
            k.key = key;
            MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, k, nBlocks, stream));
            InverseParams q = p;
            q.compBegin = c;
            q.compEnd = c + 1;
            q.acoef = k.acoef;
            q.bracketBudget = (int)kBracketIts;
            if (W.ordering) {
                MPGB_CUDA(launchSortByLast(key, 1, N, W.sortHist.as<int>(), perm, stream));
                q.perm = perm;
            }
            MPGB_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(int), stream));
            q.queue = counters;
            q.queuePass = 1;
            q.nodeBudget = kQueueNodeBudget;
            q.wideQuad = queueWideQuad(N);
            q.deferList = W.inverseList.as<int>();
            q.deferCount = counters + 1;
            q.drained = counters + 3;
            q.deferState = W.inverseState.as<double>();
            q.deferStateCap = stateCap;
            MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, q, nBlocks, stream));
            // The deferred points, kWarpGroup lanes each.
            InverseParams wp = q;
            wp.queuePass = 0;
            wp.nodeBudget = 0;
            wp.warpPass = 1;
            wp.queue = counters + 2;
            wp.listCount = counters + 1;
            wp.stack = W.inverseStack.as<QEntry>();
            wp.stackCap = kWarpStackCap;
            MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, wp, warpBlocks, stream));
        }
        Finish(stream, "Inverse");
        return;
    }
    // Sigmoid expansions, one component at a time, in two passes (see
    // InverseParams): the first gives every point kFirstPassBracketIts
    // bracket-doubling steps, the second finishes the points that needed
    // more, sorted by the root estimate the first pass leaves for them.
    for (int c = 0; c < p.nComps; ++c) {
        InverseParams first = p;
        first.compBegin = c;
        first.compEnd = c + 1;
        first.bracketBudget = kFirstPassBracketIts;
        MPGB_CUDA(cudaMemsetAsync(key, 0xff, (size_t)N * sizeof(double), stream));  // NaN: not deferred
        MPGB_CUDA(cudaMemsetAsync(deferCount, 0, sizeof(int), stream));
        first.deferKey = key;
        first.deferCount = deferCount;
        MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, first, nBlocks, stream));
        MPGB_CUDA(launchSortByLast(key, 1, N, W.sortHist.as<int>(), perm, stream));
        InverseParams second = first;
        second.perm = perm;
        second.listCount = deferCount;
        second.bracketBudget = (int)kBracketIts;
        second.deferKey = nullptr;
        second.deferCount = nullptr;
        // One warp per block: the second pass often has few points, whose
        // warps then spread over the SMs instead of sharing a few of them.
        second.tpb = 32;
        MPGB_CUDA(launchInverse(W.basis, posCode(opts_), W.pmax, second, (int)((N + 31) / 32), stream));
    }
    Finish(stream, "Inverse");
}

void MonotoneMapBase::FusedForwardAdjoint(StridedMatrix const& pts, StridedMatrix const& sens,
                                          StridedMatrix const& logdetSens, double logdetSensScale,
                                          StridedMatrix const& outEval, StridedMatrix const& outLogDet,
                                          double* coeffGrad, StridedMatrix const& inputGrad, cudaStream_t stream) {
    CheckCoefficients("FusedForwardAdjoint");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "FusedForwardAdjoint");
    if (!sens.empty()) checkMatrix(sens, outputDim, N, "sens", "FusedForwardAdjoint");
    if (!logdetSens.empty() && logdetSens.rows * logdetSens.cols != N)
        throw std::invalid_argument("FusedForwardAdjoint: logdet_sens must hold N values.");
    if (!outEval.empty()) checkMatrix(outEval, outputDim, N, "out_eval", "FusedForwardAdjoint");
    if (!outLogDet.empty() && outLogDet.rows * outLogDet.cols != N)
        throw std::invalid_argument("FusedForwardAdjoint: out_logdet must hold N values.");
    if (!inputGrad.empty()) checkMatrix(inputGrad, inputDim, N, "input_grad", "FusedForwardAdjoint");
    // Parts of the call whose integrand carries the nugget (CoeffGrad,
    // Gradient, the discrete log-determinant, MonotoneComponent.h:622-965).
    const bool nuggetParts = coeffGrad || !inputGrad.empty() || (!outLogDet.empty() && !opts_.contDeriv);
    if (opts_.nugget != 0.0 && !outEval.empty() && nuggetParts) {
        // The values are those of Evaluate, which integrates without the
        // nugget, and the adjoints those of CoeffGrad / Gradient, which
        // integrate with it (different quadrature trees): two passes.
        FusedForwardAdjoint(pts, sens, logdetSens, logdetSensScale, StridedMatrix(), outLogDet, coeffGrad, inputGrad,
                            stream);
        EvaluateImpl(pts, outEval, stream);
        return;
    }
    Prepare(stream);
    MapWorkspace& W = *ws_;
    const int nComps = (int)parts_.size();
    const long long ldStrideL = logdetSens.empty() ? 0 : ((logdetSens.rows == 1) ? logdetSens.colStride : logdetSens.rowStride);
    if (N == 0) {
        if (coeffGrad) MPGB_CUDA(cudaMemsetAsync(coeffGrad, 0, numCoeffs * sizeof(double), stream));
        Finish(stream, "FusedForwardAdjoint");
        return;
    }
    // Pass 1: per-component outputs and the reduced coefficient adjoint.
    const bool wantCoef = coeffGrad != nullptr;
    const bool wantLogDet = !outLogDet.empty();
    if (wantCoef || !outEval.empty() || wantLogDet) {
        std::vector<long long> rowBase;
        std::vector<std::vector<int>> itemsOf;
        long long rcTotal = 0;
        auto items = itemsPerComp(parts_, N, W.numSMs, wantCoef, &rowBase, &itemsOf, -1, &rcTotal);
        uploadItems(W, items, stream);
        FusedParams p{};
        baseParams(W, opts_, p, N);
        p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
        p.flags = 0;
        if (wantCoef) p.rcache = rectCache(W, rcTotal, stream);
        orderPoints(W, parts_, pts, p, -1, stream);
        if (!outEval.empty()) {
            p.flags |= kFlagEval;
            p.outEval = outEval.data; p.evalRs = outEval.rowStride; p.evalCs = outEval.colStride;
            p.nugget = 0.0;  // (nothing else in this pass integrates with the nugget)
        }
        if (wantLogDet) {
            // Per-component log-dets into scratch rows, summed in component order below.
            W.logdetRows.ensure((size_t)nComps * N * sizeof(double), stream);
            p.flags |= kFlagLogDet;
            p.outLogDet = W.logdetRows.as<double>();
            p.logDetStride = 1;
        }
        int needJ = 0;
        if (wantCoef) {
            p.flags |= kFlagCoefReduced;
            p.sens = sens.data; p.sensRs = sens.rowStride; p.sensCs = sens.colStride;
            p.lsens = logdetSens.data; p.lsensStride = ldStrideL; p.lsensScale = logdetSensScale;
            size_t nPart = rowBase.empty() ? 1 : (size_t)(rowBase.back() + parts_[items.back().c0].prog->numTerms);
            size_t tot = 0;
            for (auto& it : items)
                tot = std::max<size_t>(tot, (size_t)it.partialBase +
                                                (size_t)parts_[it.c0].prog->numTerms * parts_[it.c0].prog->cSegs);
            nPart = std::max(nPart, tot);
            W.partials.ensure(nPart * sizeof(double), stream);
            p.partials = W.partials.as<double>();
            needJ = sens.empty() ? 0 : 1;
        }
        if (wantLogDet) {
            // One component per item: each writes its component's row of the
            // scratch, summed in component order below.
            p.logDetCompStride = N;
            launch(W, opts_, p, (int)items.size(), needJ, 0, stream);
            sumRowsKernel<<<(unsigned)((N + 255) / 256), 256, 0, stream>>>(
                W.logdetRows.as<double>(), nComps, N, outLogDet.data,
                (outLogDet.rows == 1) ? outLogDet.colStride : outLogDet.rowStride);
            MPGB_CUDA(cudaGetLastError());
            countLaunches(stream, 1);
        } else {
            launch(W, opts_, p, (int)items.size(), needJ, 0, stream);
        }
        if (wantCoef) {
            // Fixed-order reduction of each component's partial rows.
            std::vector<long long> rb;
            W.rowBase.ensure(sizeof(long long) * std::max<size_t>(1, rowBase.size()), stream);
            for (int c = 0; c < nComps; ++c) {
                for (int id : itemsOf[c])
                    for (int sg = 0; sg < parts_[c].prog->cSegs; ++sg)
                        rb.push_back(items[id].partialBase + (long long)sg * parts_[c].prog->numTerms);
            }
            MPGB_CUDA(cudaMemcpyAsync(W.rowBase.p, rb.data(), rb.size() * sizeof(long long), cudaMemcpyHostToDevice,
                                      stream));
            // Every component's rows in one launch.
            std::vector<KLReduceDesc> rd(nComps);
            int off = 0, maxTerms = 0;
            for (int c = 0; c < nComps; ++c) {
                KLReduceDesc& q = rd[c];
                q = KLReduceDesc{};
                q.rowOff = off;
                q.nRows = (int)itemsOf[c].size() * parts_[c].prog->cSegs;
                q.nTerms = parts_[c].prog->numTerms;
                q.outOff = (int)parts_[c].mapCoeffOffset;
                q.comp = c;
                off += q.nRows;
                maxTerms = std::max(maxTerms, q.nTerms);
            }
            W.reduceDesc.ensure(rd.size() * sizeof(KLReduceDesc), stream);
            MPGB_CUDA(cudaMemcpyAsync(W.reduceDesc.p, rd.data(), rd.size() * sizeof(KLReduceDesc),
                                      cudaMemcpyHostToDevice, stream));
            MPGB_CUDA(launchKLReduce(W.partials.as<double>(), W.rowBase.as<long long>(),
                                     W.reduceDesc.as<KLReduceDesc>(), nComps, maxTerms, coeffGrad, nullptr, nullptr,
                                     1.0, nullptr, stream));
        }
    }
    // Pass 2: input gradient (sums over components per point).
    if (!inputGrad.empty()) {
        if (!opts_.contDeriv && (logdetSens.data || logdetSensScale != 0.0))
            throw std::invalid_argument("Discrete derivative version is not implemented yet (To Do)");
        auto items = itemsAllComps(N, nComps);
        uploadItems(W, items, stream);
        FusedParams p{};
        baseParams(W, opts_, p, N);
        p.flags = kFlagInput;
        p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
        p.sens = sens.data; p.sensRs = sens.rowStride; p.sensCs = sens.colStride;
        p.lsens = logdetSens.data; p.lsensStride = ldStrideL; p.lsensScale = logdetSensScale;
        p.outInput = inputGrad.data; p.inputRs = inputGrad.rowStride; p.inputCs = inputGrad.colStride;
        const int nj = sens.empty() ? 0 : 1;
        launch(W, opts_, p, (int)items.size(), nj, nj, stream);
    }
    Finish(stream, "FusedForwardAdjoint");
}

static KLPlan& klPlan(MapWorkspace& W, const std::vector<MonotoneMapBase::Part>& parts, long long N, int onlyComp,
                      cudaStream_t stream) {
    static thread_local int dummy = 0;
    (void)dummy;
    for (auto& p : W.klPlans)
        if (p->N == N && p->onlyComp == onlyComp) return *p;
    W.klPlans.emplace_back(new KLPlan());
    KLPlan& P = *W.klPlans.back();
    P.N = N;
    P.onlyComp = onlyComp;
    std::vector<long long> rowBase;
    auto items = itemsPerComp(parts, N, W.numSMs, true, &rowBase, &P.itemsOf, onlyComp, &P.rcTotal);
    P.nItems = (int)items.size();
    for (auto& it : items)
        P.partialDoubles = std::max<size_t>(P.partialDoubles, (size_t)it.partialBase + (size_t)parts[it.c0].prog->numTerms *
                                                                                      parts[it.c0].prog->cSegs);
    std::vector<long long> rb;
    std::vector<int> ls;
    P.rowOff.assign(parts.size() + 1, 0);
    P.lossOff.assign(parts.size() + 1, 0);
    for (size_t c = 0; c < parts.size(); ++c) {
        P.rowOff[c] = (int)rb.size();
        P.lossOff[c] = (int)ls.size();
        for (int id : P.itemsOf[c]) {
            for (int sg = 0; sg < parts[c].prog->cSegs; ++sg)
                rb.push_back(items[id].partialBase + (long long)sg * parts[c].prog->numTerms);
            ls.push_back(items[id].lossSlot);
        }
    }
    P.rowOff[parts.size()] = (int)rb.size();
    P.lossOff[parts.size()] = (int)ls.size();
    P.items.ensure(items.size() * sizeof(WorkItem), stream);
    P.rowBase.ensure(std::max<size_t>(1, rb.size()) * sizeof(long long), stream);
    P.lossSlots.ensure(std::max<size_t>(1, ls.size()) * sizeof(int), stream);
    MPGB_CUDA(cudaMemcpy(P.items.p, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    if (!rb.empty()) {
        MPGB_CUDA(cudaMemcpy(P.rowBase.p, rb.data(), rb.size() * sizeof(long long), cudaMemcpyHostToDevice));
        MPGB_CUDA(cudaMemcpy(P.lossSlots.p, ls.data(), ls.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    std::vector<KLReduceDesc> rd;
    for (size_t c = 0; c < parts.size(); ++c) {
        if (onlyComp >= 0 && (int)c != onlyComp) continue;
        KLReduceDesc q{};
        q.rowOff = P.rowOff[c];
        q.nRows = P.rowOff[c + 1] - P.rowOff[c];
        q.nTerms = parts[c].prog->numTerms;
        q.outOff = (int)parts[c].mapCoeffOffset;
        q.lossOff = P.lossOff[c];
        q.nLoss = P.lossOff[c + 1] - P.lossOff[c];
        q.comp = (int)c;
        rd.push_back(q);
        P.maxTerms = std::max(P.maxTerms, q.nTerms);
    }
    P.nReduce = (int)rd.size();
    P.reduceDesc.ensure(std::max<size_t>(1, rd.size()) * sizeof(KLReduceDesc), stream);
    if (!rd.empty())
        MPGB_CUDA(cudaMemcpy(P.reduceDesc.p, rd.data(), rd.size() * sizeof(KLReduceDesc), cudaMemcpyHostToDevice));
    return P;
}

// The KL step's processing order, kept in the plan (see KLPlan::perm).  An
// order computed inside a stream capture is not kept: its sort has not run.
static void orderPointsKL(MapWorkspace& W, KLPlan& P, const std::vector<MonotoneMapBase::Part>& parts,
                          StridedMatrix const& pts, FusedParams& p, int onlyComp, cudaStream_t stream) {
    p.perm = nullptr;
    p.permStride = 0;
    const long long N = pts.cols;
    if (!W.ordering || N < 2 * kTpb || W.basis == kBasisSigmoid) return;
    if (P.permPts != pts.data || P.permRs != pts.rowStride || P.permCs != pts.colStride) {
        const size_t nComps = parts.size();
        P.perm.ensure(nComps * (size_t)N * sizeof(int), stream);
        // room for the step's all-component cost-order sort as well, which
        // runs inside graph capture and so cannot allocate
        W.sortHist.ensure(nComps * sortScratchInts(N) * sizeof(int), stream);
        for (size_t c = 0; c < nComps; ++c) {
            if (onlyComp >= 0 && (int)c != onlyComp) continue;
            const double* xd = pts.data + (int64_t)(parts[c].prog->D - 1) * pts.rowStride;
            MPGB_CUDA(launchSortByLast(xd, pts.colStride, N, W.sortHist.as<int>(), P.perm.as<int>() + c * (size_t)N,
                                       stream));
        }
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        MPGB_CUDA(cudaStreamIsCapturing(stream, &cs));
        if (cs == cudaStreamCaptureStatusNone) {
            P.permPts = pts.data;
            P.permRs = pts.rowStride;
            P.permCs = pts.colStride;
        } else {
            P.permPts = nullptr;
        }
    }
    p.perm = P.perm.as<int>();
    p.permStride = N;
}

void MonotoneMapBase::KLObjective(StridedMatrix const& pts, double* lossPerComp, double* grad, cudaStream_t stream) {
    KLObjective(pts, lossPerComp, grad, -1, stream);
}

void MonotoneMapBase::KLObjective(StridedMatrix const& pts, double* lossPerComp, double* grad, int onlyComp,
                                  cudaStream_t stream) {
    CheckCoefficients("KLObjective");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "KLObjective");
    if (N == 0) throw std::invalid_argument("KLObjective: no samples.");
    if (onlyComp >= (int)parts_.size()) throw std::out_of_range("KLObjective: component index out of range.");
    Prepare(stream);
    MapWorkspace& W = *ws_;
    if (opts_.nugget != 0.0) {
        size_t maxTerms = 1;
        for (auto& pt : parts_) maxTerms = std::max<size_t>(maxTerms, pt.prog->numTerms);
        W.klT.ensure((size_t)N * sizeof(double), stream);
        W.klLd.ensure((size_t)N * sizeof(double), stream);
        W.klDT.ensure(maxTerms * N * sizeof(double), stream);
        W.klDL.ensure(maxTerms * N * sizeof(double), stream);
        KLObjectiveCalls(pts, lossPerComp, grad, onlyComp, W.klT.as<double>(), W.klLd.as<double>(),
                         W.klDT.as<double>(), W.klDL.as<double>(), stream);
        if (async_) return;
        // (the calls went to the components, whose status words hold the flags)
        int st = 0;
        for (auto& pt : parts_)
            if (auto* c = dynamic_cast<MonotoneMapBase*>(pt.owner)) st |= c->CheckStatus(stream);
        if (st & kStatusInf)
            throw IntegrandError("KLObjective: MonotoneIntegrand: nan was encountered in value of g(df(...)).");
        if (st & kStatusBudget) throw std::runtime_error("KLObjective: adaptive quadrature exceeded its interval budget.");
        return;
    }
    KLPlan& P = klPlan(W, parts_, N, onlyComp, stream);
    W.partials.ensure(std::max<size_t>(1, P.partialDoubles) * sizeof(double), stream);
    W.lossPart.ensure(std::max(1, P.nItems) * sizeof(double), stream);
    FusedParams p{};
    baseParams(W, opts_, p, N);
    p.flags = kFlagKL | kFlagCoefReduced;
    p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
    p.sensScale = 1.0 / (double)N;
    p.lsensScale = -1.0 / (double)N;
    p.partials = W.partials.as<double>();
    p.lossPartials = W.lossPart.as<double>();
    p.items = P.items.as<WorkItem>();
    p.rcache = rectCache(W, P.rcTotal, stream);
    orderPointsKL(W, P, parts_, pts, p, onlyComp, stream);
    const bool costOrder = p.perm != nullptr;
    if (costOrder) {
        P.costKey.ensure(parts_.size() * (size_t)N * sizeof(double), stream);
        p.costKey = P.costKey.as<double>();
        p.costStride = N;
    }
    const size_t smem = fusedSmemBytes(p.tpb, p.dmax, p.nBmax, p.depthMax, W.pmax, false);
    if (smem > 227 * 1024) throw std::invalid_argument("Component too large for the shared-memory tile.");
    p.stageDoubles = stageDoubles(W, p, false);
    MPGB_CUDA(launchFused(W.basis, posCode(opts_), W.pmax, p, P.nItems, 1, opts_.contDeriv ? 0 : 2, stream));
    MPGB_CUDA(launchKLReduce(W.partials.as<double>(), P.rowBase.as<long long>(), P.reduceDesc.as<KLReduceDesc>(),
                             P.nReduce, P.maxTerms, grad, W.lossPart.as<double>(), P.lossSlots.as<int>(),
                             1.0 / (double)N, lossPerComp, stream));
    if (costOrder) {
        // the processing order of the next call: every component's samples
        // sorted in one launch set
        const size_t c0 = onlyComp >= 0 ? (size_t)onlyComp : 0;
        const int nSeg = onlyComp >= 0 ? 1 : (int)parts_.size();
        MPGB_CUDA(launchSortByLastSegments(P.costKey.as<double>() + c0 * (size_t)N, 1, N, nSeg, N,
                                           W.sortHist.as<int>(), P.perm.as<int>() + c0 * (size_t)N, N, stream));
    }
    Finish(stream, "KLObjective");
}

void MonotoneMapBase::KLObjectiveCalls(StridedMatrix const& pts, double* lossPerComp, double* grad, int onlyComp,
                                       double* T, double* Ld, double* DT, double* DL, cudaStream_t stream) {
    const long long n = pts.cols;
    for (int c = 0; c < (int)parts_.size(); ++c) {
        if (onlyComp >= 0 && c != onlyComp) continue;
        const Part& p = parts_[c];
        auto* comp = dynamic_cast<MonotoneMapBase*>(p.owner);
        if (!comp || p.owner->numCoeffs != (unsigned)p.prog->numTerms)
            throw std::invalid_argument("KLObjective: the reference call sequence needs a map of monotone components.");
        const int nt = p.prog->numTerms;
        StridedMatrix sl(pts.data, p.prog->D, n, pts.rowStride, pts.colStride);
        StridedMatrix Tm(T, 1, n, n, 1), Lm(Ld, 1, n, n, 1), DTm(DT, nt, n, n, 1), DLm(DL, nt, n, n, 1);
        // Asynchronous: the caller checks the status once for all components.
        const bool wasAsync = comp->Async();
        comp->SetAsync(true);
        comp->EvaluateImpl(sl, Tm, stream);
        comp->LogDeterminantImpl(sl, Lm, stream);
        comp->CoeffGradImpl(sl, Tm, DTm, stream);
        comp->LogDeterminantCoeffGradImpl(sl, DLm, stream);
        comp->SetAsync(wasAsync);
        MPGB_CUDA(launchDenseKLReduce(T, Ld, DT, DL, nt, n, lossPerComp + p.outRow, grad + p.mapCoeffOffset, stream));
    }
}

// Implicit-function adjoint of the inverse.  For the functional
// L = sum w(k,i) x(k,i) of x = T^{-1}(x1, r) the adjoint solves, per point,
// (dT/dx)^T lambda = w: lambda_k = (w_k - sum_{m>k} lambda_m dT_m/dx_k) / dT_k/dx_k,
// components last to first.  Each component is one fused launch over all
// points: it reads the running sums from ptsGrad, forms lambda_k, adds
// lambda_k dT_k/dx_j (forward mode over the prefix tree plus the parameter
// quadrature) to rows j < k, and reduces lambda_k dT_k/dc into partial rows;
// dL/dc_k = -sum_i lambda_k dT_k/dc.
void MonotoneMapBase::InverseCoeffGrad(StridedMatrix const& pts, StridedMatrix const& w, double* coeffGrad,
                                       StridedMatrix const& ptsGrad, cudaStream_t stream) {
    CheckCoefficients("InverseCoeffGrad");
    const long long N = pts.cols;
    checkMatrix(pts, inputDim, N, "pts", "InverseCoeffGrad");
    checkMatrix(w, outputDim, N, "w", "InverseCoeffGrad");
    if (!ptsGrad.empty()) checkMatrix(ptsGrad, inputDim, N, "pts_grad", "InverseCoeffGrad");
    const int extra = (int)inputDim - (int)outputDim;
    for (auto& pt : parts_)
        if (pt.prog->D - 1 != extra + (int)pt.outRow)
            throw std::invalid_argument("InverseCoeffGrad: component inputs are not triangular in the map outputs.");
    if (!coeffGrad && ptsGrad.empty()) return;
    Prepare(stream);
    MapWorkspace& W = *ws_;
    if (N == 0) {
        if (coeffGrad) MPGB_CUDA(cudaMemsetAsync(coeffGrad, 0, numCoeffs * sizeof(double), stream));
        Finish(stream, "InverseCoeffGrad");
        return;
    }
    StridedMatrix G = ptsGrad;
    if (G.empty()) {
        W.implicitAcc.ensure((size_t)inputDim * N * sizeof(double), stream);
        G = StridedMatrix(W.implicitAcc.as<double>(), inputDim, N, N, 1);
    }
    // Components in decreasing output row.
    std::vector<int> order(parts_.size());
    for (size_t c = 0; c < parts_.size(); ++c) order[c] = (int)c;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return parts_[a].outRow > parts_[b].outRow; });
    const bool wantCoef = coeffGrad != nullptr;
    for (size_t q = 0; q < order.size(); ++q) {
        const int c = order[q];
        std::vector<long long> rowBase;
        std::vector<std::vector<int>> itemsOf;
        long long rcTotal = 0;
        auto items = itemsPerComp(parts_, N, W.numSMs, wantCoef, &rowBase, &itemsOf, c, &rcTotal);
        uploadItems(W, items, stream);
        FusedParams p{};
        baseParams(W, opts_, p, N);
        if (wantCoef) p.rcache = rectCache(W, rcTotal, stream);
        p.flags = kFlagInput | kFlagImplicit | (q == 0 ? kFlagImplicitFirst : 0) | (wantCoef ? kFlagCoefReduced : 0);
        p.pts = pts.data; p.ptsRs = pts.rowStride; p.ptsCs = pts.colStride;
        p.sens = w.data; p.sensRs = w.rowStride; p.sensCs = w.colStride;
        p.lsens = nullptr; p.lsensScale = 0.0;
        p.outInput = G.data; p.inputRs = G.rowStride; p.inputCs = G.colStride;
        p.negRows = (q + 1 == order.size()) ? extra : 0;
        if (wantCoef) {
            size_t nPart = 1;
            for (auto& it : items)
                nPart = std::max<size_t>(nPart, (size_t)it.partialBase +
                                                    (size_t)parts_[c].prog->numTerms * parts_[c].prog->cSegs);
            W.partials.ensure(nPart * sizeof(double), stream);
            p.partials = W.partials.as<double>();
        }
        orderPoints(W, parts_, pts, p, c, stream);
        launch(W, opts_, p, (int)items.size(), 1, 0, stream);
        if (wantCoef) {
            W.rowBase.ensure(sizeof(long long) * std::max<size_t>(1, rowBase.size()), stream);
            MPGB_CUDA(cudaMemcpyAsync(W.rowBase.p, rowBase.data(), rowBase.size() * sizeof(long long),
                                      cudaMemcpyHostToDevice, stream));
            MPGB_CUDA(launchReduceRows(W.partials.as<double>(), W.rowBase.as<long long>(), (int)rowBase.size(),
                                       parts_[c].prog->numTerms, -1.0, coeffGrad + parts_[c].mapCoeffOffset, 0,
                                       stream));
        }
    }
    Finish(stream, "InverseCoeffGrad");
}

// ---------------------------------------------------------------------------
// MonotoneComponent / TriangularMap / MapFactory
// ---------------------------------------------------------------------------
MonotoneComponent::MonotoneComponent(FixedMultiIndexSet const& mset, MapOptions const& opts)
    : MonotoneMapBase(mset.Length(), 1, mset.Size(), opts), mset_(mset) {
    validateOptions(opts);
    auto prog = std::make_shared<ComponentProgram>(mset);
    parts_.push_back({prog, this, 0, 0, 0});
}

void ConditionalMapBase::FillCoeffBoundsImpl(double* lb, double* ub) const {
    for (unsigned i = 0; i < numCoeffs; ++i) {
        lb[i] = -std::numeric_limits<double>::infinity();
        ub[i] = std::numeric_limits<double>::infinity();
    }
}

// HandleSigmoidComponentErrors (src/MapFactory.cpp:320-348).
static void validateSigmoidOptions(MapOptions const& o) {
    static const char* btypes[] = {"ProbabilistHermite", "PhysicistHermite", "HermiteFunctions"};
    if (o.basisType != BasisTypes::HermiteFunctions) {
        std::ostringstream os;
        os << "Unsupported basis type for sigmoid expansion: " << btypes[(int)o.basisType];
        throw std::invalid_argument(os.str());
    }
    if (o.posFuncType != PosFuncTypes::Exp && o.posFuncType != PosFuncTypes::SoftPlus)
        throw std::invalid_argument("Unsupported positive function type for sigmoid expansion.");
    if (o.edgeType != EdgeTypes::SoftPlus) throw std::invalid_argument("Unsupported edge type for sigmoid expansion.");
    if (o.sigmoidType != SigmoidTypes::Logistic)
        throw std::invalid_argument("Unsupported sigmoid type for sigmoid expansion.");
}

// The options a sigmoid expansion keeps: the quadrature fields play no part
// (their defaults keep the launch constants valid) and the derivative is exact.
static MapOptions sigmoidOptions(MapOptions o) {
    MapOptions d;
    o.quadType = d.quadType;
    o.quadAbsTol = d.quadAbsTol;
    o.quadRelTol = d.quadRelTol;
    o.quadMaxSub = d.quadMaxSub;
    o.quadMinSub = d.quadMinSub;
    o.quadPts = d.quadPts;
    o.contDeriv = true;
    o.nugget = 0.0;
    return o;
}

SigmoidComponent::SigmoidComponent(FixedMultiIndexSet const& mset, Sigmoid1dParams const& sigmoid,
                                   MapOptions const& opts)
    : MonotoneMapBase(mset.Length(), 1, mset.Size(), sigmoidOptions(opts)), mset_(mset), sig_(sigmoid) {
    validateSigmoidOptions(opts);
    sig_.Validate();
    const unsigned last = mset.MaxDegrees()[mset.Length() - 1];
    if ((int)last > sig_.Order()) {
        std::ostringstream os;
        os << "Sigmoid basis evaluation order too large: the multi-index set uses order " << last
           << " in the last input, the basis has order " << sig_.Order() << ".";
        throw std::invalid_argument(os.str());
    }
    auto prog = std::make_shared<ComponentProgram>(mset);
    prog->SetSigmoid(sig_, mset.Length() > 1);
    parts_.push_back({prog, this, 0, 0, 0});
}

std::vector<unsigned int> SigmoidComponent::DiagonalCoeffIndices() const {
    if (IsUnivariate()) {
        std::vector<unsigned int> all(numCoeffs);
        std::iota(all.begin(), all.end(), 0u);
        return all;
    }
    return mset_.NonzeroDiagonalEntries();
}

void SigmoidComponent::FillCoeffBoundsImpl(double* lb, double* ub) const {
    ConditionalMapBase::FillCoeffBoundsImpl(lb, ub);
    for (unsigned i : DiagonalCoeffIndices()) lb[i] = 0.0;
    if (IsUnivariate() && numCoeffs > 0) lb[0] = -std::numeric_limits<double>::infinity();
}

static void collectParts(ConditionalMapBase* comp, unsigned row, unsigned coeffOff,
                         std::vector<MonotoneMapBase::Part>& out, const MapOptions** optsSeen) {
    auto* mono = dynamic_cast<MonotoneMapBase*>(comp);
    if (!mono) throw std::invalid_argument("TriangularMap: components must be monotone components or triangular maps.");
    if (*optsSeen) {
        const MapOptions& a = **optsSeen;
        const MapOptions& b = mono->Options();
        if (a.basisType != b.basisType || a.posFuncType != b.posFuncType || a.quadAbsTol != b.quadAbsTol ||
            a.quadRelTol != b.quadRelTol || a.quadMaxSub != b.quadMaxSub || a.quadMinSub != b.quadMinSub ||
            a.quadPts != b.quadPts || a.basisNorm != b.basisNorm || a.nugget != b.nugget)
            throw std::invalid_argument("TriangularMap: components must share basis, rectifier and quadrature options.");
    } else {
        *optsSeen = &mono->Options();
    }
    (void)row;
    (void)coeffOff;
}

TriangularMap::TriangularMap(std::vector<std::shared_ptr<ConditionalMapBase>> const& components, bool moveCoeffs)
    : MonotoneMapBase(components.empty() ? 0 : components.back()->inputDim,
                      [&] { unsigned s = 0; for (auto& c : components) s += c->outputDim; return s; }(),
                      [&] { unsigned s = 0; for (auto& c : components) s += c->numCoeffs; return s; }(),
                      MapOptions()),
      comps_(components) {
    if (components.empty()) throw std::invalid_argument("TriangularMap: no components.");
    for (unsigned i = 0; i < comps_.size(); ++i) {
        if (comps_[i]->outputDim > comps_[i]->inputDim) {
            std::ostringstream os;
            os << "In TriangularMap constructor, the output dimension (" << comps_[i]->outputDim << ") of component " << i
               << " is greater than the input dimension (" << comps_[i]->inputDim << ").";
            throw std::invalid_argument(os.str());
        }
    }
    for (unsigned i = 1; i < comps_.size(); ++i) {
        if (comps_[i]->inputDim != comps_[i - 1]->inputDim + comps_[i]->outputDim) {
            std::ostringstream os;
            os << "In TriangularMap constructor, the input dimension of component " << i << " is "
               << comps_[i]->inputDim << ", but is expected to be the sum of the input dimension for component " << i - 1
               << "and output dimension for component " << i << ", which is " << comps_[i - 1]->inputDim << " + "
               << comps_[i]->outputDim << " = " << comps_[i - 1]->inputDim + comps_[i]->outputDim << ".";
            throw std::invalid_argument(os.str());
        }
    }
    const MapOptions* seen = nullptr;
    unsigned row = 0, coff = 0;
    for (auto& c : comps_) {
        collectParts(c.get(), row, coff, parts_, &seen);
        auto* mono = dynamic_cast<MonotoneMapBase*>(c.get());
        for (auto& sub : mono->Parts()) {
            Part np = sub;
            np.outRow = row + sub.outRow;
            np.mapCoeffOffset = coff + sub.mapCoeffOffset;
            parts_.push_back(np);
        }
        row += c->outputDim;
        coff += c->numCoeffs;
    }
    opts_ = *seen;
    if (moveCoeffs) {
        std::vector<double> all;
        for (unsigned i = 0; i < comps_.size(); ++i) {
            if (!comps_[i]->CheckCoefficients()) {
                std::ostringstream os;
                os << "In TriangularMap constructor, moveCoeffs set to true, but component " << i
                   << " doesn't have coeffs set";
                throw std::invalid_argument(os.str());
            }
            auto h = comps_[i]->CoeffMap();
            all.insert(all.end(), h.begin(), h.end());
        }
        MPGB_CUDA(cudaMalloc(&owned_, std::max<size_t>(1, all.size()) * sizeof(double)));
        if (!all.empty())
            MPGB_CUDA(cudaMemcpy(owned_, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice));
        WrapCoeffsLabeled(owned_, numCoeffs, "coeffs");
    }
}

void TriangularMap::FillCoeffBoundsImpl(double* lb, double* ub) const {
    unsigned off = 0;
    for (auto& c : comps_) {
        c->FillCoeffBoundsImpl(lb + off, ub + off);
        off += c->numCoeffs;
    }
}

// The components view slices of the map's coefficients, under its label.
void TriangularMap::SetCoeffs(const double* coeffs, unsigned int n, bool host, cudaStream_t stream) {
    ConditionalMapBase::SetCoeffs(coeffs, n, host, stream);
    unsigned off = 0;
    for (auto& c : comps_) {
        c->WrapCoeffsLabeled(coeffs_ + off, c->numCoeffs, coeffLabel_);
        off += c->numCoeffs;
    }
}

void TriangularMap::WrapCoeffsLabeled(double* deviceCoeffs, unsigned int n, std::string const& label) {
    ConditionalMapBase::WrapCoeffsLabeled(deviceCoeffs, n, label);
    unsigned off = 0;
    for (auto& c : comps_) {
        c->WrapCoeffsLabeled(coeffs_ + off, c->numCoeffs, coeffLabel_);
        off += c->numCoeffs;
    }
}

namespace MapFactory {
std::shared_ptr<ConditionalMapBase> CreateComponent(FixedMultiIndexSet const& mset, MapOptions opts) {
    auto c = std::make_shared<MonotoneComponent>(mset, opts);
    // Zero-initialised coefficients (src/MapFactoryImpl4.cpp:26-27).
    std::vector<double> z(c->numCoeffs, 0.0);
    c->SetCoeffs(z.data(), c->numCoeffs, true);
    return c;
}

std::shared_ptr<ConditionalMapBase> CreateTriangular(unsigned int inputDim, unsigned int outputDim,
                                                     unsigned int totalOrder, MapOptions options) {
    if (outputDim == 0 || outputDim > inputDim)
        throw std::invalid_argument("CreateTriangular: need 0 < outputDim <= inputDim.");
    validateOptions(options);
    std::vector<std::shared_ptr<ConditionalMapBase>> comps(outputDim);
    const unsigned extra = inputDim - outputDim;
    for (unsigned i = 0; i < outputDim; ++i) {
        FixedMultiIndexSet mset(i + extra + 1, totalOrder);
        comps[i] = std::make_shared<MonotoneComponent>(mset, options);
    }
    auto out = std::make_shared<TriangularMap>(comps);
    std::vector<double> z(out->numCoeffs, 0.0);
    out->SetCoeffs(z.data(), out->numCoeffs, true);
    return out;
}

// CreateSigmoidExpansionTemplate (src/MapFactory.cpp:256-318).
std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(FixedMultiIndexSet const& mset,
                                                           std::vector<double> const& centers, MapOptions opts) {
    validateSigmoidOptions(opts);
    auto sig = Sigmoid1dParams::FromCenters(centers, opts.edgeShape, opts.sigmoidBasisSumType);
    auto c = std::make_shared<SigmoidComponent>(mset, sig, opts);
    std::vector<double> z(c->numCoeffs, 0.0);
    c->SetCoeffs(z.data(), c->numCoeffs, true);
    return c;
}

std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(unsigned int inputDim, unsigned int offDiagOrder,
                                                           unsigned int crossOrder, std::vector<double> const& centers,
                                                           MapOptions opts) {
    validateSigmoidOptions(opts);
    if (inputDim == 0) throw std::invalid_argument("CreateSigmoidComponent: inputDim must be positive.");
    const int numSig = Sigmoid1dParams::ComputeNumSigmoids((unsigned)centers.size(), opts.sigmoidBasisSumType);
    if (numSig < 0) throw std::invalid_argument("Sigmoid: centers/widths/weights too short.");
    if (inputDim == 1) return CreateSigmoidComponent(FixedMultiIndexSet(1, numSig + 3), centers, opts);
    // Leading-input terms, then leading x sigmoid terms (order 0 excluded: it is in the first block).
    FixedMultiIndexSet m1 = FixedMultiIndexSet(inputDim - 1, offDiagOrder).Cartesian(FixedMultiIndexSet(1, 0));
    FixedMultiIndexSet m2 =
        FixedMultiIndexSet(inputDim - 1, crossOrder).Cartesian(FixedMultiIndexSet(1, numSig + 3, 1));
    return CreateSigmoidComponent(m1.Concatenate(m2), centers, opts);
}

std::shared_ptr<ConditionalMapBase> CreateSigmoidComponent(unsigned int inputDim, unsigned int totalOrder,
                                                           std::vector<double> const& centers, MapOptions opts) {
    return CreateSigmoidComponent(inputDim, totalOrder, totalOrder, centers, opts);
}

// src/MapFactory.cpp:389-407: component i has input dimension
// inputDim - outputDim + i + 1 and the centers centers[i].
std::shared_ptr<ConditionalMapBase> CreateSigmoidTriangular(unsigned int inputDim, unsigned int outputDim,
                                                            unsigned int totalOrder,
                                                            std::vector<std::vector<double>> const& centers,
                                                            MapOptions opts) {
    if (outputDim > inputDim) {
        std::ostringstream os;
        os << "CreateSigmoidTriangular: Output dimension " << outputDim << " cannot be greater than input dimension "
           << inputDim;
        throw std::invalid_argument(os.str());
    }
    if (outputDim == 0 || centers.size() != outputDim)
        throw std::invalid_argument("CreateSigmoidTriangular: need one vector of centers per output.");
    std::vector<std::shared_ptr<ConditionalMapBase>> comps(outputDim);
    for (unsigned i = 0; i < outputDim; ++i)
        comps[i] = CreateSigmoidComponent(inputDim - outputDim + i + 1, totalOrder, centers[i], opts);
    auto out = std::make_shared<TriangularMap>(comps);
    std::vector<double> z(out->numCoeffs, 0.0);
    out->SetCoeffs(z.data(), out->numCoeffs, true);
    return out;
}
}  // namespace MapFactory

}  // namespace mpgb

// ===========================================================================
// C ABI
// ===========================================================================
using namespace mpgb;

namespace mpgb {
int trainMapImpl(void* mapObj, mpgb_matrix samples, const mpgb_train_options* opts, double* loss_per_comp,
                 mpgb_train_result* res, void* stream, char* err, int errLen);
int trainMapAdaptiveImpl(unsigned int n_sets, const unsigned int* num_terms, const unsigned int* multis,
                         mpgb_matrix train, mpgb_matrix test, const mpgb_atm_options* opts, mpgb_map** out,
                         mpgb_atm_result* result, unsigned int* final_num_terms, void* stream, char* err, int errLen);
int reducedMarginImpl(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_out,
                      unsigned int* out, unsigned int cap_rows);
int expandImpl(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_terms_out,
               unsigned int* terms_out, unsigned int* n_idx_out, unsigned int* idx_out, unsigned int cap);
int optimizerSelfTestImpl(int algorithm, int which, int n, int maxIters, const double* dinv, double* xOut,
                          double* fOut, int* itersOut, int* evalsOut);
int klStepTimeImpl(void* mapObj, mpgb_matrix samples, int mode, int steps, double* ms_per_step, double* loss,
                   double* grad, void* stream, char* err, int errLen);
}

namespace {
thread_local std::string g_lastError;

}  // namespace

namespace mpgb {
void setLastError(const std::string& msg) { g_lastError = msg; }
}  // namespace mpgb

namespace {

template <class F>
int guard(F&& f) {
    try {
        f();
        return MPGB_OK;
    } catch (IntegrandError const& e) {
        g_lastError = e.what();
        return MPGB_ERR_INTEGRAND;
    } catch (CudaError const& e) {
        g_lastError = e.what();
        return MPGB_ERR_CUDA;
    } catch (std::invalid_argument const& e) {
        g_lastError = e.what();
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::out_of_range const& e) {
        g_lastError = e.what();
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        g_lastError = e.what();
        return MPGB_ERR_RUNTIME;
    } catch (...) {
        g_lastError = "unknown error";
        return MPGB_ERR_RUNTIME;
    }
}


MonotoneMapBase* mono(mpgb_map* m) {
    if (!m || !m->obj) throw std::invalid_argument("null map handle");
    auto* p = dynamic_cast<MonotoneMapBase*>(m->obj.get());
    if (!p) throw std::invalid_argument("map is not a monotone map");
    return p;
}

bool isHostPtr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

StridedMatrix toSM(const mpgb_matrix& m) { return StridedMatrix(m.data, m.rows, m.cols, m.row_stride, m.col_stride); }

// Host staging: host matrices are copied to (or from) contiguous row-major
// device buffers owned by the map (grow-only, reused across calls).
struct Stager {
    cudaStream_t s;
    MonotoneMapBase* m;
    int next = 0;
    std::vector<std::pair<StridedMatrix, StridedMatrix>> copyBack;  // (device, host)
    bool staged = false;
    Stager(cudaStream_t st, MonotoneMapBase* map) : s(st), m(map) {}
    static void copy2D(const StridedMatrix& dst, const StridedMatrix& src, cudaMemcpyKind kind, cudaStream_t s) {
        if (src.rows == 0 || src.cols == 0) return;
        if (src.colStride == 1 && dst.colStride == 1) {
            MPGB_CUDA(cudaMemcpy2DAsync(dst.data, dst.rowStride * 8, src.data, src.rowStride * 8, src.cols * 8,
                                        src.rows, kind, s));
        } else if (src.rows == 1) {
            MPGB_CUDA(cudaMemcpy2DAsync(dst.data, dst.colStride * 8, src.data, src.colStride * 8, 8, src.cols, kind, s));
        } else {
            for (int64_t r = 0; r < src.rows; ++r)
                MPGB_CUDA(cudaMemcpy2DAsync(dst.data + r * dst.rowStride, dst.colStride * 8,
                                            src.data + r * src.rowStride, src.colStride * 8, 8, src.cols, kind, s));
        }
    }
    double* buffer(size_t n) {
        if (next >= 8) throw std::invalid_argument("too many host-staged arrays in one call");
        staged = true;
        return m->StagingBuffer(next++, std::max<size_t>(1, n) * 8, s);
    }
    StridedMatrix in(const mpgb_matrix& mm) {
        StridedMatrix h = toSM(mm);
        if (!mm.data || !isHostPtr(mm.data)) return h;
        StridedMatrix dm(buffer((size_t)mm.rows * mm.cols), mm.rows, mm.cols, mm.cols, 1);
        copy2D(dm, h, cudaMemcpyHostToDevice, s);
        return dm;
    }
    StridedMatrix out(const mpgb_matrix& mm) {
        StridedMatrix h = toSM(mm);
        if (!mm.data || !isHostPtr(mm.data)) return h;
        StridedMatrix dm(buffer((size_t)mm.rows * mm.cols), mm.rows, mm.cols, mm.cols, 1);
        copyBack.push_back({dm, h});
        return dm;
    }
    double* outVec(double* p, size_t n) {
        if (!p || !isHostPtr(p)) return p;
        double* d = buffer(n);
        copyBack.push_back({StridedMatrix(d, 1, (int64_t)n, (int64_t)n, 1), StridedMatrix(p, 1, (int64_t)n, (int64_t)n, 1)});
        return d;
    }
    void finish() {
        for (auto& pr : copyBack) copy2D(pr.second, pr.first, cudaMemcpyDeviceToHost, s);
        if (staged) MPGB_CUDA(cudaStreamSynchronize(s));
    }
};

}  // namespace

extern "C" {

const char* mpgb_version(void) { return "mpart_gb300 0.1.0 (sm_103a, FP64)"; }
const char* mpgb_last_error(void) { return g_lastError.c_str(); }

int mpgb_map_options_default(mpgb_map_options* o) {
    return guard([&] {
        if (!o) throw std::invalid_argument("null options");
        MapOptions m;
        o->basis_type = (int)m.basisType;
        o->pos_func_type = (int)m.posFuncType;
        o->quad_type = (int)m.quadType;
        o->quad_abs_tol = m.quadAbsTol;
        o->quad_rel_tol = m.quadRelTol;
        o->quad_max_sub = m.quadMaxSub;
        o->quad_min_sub = m.quadMinSub;
        o->quad_pts = m.quadPts;
        o->cont_deriv = m.contDeriv;
        o->basis_norm = m.basisNorm;
        o->nugget = m.nugget;
        o->sigmoid_type = (int)m.sigmoidType;
        o->edge_type = (int)m.edgeType;
        o->edge_shape = m.edgeShape;
        o->sigmoid_sum_type = (int)m.sigmoidBasisSumType;
    });
}

int mpgb_create_component(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                          const unsigned int* nz_dims, const unsigned int* nz_orders, const mpgb_map_options* opts,
                          mpgb_map** out) {
    return guard([&] {
        if (!out || !nz_starts) throw std::invalid_argument("null argument");
        std::vector<unsigned> s(nz_starts, nz_starts + num_terms + 1);
        const unsigned nnz = s.back();
        if (nnz > 0 && (!nz_dims || !nz_orders)) throw std::invalid_argument("null nonzero arrays");
        std::vector<unsigned> d(nz_dims, nz_dims + nnz), o(nz_orders, nz_orders + nnz);
        FixedMultiIndexSet ms(dim, s, d, o);
        *out = new mpgb_map{MapFactory::CreateComponent(ms, mapOptionsFromC(opts))};
    });
}

int mpgb_create_component_total_order(unsigned int dim, unsigned int order, const mpgb_map_options* opts,
                                      mpgb_map** out) {
    return guard([&] {
        if (!out) throw std::invalid_argument("null argument");
        FixedMultiIndexSet ms(dim, order);
        *out = new mpgb_map{MapFactory::CreateComponent(ms, mapOptionsFromC(opts))};
    });
}

int mpgb_create_triangular(unsigned int input_dim, unsigned int output_dim, unsigned int total_order,
                           const mpgb_map_options* opts, mpgb_map** out) {
    return guard([&] {
        if (!out) throw std::invalid_argument("null argument");
        *out = new mpgb_map{MapFactory::CreateTriangular(input_dim, output_dim, total_order, mapOptionsFromC(opts))};
    });
}

int mpgb_create_triangular_from_components(mpgb_map* const* components, unsigned int n, int move_coeffs,
                                           mpgb_map** out) {
    return guard([&] {
        if (!out || !components) throw std::invalid_argument("null argument");
        std::vector<std::shared_ptr<ConditionalMapBase>> v;
        for (unsigned i = 0; i < n; ++i) {
            if (!components[i]) throw std::invalid_argument("null component");
            v.push_back(components[i]->obj);
        }
        *out = new mpgb_map{std::make_shared<TriangularMap>(v, move_coeffs != 0)};
    });
}

static std::vector<double> hostVector(const double* p, unsigned n) {
    if (n && !p) throw std::invalid_argument("null centers");
    return std::vector<double>(p, p + n);
}

int mpgb_create_sigmoid_component(unsigned int input_dim, unsigned int off_diag_order, unsigned int cross_order,
                                  const double* centers, unsigned int n_centers, const mpgb_map_options* opts,
                                  mpgb_map** out) {
    return guard([&] {
        if (!out) throw std::invalid_argument("null argument");
        *out = new mpgb_map{MapFactory::CreateSigmoidComponent(input_dim, off_diag_order, cross_order,
                                                               hostVector(centers, n_centers), mapOptionsFromC(opts))};
    });
}

int mpgb_create_sigmoid_component_mset(unsigned int dim, unsigned int num_terms, const unsigned int* nz_starts,
                                       const unsigned int* nz_dims, const unsigned int* nz_orders,
                                       const double* centers, unsigned int n_centers,
                                       const mpgb_map_options* opts, mpgb_map** out) {
    return guard([&] {
        if (!out || !nz_starts) throw std::invalid_argument("null argument");
        std::vector<unsigned> st(nz_starts, nz_starts + num_terms + 1);
        const unsigned nnz = st.back();
        if (nnz > 0 && (!nz_dims || !nz_orders)) throw std::invalid_argument("null nonzero arrays");
        FixedMultiIndexSet ms(dim, st, std::vector<unsigned>(nz_dims, nz_dims + nnz),
                              std::vector<unsigned>(nz_orders, nz_orders + nnz));
        *out = new mpgb_map{MapFactory::CreateSigmoidComponent(ms, hostVector(centers, n_centers), mapOptionsFromC(opts))};
    });
}

int mpgb_create_sigmoid_triangular(unsigned int input_dim, unsigned int output_dim, unsigned int total_order,
                                   const double* centers, unsigned int n_centers, int64_t row_stride,
                                   int64_t col_stride, const mpgb_map_options* opts, mpgb_map** out) {
    return guard([&] {
        if (!out || (n_centers && !centers)) throw std::invalid_argument("null argument");
        std::vector<std::vector<double>> cs(output_dim, std::vector<double>(n_centers));
        for (unsigned j = 0; j < output_dim; ++j)
            for (unsigned i = 0; i < n_centers; ++i) cs[j][i] = centers[(int64_t)i * row_stride + (int64_t)j * col_stride];
        *out = new mpgb_map{MapFactory::CreateSigmoidTriangular(input_dim, output_dim, total_order, cs, mapOptionsFromC(opts))};
    });
}

int mpgb_map_coeff_bounds(const mpgb_map* map, double* lb, double* ub) {
    return guard([&] {
        if (!map || !lb || !ub) throw std::invalid_argument("null argument");
        map->obj->FillCoeffBoundsImpl(lb, ub);
    });
}

int mpgb_map_kind(const mpgb_map* map, int* kind) {
    return guard([&] {
        if (!map || !kind) throw std::invalid_argument("null argument");
        if (dynamic_cast<TriangularMap*>(map->obj.get())) *kind = -1;
        else if (auto* s = dynamic_cast<SigmoidComponent*>(map->obj.get())) *kind = s->IsUnivariate() ? 2 : 1;
        else *kind = 0;
    });
}

int mpgb_component_sigmoid(const mpgb_map* component, double* centers, double* widths, double* weights,
                           unsigned int* n_centers, unsigned int* starts, unsigned int* n_starts) {
    return guard([&] {
        if (!component) throw std::invalid_argument("null map handle");
        auto* s = dynamic_cast<SigmoidComponent*>(component->obj.get());
        if (!s) throw std::invalid_argument("not a sigmoid expansion");
        const Sigmoid1dParams& p = s->GetSigmoid();
        if (n_centers) *n_centers = (unsigned)p.centers.size();
        if (n_starts) *n_starts = (unsigned)p.startInds.size();
        if (centers) std::copy(p.centers.begin(), p.centers.end(), centers);
        if (widths) std::copy(p.widths.begin(), p.widths.end(), widths);
        if (weights) std::copy(p.weights.begin(), p.weights.end(), weights);
        if (starts) std::copy(p.startInds.begin(), p.startInds.end(), starts);
    });
}

int mpgb_sigmoid_params(const double* centers, unsigned int n, double edge_shape, int sum_type,
                        double* out_centers, double* widths, double* weights, unsigned int* starts,
                        unsigned int* n_starts) {
    return guard([&] {
        if (sum_type < 0 || sum_type > 1) throw std::invalid_argument("invalid sigmoid sum type");
        Sigmoid1dParams p = Sigmoid1dParams::FromCenters(hostVector(centers, n), edge_shape, (SigmoidSumSizeType)sum_type);
        if (out_centers) std::copy(p.centers.begin(), p.centers.end(), out_centers);
        if (widths) std::copy(p.widths.begin(), p.widths.end(), widths);
        if (weights) std::copy(p.weights.begin(), p.weights.end(), weights);
        if (starts) std::copy(p.startInds.begin(), p.startInds.end(), starts);
        if (n_starts) *n_starts = (unsigned)p.startInds.size();
    });
}

int mpgb_sigmoid1d_evaluate(const double* centers, const double* widths, const double* weights, unsigned int n,
                            const unsigned int* starts, unsigned int n_starts, int which, unsigned int max_order,
                            const double* x, int64_t n_x, int64_t x_stride, double* out, double* d1, double* d2,
                            void* stream) {
    return guard([&] {
        if (which < 0 || which > 2) throw std::invalid_argument("which must be 0, 1 or 2");
        Sigmoid1dParams p;
        p.centers = hostVector(centers, n);
        p.widths = hostVector(widths, n);
        p.weights = hostVector(weights, n);
        if (n_starts && !starts) throw std::invalid_argument("null starts");
        p.startInds.assign(starts, starts + n_starts);
        p.Validate();
        if ((int)max_order > p.Order()) throw std::invalid_argument("Sigmoid basis evaluation order too large.");
        if (n_x <= 0) return;
        if (!x || !out || (which >= 1 && !d1) || (which == 2 && !d2)) throw std::invalid_argument("null array");
        cudaStream_t s = (cudaStream_t)stream;
        std::vector<int32_t> st(p.startInds.begin(), p.startInds.end());
        DevBuf buf;
        const size_t nd = 3 * (size_t)n, ni = st.size();
        buf.ensure(nd * sizeof(double) + ni * sizeof(int32_t) + 16, s);
        double* dp = buf.as<double>();
        MPGB_CUDA(cudaMemcpyAsync(dp, p.centers.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
        MPGB_CUDA(cudaMemcpyAsync(dp + n, p.widths.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
        MPGB_CUDA(cudaMemcpyAsync(dp + 2 * n, p.weights.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
        int32_t* ip = (int32_t*)(dp + nd);
        if (ni) MPGB_CUDA(cudaMemcpyAsync(ip, st.data(), ni * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        CompDesc c{};
        c.sigC = dp; c.sigW = dp + n; c.sigWt = dp + 2 * n; c.sigStart = ip;
        c.sigN = (int)n; c.sigNStarts = (int)ni;
        MPGB_CUDA(launchSigmoidEval(c, (int)max_order, x, n_x, x_stride, out, which >= 1 ? d1 : nullptr,
                                    which == 2 ? d2 : nullptr, s));
        MPGB_CUDA(cudaStreamSynchronize(s));
    });
}

int mpgb_map_destroy(mpgb_map* map) {
    return guard([&] { delete map; });
}

int mpgb_map_dims(const mpgb_map* map, unsigned int* in, unsigned int* outd, unsigned int* nc) {
    return guard([&] {
        if (!map) throw std::invalid_argument("null map handle");
        if (in) *in = map->obj->inputDim;
        if (outd) *outd = map->obj->outputDim;
        if (nc) *nc = map->obj->numCoeffs;
    });
}

int mpgb_map_num_components(const mpgb_map* map, unsigned int* n) {
    return guard([&] {
        if (!map || !n) throw std::invalid_argument("null argument");
        auto* t = dynamic_cast<TriangularMap*>(map->obj.get());
        *n = t ? t->NumComponents() : 1;
    });
}

int mpgb_map_is_triangular(const mpgb_map* map, int* is_triangular) {
    return guard([&] {
        if (!map || !is_triangular) throw std::invalid_argument("null argument");
        *is_triangular = dynamic_cast<TriangularMap*>(map->obj.get()) ? 1 : 0;
    });
}

int mpgb_map_get_component(mpgb_map* map, unsigned int i, mpgb_map** out) {
    return guard([&] {
        if (!map || !out) throw std::invalid_argument("null argument");
        auto* t = dynamic_cast<TriangularMap*>(map->obj.get());
        if (!t) {
            if (i != 0) throw std::out_of_range("component index out of range");
            *out = new mpgb_map{map->obj};
            return;
        }
        if (i >= t->NumComponents()) throw std::out_of_range("component index out of range");
        *out = new mpgb_map{t->GetComponent(i)};
    });
}

int mpgb_set_coeffs(mpgb_map* map, const double* coeffs, unsigned int n, int is_host, void* stream) {
    return guard([&] {
        if (!map) throw std::invalid_argument("null map handle");
        if (n && !coeffs) throw std::invalid_argument("null coefficients");
        map->obj->SetCoeffs(coeffs, n, is_host != 0, (cudaStream_t)stream);
        if (!map->obj->Async()) MPGB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    });
}

int mpgb_wrap_coeffs(mpgb_map* map, double* device_coeffs, unsigned int n) {
    return guard([&] {
        if (!map) throw std::invalid_argument("null map handle");
        map->obj->WrapCoeffs(device_coeffs, n);
    });
}

int mpgb_get_coeffs(const mpgb_map* map, double* host_out, unsigned int n) {
    return guard([&] {
        if (!map || !host_out) throw std::invalid_argument("null argument");
        if (n != map->obj->numCoeffs) throw std::invalid_argument("wrong coefficient count");
        auto v = map->obj->CoeffMap();
        std::copy(v.begin(), v.end(), host_out);
    });
}

int mpgb_coeffs_device_ptr(const mpgb_map* map, double** out) {
    return guard([&] {
        if (!map || !out) throw std::invalid_argument("null argument");
        *out = map->obj->Coeffs();
    });
}

int mpgb_set_point_ordering(mpgb_map* map, int on) {
    return guard([&] { mono(map)->SetPointOrdering(on != 0); });
}

int mpgb_set_async(mpgb_map* map, int async) {
    return guard([&] {
        if (!map) throw std::invalid_argument("null map handle");
        map->obj->SetAsync(async != 0);
    });
}

int mpgb_check_status(mpgb_map* map, void* stream, int* status) {
    return guard([&] {
        int st = mono(map)->CheckStatus((cudaStream_t)stream);
        if (status) *status = st;
    });
}

int mpgb_evaluate(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto O = st.out(out);
        mono(map)->EvaluateImpl(P, O, s);
        st.finish();
    });
}

int mpgb_log_determinant(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto O = st.out(out);
        mono(map)->LogDeterminantImpl(P, O, s);
        st.finish();
    });
}

int mpgb_inverse(mpgb_map* map, mpgb_matrix x1, mpgb_matrix r, mpgb_matrix out, double xtol, double ytol,
                 int* device_info, void* stream) {
    return mpgb_inverse_method(map, x1, r, out, xtol, ytol, MPGB_INVERSE_BRACKET, device_info, stream);
}

int mpgb_inverse_method(mpgb_map* map, mpgb_matrix x1, mpgb_matrix r, mpgb_matrix out, double xtol, double ytol,
                        int method, int* device_info, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto X = st.in(x1);
        auto R = st.in(r);
        auto O = st.out(out);
        InverseOptions io;
        io.xtol = xtol;
        io.ytol = ytol;
        io.method = method;
        mono(map)->InverseImpl(X, R, O, io, device_info, s);
        st.finish();
    });
}

int mpgb_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto S = st.in(sens);
        auto O = st.out(out);
        mono(map)->CoeffGradImpl(P, S, O, s);
        st.finish();
    });
}

int mpgb_gradient(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto S = st.in(sens);
        auto O = st.out(out);
        mono(map)->GradientImpl(P, S, O, s);
        st.finish();
    });
}

int mpgb_log_determinant_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto O = st.out(out);
        mono(map)->LogDeterminantCoeffGradImpl(P, O, s);
        st.finish();
    });
}

int mpgb_log_determinant_input_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix out, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto O = st.out(out);
        mono(map)->LogDeterminantInputGradImpl(P, O, s);
        st.finish();
    });
}

int mpgb_fused_fwd_adj(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix logdet_sens,
                       double logdet_sens_scale, mpgb_matrix out_eval, mpgb_matrix out_logdet, double* coeff_grad,
                       mpgb_matrix input_grad, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        auto* m = mono(map);
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto S = st.in(sens);
        auto L = st.in(logdet_sens);
        auto E = st.out(out_eval);
        auto D = st.out(out_logdet);
        auto G = st.out(input_grad);
        double* cg = st.outVec(coeff_grad, m->numCoeffs);
        m->FusedForwardAdjoint(P, S, L, logdet_sens_scale, E, D, cg, G, s);
        st.finish();
    });
}

int mpgb_inverse_coeff_grad(mpgb_map* map, mpgb_matrix pts, mpgb_matrix w, double* coeff_grad, mpgb_matrix pts_grad,
                            void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        auto* m = mono(map);
        Stager st(s, mono(map));
        auto P = st.in(pts);
        auto Wt = st.in(w);
        auto G = st.out(pts_grad);
        double* cg = st.outVec(coeff_grad, m->numCoeffs);
        m->InverseCoeffGrad(P, Wt, cg, G, s);
        st.finish();
    });
}

int mpgb_kl_objective(mpgb_map* map, mpgb_matrix pts, double* loss, double* grad, void* stream) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        auto* m = mono(map);
        if (!loss || !grad) throw std::invalid_argument("null output");
        Stager st(s, mono(map));
        auto P = st.in(pts);
        double* l = st.outVec(loss, m->outputDim);
        double* g = st.outVec(grad, m->numCoeffs);
        m->KLObjective(P, l, g, s);
        st.finish();
    });
}

int mpgb_train_options_default(mpgb_train_options* o) {
    return guard([&] {
        if (!o) throw std::invalid_argument("null options");
        std::memset(o, 0, sizeof(*o));
        o->max_iters = 100;
        o->max_evals = 1000;
        o->memory = 10;
        o->mode = 0;
    });
}

int mpgb_train_map(mpgb_map* map, mpgb_matrix samples, const mpgb_train_options* opts, double* loss_per_comp,
                   mpgb_train_result* result, void* stream) {
    char err[512] = {0};
    int rc = MPGB_OK;
    int g = guard([&] {
        rc = trainMapImpl(mono(map), samples, opts, loss_per_comp, result, stream, err, sizeof(err));
    });
    if (g != MPGB_OK) return g;
    if (rc != MPGB_OK) g_lastError = err;
    return rc;
}

int mpgb_kl_step_time(mpgb_map* map, mpgb_matrix samples, int mode, int steps, double* ms_per_step, double* loss,
                      double* grad, void* stream) {
    char err[512] = {0};
    int rc = MPGB_OK;
    int g = guard([&] {
        rc = klStepTimeImpl(mono(map), samples, mode, steps, ms_per_step, loss, grad, stream, err, sizeof(err));
    });
    if (g != MPGB_OK) return g;
    if (rc != MPGB_OK) g_lastError = err;
    return rc;
}

long long mpgb_launch_count(void) { return mpgb::launchCount(); }

int mpgb_atm_options_default(mpgb_atm_options* o) {
    return guard([&] {
        if (!o) throw std::invalid_argument("null options");
        std::memset(o, 0, sizeof(*o));
        mpgb_map_options_default(&o->map);
        mpgb_train_options_default(&o->train);
        o->max_patience = 10;
        o->max_size = 0x7fffffffu;
        o->max_degrees = nullptr;
        o->verbose = 0;
    });
}

int mpgb_train_map_adaptive(unsigned int n_sets, const unsigned int* num_terms, const unsigned int* multis,
                            mpgb_matrix train, mpgb_matrix test, const mpgb_atm_options* opts, mpgb_map** out,
                            mpgb_atm_result* result, unsigned int* final_num_terms, void* stream) {
    char err[512] = {0};
    int rc = MPGB_OK;
    int g = guard([&] {
        rc = trainMapAdaptiveImpl(n_sets, num_terms, multis, train, test, opts, out, result, final_num_terms, stream,
                                  err, sizeof(err));
    });
    if (g != MPGB_OK) return g;
    if (rc != MPGB_OK) g_lastError = err;
    return rc;
}

int mpgb_reduced_margin(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_out,
                        unsigned int* out, unsigned int cap_rows) {
    return guard([&] {
        if ((n && !multis) || dim == 0) throw std::invalid_argument("bad multi-index set");
        reducedMarginImpl(dim, n, multis, n_out, out, cap_rows);
    });
}

int mpgb_optimizer_self_test(int algorithm, int problem, int n, int max_iters, const double* diag_inverse,
                             double* x_out, double* f_out, int* iterations, int* evaluations) {
    return guard([&] {
        if (!x_out || !f_out || !iterations || !evaluations) throw std::invalid_argument("null output");
        optimizerSelfTestImpl(algorithm, problem, n, max_iters, diag_inverse, x_out, f_out, iterations, evaluations);
    });
}

int mpgb_multi_index_expand(unsigned int dim, unsigned int n, const unsigned int* multis, unsigned int* n_terms_out,
                            unsigned int* terms_out, unsigned int* n_idx_out, unsigned int* idx_out,
                            unsigned int cap) {
    return guard([&] {
        if ((n && !multis) || dim == 0) throw std::invalid_argument("bad multi-index set");
        expandImpl(dim, n, multis, n_terms_out, terms_out, n_idx_out, idx_out, cap);
    });
}

int mpgb_component_multi_index(const mpgb_map* component, unsigned int* dim, unsigned int* num_terms,
                               unsigned int* nnz, unsigned int* nz_starts, unsigned int* nz_dims,
                               unsigned int* nz_orders) {
    return guard([&] {
        if (!component || !component->obj) throw std::invalid_argument("null map handle");
        const FixedMultiIndexSet* ms = nullptr;
        if (auto* c = dynamic_cast<const MonotoneComponent*>(component->obj.get())) ms = &c->GetMultiIndexSet();
        else if (auto* g = dynamic_cast<const SigmoidComponent*>(component->obj.get())) ms = &g->GetMultiIndexSet();
        if (!ms) throw std::invalid_argument("not a single monotone component or sigmoid expansion");
        const FixedMultiIndexSet& m = *ms;
        if (dim) *dim = m.Length();
        if (num_terms) *num_terms = m.Size();
        if (nnz) *nnz = (unsigned)m.nzDims.size();
        if (nz_starts) std::memcpy(nz_starts, m.nzStarts.data(), m.nzStarts.size() * sizeof(unsigned));
        if (nz_dims && !m.nzDims.empty()) std::memcpy(nz_dims, m.nzDims.data(), m.nzDims.size() * sizeof(unsigned));
        if (nz_orders && !m.nzOrders.empty())
            std::memcpy(nz_orders, m.nzOrders.data(), m.nzOrders.size() * sizeof(unsigned));
    });
}

int mpgb_fp64_probe(int blocks, int threads, int iters, void* stream, float* ms) {
    return guard([&] {
        cudaStream_t s = (cudaStream_t)stream;
        double* raw = nullptr;
        MPGB_CUDA(cudaMalloc(&raw, 8));
        std::unique_ptr<double, cudaError_t (*)(void*)> d(raw, cudaFree);
        EventPair ev;
        MPGB_CUDA(cudaEventRecord(ev.a, s));
        MPGB_CUDA(launchDfmaPeak(d.get(), blocks, threads, iters, s));
        MPGB_CUDA(cudaEventRecord(ev.b, s));
        MPGB_CUDA(cudaEventSynchronize(ev.b));
        if (ms) *ms = ev.ms();
    });
}

}  // extern "C"
