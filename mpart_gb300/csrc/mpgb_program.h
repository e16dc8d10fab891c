// Internal: the component program (prefix-tree tables on the device) and
// small host helpers shared by the host translation units.
#pragma once
#include <algorithm>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mpart_gb300.h"
#include "../../include/mpart_gb300.hpp"
#include "mpgb_types.h"

namespace mpgb {

#define MPGB_CUDA(call)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            std::ostringstream os_;                                                                       \
            os_ << "CUDA error " << cudaGetErrorName(e_) << " (" << cudaGetErrorString(e_) << ") at " #call; \
            throw CudaError(os_.str());                                                                   \
        }                                                                                                 \
    } while (0)

struct CudaError : public std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Two CUDA events for timing, destroyed on every exit path.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        MPGB_CUDA(cudaEventCreate(&a));
        const cudaError_t e = cudaEventCreate(&b);
        if (e != cudaSuccess) {
            cudaEventDestroy(a);
            a = nullptr;
            MPGB_CUDA(e);
        }
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    EventPair(const EventPair&) = delete;
    EventPair& operator=(const EventPair&) = delete;
    // Milliseconds between the two events (b must have completed).
    float ms() const {
        float t = 0;
        MPGB_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
};

// Quadrature rules (AdaptiveClenshawCurtis) and basis constants for a launch.
void buildLaunchConstants(const MapOptions& o, QuadParams& q, BasisConsts& b);

// MapOptions from the C ABI's struct (defaults for a null pointer); throws
// std::invalid_argument for enum values out of range.
MapOptions mapOptionsFromC(const mpgb_map_options* o);

// Looks up the no-allocation entry point's scratch array on the current
// device (mpgb_noalloc.cu), so that the module holding it is loaded, and its
// memory reserved, when maps are created rather than inside that entry point.
void reserveNoAllocScratch() noexcept;

// ---------------------------------------------------------------------------
// Component program: the multi-index set reorganised as a prefix tree over
// the leading coordinates (see mpgb_device.cuh for the factorisation).
// ---------------------------------------------------------------------------
template <class T>
static T* toDevice(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    T* d = nullptr;
    MPGB_CUDA(cudaMalloc(&d, v.size() * sizeof(T)));
    MPGB_CUDA(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return d;
}

struct ComponentProgram {
    int D = 0, P = 0, nB = 0, nNodes = 0, nSlots = 0, nCNodes = 0, maxDepth = 0, numTerms = 0;
    std::vector<uint32_t> nodeA, nodeSlot, nodeC;
    std::vector<uint16_t> nodeCRows;
    std::vector<int32_t> slotTerm, leadDeg, rowOff, nodeCIdx;
    uint32_t *dNodeA = nullptr, *dNodeSlot = nullptr, *dNodeC = nullptr;
    uint16_t* dNodeCRows = nullptr;
    int32_t *dSlotTerm = nullptr, *dLeadDeg = nullptr, *dRowOff = nullptr, *dNodeCIdx = nullptr;
    // Work per point (FP64 operations of phases A and C), for load balancing.
    double weight = 1.0;
    // Integrand dimension of the reference component's quadrature object,
    // which its operations set in place (quad_.SetDim, MonotoneComponent.h:270,
    // :401, :599, :697, :770, :940) and its map archive records; no effect on
    // the computation here.
    unsigned quadDim = 1;
    // Reduced adjoint: the tile's points are split into cSegs segments and the
    // block's threads take (node, segment) units, so that a few hundred nodes
    // still keep every thread busy; each segment has its own partial row.
    int cSegs = 1;
    // Sigmoid expansions: kind 1 = rectified (RectifiedMultivariateExpansion),
    // kind 2 = one input without rectifier (UnivariateExpansion); kind 0 is a
    // monotone component.  The last input's Sigmoid1d parameters live on the
    // device next to the tree tables.
    int kind = 0;
    std::vector<double> sigC, sigW, sigWt;
    std::vector<int32_t> sigStart;
    double *dSigC = nullptr, *dSigW = nullptr, *dSigWt = nullptr;
    int32_t* dSigStart = nullptr;

    void SetSigmoid(Sigmoid1dParams const& sp, bool rectify) {
        kind = rectify ? 1 : 2;
        sigC = sp.centers;
        sigW = sp.widths;
        sigWt = sp.weights;
        sigStart.assign(sp.startInds.begin(), sp.startInds.end());
        dSigC = toDevice(sigC);
        dSigW = toDevice(sigW);
        dSigWt = toDevice(sigWt);
        dSigStart = toDevice(sigStart);
        // Per point: the tree walks plus a rectifier per node (phases A and C)
        // and the sigmoid sums.
        weight += 40.0 * nNodes + 10.0 * (double)sigC.size();
    }

    explicit ComponentProgram(FixedMultiIndexSet const& ms) {
        D = (int)ms.Length();
        numTerms = (int)ms.Size();
        const auto& md = ms.maxDegrees;
        P = (int)md[D - 1];
        if (P > kMaxLastOrder) {
            std::ostringstream os;
            os << "MonotoneComponent: order " << P << " in the last input exceeds the supported maximum "
               << kMaxLastOrder << ".";
            throw std::invalid_argument(os.str());
        }
        leadDeg.resize(std::max(D - 1, 0));
        rowOff.resize(std::max(D - 1, 0));
        for (int d = 0; d + 1 < D; ++d) {
            leadDeg[d] = (int)md[d];
            rowOff[d] = nB;
            nB += (int)md[d];
        }
        if (nB >= (1 << 14)) throw std::invalid_argument("MonotoneComponent: basis table too large.");
        // Trie over the leading-coordinate prefixes.
        struct TNode {
            int parent, depth, dim, order;
            std::map<std::pair<int, int>, int> children;
            std::map<int, int> kTerm;
        };
        std::vector<TNode> tn;
        tn.push_back({-1, 0, 0, 0, {}, {}});
        for (int t = 0; t < numTerms; ++t) {
            int b = (int)ms.nzStarts[t], e = (int)ms.nzStarts[t + 1];
            int k = 0;
            if (e > b && (int)ms.nzDims[e - 1] == D - 1) {
                k = (int)ms.nzOrders[e - 1];
                --e;
            }
            int cur = 0;
            for (int i = b; i < e; ++i) {
                std::pair<int, int> key((int)ms.nzDims[i], (int)ms.nzOrders[i]);
                auto it = tn[cur].children.find(key);
                if (it == tn[cur].children.end()) {
                    TNode nn{cur, tn[cur].depth + 1, key.first, key.second, {}, {}};
                    tn.push_back(nn);
                    int id = (int)tn.size() - 1;
                    tn[cur].children[key] = id;
                    cur = id;
                } else {
                    cur = it->second;
                }
            }
            if (tn[cur].kTerm.count(k))
                throw std::invalid_argument("MonotoneComponent: the multi-index set contains a repeated term.");
            tn[cur].kTerm[k] = t;
        }
        // DFS pre-order, children in increasing (dim, order).
        std::vector<int> order;
        std::vector<int> stack{0};
        while (!stack.empty()) {
            int n = stack.back();
            stack.pop_back();
            order.push_back(n);
            for (auto it = tn[n].children.rbegin(); it != tn[n].children.rend(); ++it) stack.push_back(it->second);
        }
        nNodes = (int)order.size();
        std::vector<int> slotOf(tn.size(), -1), nkOf(tn.size(), 0), browOf(tn.size(), 0);
        for (int n : order) {
            const TNode& t = tn[n];
            if (t.depth > kMaxDepth) throw std::invalid_argument("MonotoneComponent: too many nonzero factors in a term.");
            maxDepth = std::max(maxDepth, t.depth);
            int nk = t.kTerm.empty() ? 0 : t.kTerm.rbegin()->first + 1;
            int brow = (t.depth > 0) ? rowOff[t.dim] + t.order - 1 : 0;
            int slot = (int)slotTerm.size();
            for (int k = 0; k < nk; ++k) {
                auto it = t.kTerm.find(k);
                slotTerm.push_back(it == t.kTerm.end() ? -1 : it->second);
            }
            slotOf[n] = slot;
            nkOf[n] = nk;
            browOf[n] = brow;
            nodeA.push_back((uint32_t)t.depth | ((uint32_t)nk << 5) | ((uint32_t)t.dim << 10) | ((uint32_t)brow << 18));
            nodeSlot.push_back((uint32_t)slot);
        }
        nSlots = (int)slotTerm.size();
        if (nSlots >= (1 << 22)) throw std::invalid_argument("MonotoneComponent: too many terms.");
        // Nodes carrying terms, grouped by (depth, nk) for uniform warps in the reduction.
        std::vector<int> cn;
        for (int n : order)
            if (nkOf[n] > 0) cn.push_back(n);
        std::stable_sort(cn.begin(), cn.end(), [&](int a, int b) {
            if (tn[a].depth != tn[b].depth) return tn[a].depth < tn[b].depth;
            return nkOf[a] < nkOf[b];
        });
        nCNodes = (int)cn.size();
        {
            std::vector<int> cOf(tn.size(), -1);
            for (int j = 0; j < nCNodes; ++j) cOf[cn[j]] = j;
            for (int n : order) nodeCIdx.push_back(cOf[n]);
        }
        nodeCRows.assign((size_t)nCNodes * kMaxDepth, 0);
        double opsA = 0, opsC = 0;
        for (int j = 0; j < nCNodes; ++j) {
            int n = cn[j];
            nodeC.push_back((uint32_t)tn[n].depth | ((uint32_t)nkOf[n] << 5) | ((uint32_t)slotOf[n] << 10));
            std::vector<int> path;
            for (int q = n; q != 0; q = tn[q].parent) path.push_back(browOf[q]);
            std::reverse(path.begin(), path.end());
            for (size_t q = 0; q < path.size(); ++q) nodeCRows[(size_t)j * kMaxDepth + q] = (uint16_t)path[q];
            opsC += std::max(tn[n].depth - 1, 0) + nkOf[n];
        }
        for (int n : order) opsA += (tn[n].depth > 0 ? 1 : 0) + nkOf[n];
        weight = opsA + opsC + 3.0 * nB + 60.0;
        cSegs = nCNodes < 1024 ? 4 : 1;
        dNodeA = toDevice(nodeA);
        dNodeSlot = toDevice(nodeSlot);
        dNodeC = toDevice(nodeC);
        dNodeCRows = toDevice(nodeCRows);
        dSlotTerm = toDevice(slotTerm);
        dLeadDeg = toDevice(leadDeg);
        dRowOff = toDevice(rowOff);
        dNodeCIdx = toDevice(nodeCIdx);
        reserveNoAllocScratch();
    }
    ~ComponentProgram() {
        cudaFree(dNodeA);
        cudaFree(dNodeSlot);
        cudaFree(dNodeC);
        cudaFree(dNodeCRows);
        cudaFree(dSlotTerm);
        cudaFree(dLeadDeg);
        cudaFree(dRowOff);
        cudaFree(dNodeCIdx);
        cudaFree(dSigC);
        cudaFree(dSigW);
        cudaFree(dSigWt);
        cudaFree(dSigStart);
    }
};

// Records the message returned by mpgb_last_error() on this thread.
void setLastError(const std::string& msg);

// Clenshaw-Curtis points and weights on [-1, 1], as
// ClenshawCurtisQuadrature::GetRule computes them (Quadrature.h:212-258).
void ccRule(unsigned numPts, double* wts, double* pts);

}  // namespace mpgb

// Handle behind the C ABI's opaque mpgb_map.
struct mpgb_map {
    std::shared_ptr<mpgb::ConditionalMapBase> obj;
};
