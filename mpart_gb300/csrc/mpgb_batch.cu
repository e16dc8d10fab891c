// Batch of independent maps (uneven dimensions, orders and point counts):
// forward, log-determinant and reduced coefficient adjoint of every map in
// one persistent launch.
//
// The reference evaluates maps one at a time, each through its own Kokkos
// launches (MParT/ConditionalMapBase.h, MParT/MonotoneComponent.h); many small
// maps then leave most of the device idle.  Here every component of every map
// is cut into work items (strided tile sets of its points, sorted by |x_D|
// within the component), all items go into one queue ordered by estimated
// cost, and a persistent kernel drains the queue.  The number of tiles per
// item is chosen per (dimension, order) bucket, and the block size per batch,
// by MapBatch::Autotune, which times the candidates on the caller's data.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "mpgb_launch.h"
#include "mpgb_program.h"

namespace mpgb {
namespace {

// Grow-only device buffer (freed after a device synchronisation).
struct Buf {
    void* p = nullptr;
    size_t n = 0;
    void ensure(size_t bytes) {
        if (bytes <= n) return;
        if (p) {
            MPGB_CUDA(cudaDeviceSynchronize());
            cudaFree(p);
            p = nullptr;
            n = 0;
        }
        MPGB_CUDA(cudaMalloc(&p, bytes));
        n = bytes;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    ~Buf() {
        if (p) cudaFree(p);
    }
};

// ---------------------------------------------------------------------------
// Segmented stable counting sort by |x_D| (the single-map sort, one segment
// per component): chunks of 1024 points, 256 buckets of width 1/32.
// ---------------------------------------------------------------------------
constexpr int kBuckets = 256;
constexpr int kChunk = 1024;

struct SortSeg {
    const double* xd;
    long long stride;
    long long N;
    int* perm;
    int chunk0, nChunks;
};

__device__ __forceinline__ int bucketOf(double x) { return sortBucket(x); }

__global__ void segHistKernel(const SortSeg* segs, const int* chunkSeg, int* hist) {
    __shared__ int h[kBuckets];
    const SortSeg sg = segs[chunkSeg[blockIdx.x]];
    for (int t = threadIdx.x; t < kBuckets; t += blockDim.x) h[t] = 0;
    __syncthreads();
    const long long base = (long long)(blockIdx.x - sg.chunk0) * kChunk;
    for (int j = threadIdx.x; j < kChunk; j += blockDim.x) {
        const long long i = base + j;
        if (i < sg.N) atomicAdd(&h[bucketOf(sg.xd[i * sg.stride])], 1);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kBuckets; t += blockDim.x) hist[(long long)blockIdx.x * kBuckets + t] = h[t];
}

// One block of kBuckets threads per segment.
__global__ void segScanKernel(const SortSeg* segs, int* hist) {
    __shared__ int tot[kBuckets];
    const SortSeg sg = segs[blockIdx.x];
    const int b = threadIdx.x;
    int s = 0;
    for (int k = 0; k < sg.nChunks; ++k) s += hist[(long long)(sg.chunk0 + k) * kBuckets + b];
    tot[b] = s;
    __syncthreads();
    if (b == 0) {
        int run = 0;
        for (int q = 0; q < kBuckets; ++q) {
            const int v = tot[q];
            tot[q] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = tot[b];
    for (int k = 0; k < sg.nChunks; ++k) {
        int* h = &hist[(long long)(sg.chunk0 + k) * kBuckets + b];
        const int v = *h;
        *h = run;
        run += v;
    }
}

// One warp per chunk; chunk order kept within each bucket.
__global__ void segScatterKernel(const SortSeg* segs, const int* chunkSeg, const int* off) {
    __shared__ int cnt[kBuckets];
    const SortSeg sg = segs[chunkSeg[blockIdx.x]];
    const int lane = threadIdx.x;
    for (int t = lane; t < kBuckets; t += 32) cnt[t] = 0;
    __syncwarp();
    const long long base = (long long)(blockIdx.x - sg.chunk0) * kChunk;
    const unsigned lt = (1u << lane) - 1u;
    for (int c = 0; c < kChunk / 32; ++c) {
        const long long i = base + c * 32 + lane;
        const bool active = i < sg.N;
        const int key = active ? bucketOf(sg.xd[i * sg.stride]) : kBuckets + lane;
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        const int rank = __popc(grp & lt);
        int slot = 0;
        if (active) slot = cnt[key];
        __syncwarp();
        if (active) {
            sg.perm[off[(long long)blockIdx.x * kBuckets + key] + slot + rank] = (int)i;
            if (rank == 0) cnt[key] = slot + __popc(grp);
        }
        __syncwarp();
    }
}

// Coefficients of every component into the gathered slot table.
struct GatherSeg {
    const double* src;
    const int32_t* slotTerm;
    int off, nSlots;
};

__global__ void gatherSegKernel(const GatherSeg* g, double* cm) {
    const GatherSeg s = g[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.nSlots) return;
    const int t = s.slotTerm[j];
    cm[s.off + j] = t >= 0 ? s.src[t] : 0.0;
}

// Fixed-order reduction of each component's partial rows (the single-map
// reduction: 8 strided groups, then the groups in order).
struct ReduceSeg {
    long long rowOff;  // first entry of the component in rowBase
    int nRows, nTerms;
    double* out;
};

__global__ void reduceSegKernel(const double* part, const long long* rowBase, const ReduceSeg* segs) {
    __shared__ double red[8][33];
    const ReduceSeg sg = segs[blockIdx.y];
    const int t = blockIdx.x * 32 + threadIdx.x;
    const int g = threadIdx.y;
    double s = 0.0;
    if (t < sg.nTerms)
        for (int r = g; r < sg.nRows; r += 8) s += part[rowBase[sg.rowOff + r] + t];
    red[g][threadIdx.x] = s;
    __syncthreads();
    if (g == 0 && t < sg.nTerms) {
        double v = 0.0;
        for (int q = 0; q < 8; ++q) v += red[q][threadIdx.x];
        sg.out[t] = v;
    }
}

// Log-determinant of each map: its components' rows summed in component order.
struct LogdetSeg {
    const double* rows;
    int nComps;
    long long N;
    double* out;
    long long stride;
};

__global__ void logdetSegKernel(const LogdetSeg* segs) {
    const LogdetSeg sg = segs[blockIdx.y];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sg.N) return;
    double s = 0.0;
    for (int r = 0; r < sg.nComps; ++r) s += sg.rows[(long long)r * sg.N + i];
    sg.out[i * sg.stride] = s;
}

// Batch arguments are used in place: each must be device (or managed) memory.
void requireDevice(const void* p, const char* what, int map) {
    if (!p) return;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        a.type = cudaMemoryTypeUnregistered;
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) {
        std::ostringstream os;
        os << "MapBatch: " << what << " of map " << map << " is not device memory.";
        throw std::invalid_argument(os.str());
    }
}

template <class T>
void upload(Buf& b, const std::vector<T>& v, cudaStream_t s) {
    b.ensure(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!v.empty()) MPGB_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

// ---------------------------------------------------------------------------
// MapBatch
// ---------------------------------------------------------------------------
struct BatchComp {
    int map, part;
    const ComponentProgram* prog;
    int slotOffset;
};

class MapBatch {
public:
    explicit MapBatch(std::vector<std::shared_ptr<ConditionalMapBase>> const& maps) : keep_(maps) {
        if (maps.empty()) throw std::invalid_argument("MapBatch: no maps.");
        for (auto& m : maps) {
            auto* mm = dynamic_cast<MonotoneMapBase*>(m.get());
            if (!mm) throw std::invalid_argument("MapBatch: maps must be monotone components or triangular maps.");
            for (auto& pt : mm->Parts())
                if (pt.prog->kind != 0)
                    throw std::invalid_argument("MapBatch: sigmoid expansions are not provided for batches.");
            maps_.push_back(mm);
        }
        const MapOptions& a = maps_[0]->Options();
        for (auto* m : maps_) {
            const MapOptions& b = m->Options();
            if (a.basisType != b.basisType || a.posFuncType != b.posFuncType || a.quadAbsTol != b.quadAbsTol ||
                a.quadRelTol != b.quadRelTol || a.quadMaxSub != b.quadMaxSub || a.quadMinSub != b.quadMinSub ||
                a.quadPts != b.quadPts || a.basisNorm != b.basisNorm || a.nugget != b.nugget)
                throw std::invalid_argument("MapBatch: maps must share basis, rectifier and quadrature options.");
        }
        opts_ = a;
        if (!opts_.contDeriv)
            throw std::invalid_argument("MapBatch: contDeriv = false (discrete derivative) is not provided for batches.");
        basis_ = opts_.basisType == BasisTypes::HermiteFunctions ? kBasisHermiteFunctions : kBasisProbHermite;
        pos_ = opts_.posFuncType == PosFuncTypes::Exp ? kPosExp : kPosSoftPlus;
        buildLaunchConstants(opts_, quad_, bc_);
        int slot = 0;
        for (size_t m = 0; m < maps_.size(); ++m) {
            const auto& parts = maps_[m]->Parts();
            for (size_t c = 0; c < parts.size(); ++c) {
                const ComponentProgram* pg = parts[c].prog.get();
                if (batchOrderClass(pg->P) < 0)
                    throw std::invalid_argument("MapBatch: last-coordinate orders above 8 are not supported.");
                comps_.push_back({(int)m, (int)c, pg, slot});
                slot += pg->nSlots;
                dmax_ = std::max(dmax_, pg->D);
                nBmax_ = std::max(nBmax_, pg->nB);
                depthMax_ = std::max(depthMax_, pg->maxDepth);
                pclass_ = std::max(pclass_, batchOrderClass(pg->P));
                if (pg->nSlots + pg->nNodes <= kStageCap) stageNeed_ = std::max(stageNeed_, pg->nSlots + pg->nNodes);
            }
        }
        totalSlots_ = slot;
        if (comps_.size() > 65535 || maps_.size() > 65535)
            throw std::invalid_argument("MapBatch: at most 65535 maps and 65535 components in all.");
        std::vector<CompDesc> cd;
        for (auto& bc : comps_) {
            const ComponentProgram& p = *bc.prog;
            const auto& part = maps_[bc.map]->Parts()[bc.part];
            CompDesc c{};
            c.D = p.D; c.P = p.P; c.nB = p.nB; c.nNodes = p.nNodes; c.nSlots = p.nSlots; c.nCNodes = p.nCNodes;
            c.maxDepth = p.maxDepth; c.numTerms = p.numTerms; c.outRow = (int)part.outRow;
            c.coeffOffset = (int)part.mapCoeffOffset; c.slotOffset = bc.slotOffset; c.cSegs = p.cSegs;
            c.nodeA = p.dNodeA; c.nodeSlot = p.dNodeSlot; c.nodeC = p.dNodeC; c.nodeCRows = p.dNodeCRows;
            c.slotTerm = p.dSlotTerm; c.leadDeg = p.dLeadDeg; c.rowOff = p.dRowOff;
            cd.push_back(c);
        }
        compDesc_.ensure(cd.size() * sizeof(CompDesc));
        MPGB_CUDA(cudaMemcpy(compDesc_.p, cd.data(), cd.size() * sizeof(CompDesc), cudaMemcpyHostToDevice));
        status_.ensure(sizeof(int) * 2);
        MPGB_CUDA(cudaMemset(status_.p, 0, sizeof(int) * 2));
        int dev = 0;
        MPGB_CUDA(cudaGetDevice(&dev));
        MPGB_CUDA(cudaDeviceGetAttribute(&numSMs_, cudaDevAttrMultiProcessorCount, dev));
        MPGB_CUDA(cudaDeviceGetAttribute(&smemPerSM_, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    }

    int NumMaps() const { return (int)maps_.size(); }
    int NumComponents() const { return (int)comps_.size(); }
    int Tpb() const { return tpb_; }
    // Tiles (of tpb points) per work item for a component of input dimension d
    // and last-coordinate order p (default before tuning: 4).
    int TilesPerItem(int d, int p) const {
        auto it = tiles_.find({d, p});
        return it == tiles_.end() ? kDefaultTiles : it->second;
    }
    std::vector<std::pair<std::pair<int, int>, int>> Buckets() const {
        std::map<std::pair<int, int>, int> b;
        for (auto& c : comps_) b[{c.prog->D, c.prog->P}] = TilesPerItem(c.prog->D, c.prog->P);
        return {b.begin(), b.end()};
    }
    void SetTuning(int tpb, std::map<std::pair<int, int>, int> const& tiles) {
        if (tpb != 64 && tpb != 128) throw std::invalid_argument("MapBatch: block size must be 64 or 128.");
        for (auto& kv : tiles)
            if (kv.second < 1) throw std::invalid_argument("MapBatch: tiles per item must be positive.");
        tpb_ = tpb;
        tiles_ = tiles;
    }

    // pts[m]: inputDim_m x N_m; sens[m]: outputDim_m x N_m (or empty: no
    // value term); outEval[m], outLogDet[m] may be empty; coeffGrad[m] may be
    // null.  coeffGrad[m] receives sum_i [sens dT/dc + lsensScale dlogdet/dc].
    // All pointers are device pointers.
    void FusedForwardAdjoint(const StridedMatrix* pts, const StridedMatrix* sens, double lsensScale,
                             const StridedMatrix* outEval, const StridedMatrix* outLogDet, double* const* coeffGrad,
                             cudaStream_t s) {
        bool anyEval = false;
        for (size_t m = 0; m < maps_.size(); ++m) anyEval |= !outEval[m].empty();
        if (maps_[0]->Options().nugget != 0.0 && anyEval) {
            // Evaluate integrates without the nugget (MonotoneComponent.h:290),
            // the coefficient adjoint with it: the values come from each map's
            // Evaluate after the batch launch.
            std::vector<StridedMatrix> none(maps_.size());
            stage(pts, sens, lsensScale, none.data(), outLogDet, coeffGrad, s);
            runKernel(items_, s);
            finishOutputs(s);
            checkStatus(s);
            for (size_t m = 0; m < maps_.size(); ++m)
                if (!outEval[m].empty()) maps_[m]->EvaluateImpl(pts[m], outEval[m], s);
            return;
        }
        stage(pts, sens, lsensScale, outEval, outLogDet, coeffGrad, s);
        runKernel(items_, s);
        finishOutputs(s);
        checkStatus(s);
    }

    // Times the candidates on these inputs and keeps the fastest: per block
    // size, each (dimension, order) bucket's tiles per item by timing a launch
    // of that bucket's items alone; then whole calls (tables, sort, launch and
    // the gradient reduction, best of at least 3) of the starting tuning and
    // of the tuned set per block size; then, on whole calls, halving and
    // doubling the tiles of the four buckets with the most work.  Returns the
    // ms of the chosen one.
    double Autotune(const StridedMatrix* pts, const StridedMatrix* sens, double lsensScale, int reps,
                    cudaStream_t s) {
        reps = std::max(1, reps);
        const int tilesC[] = {1, 2, 4, 8, 16};
        std::vector<StridedMatrix> none(maps_.size());
        std::vector<double*> noGrad(maps_.size(), nullptr);
        // The tuning in force is a candidate too: the result is never slower
        // (as timed) than the starting point.
        std::map<std::pair<int, int>, int> bestTiles;
        for (auto& b : Buckets()) bestTiles[b.first] = b.second;
        int bestTpb = tpb_;
        const int callReps = std::max(reps, 3);
        double bestMs = timeCall(pts, sens, lsensScale, callReps, s);
        for (int tpb : {64, 128}) {
            std::map<std::pair<int, int>, int> tiles;
            for (auto& b : Buckets()) tiles[b.first] = kDefaultTiles;
            SetTuning(tpb, tiles);
            for (auto& b : Buckets()) {
                double best = 1e300;
                int arg = kDefaultTiles;
                for (int t : tilesC) {
                    tiles[b.first] = t;
                    SetTuning(tpb, tiles);
                    stage(pts, sens, lsensScale, none.data(), none.data(), noGrad.data(), s);
                    std::vector<WorkItem> sub;
                    for (size_t k = 0; k < items_.size(); ++k) {
                        const auto& c = comps_[items_[k].c0];
                        if (c.prog->D == b.first.first && c.prog->P == b.first.second) sub.push_back(items_[k]);
                    }
                    const double ms = timeKernel(sub, reps, s);
                    if (ms < best) { best = ms; arg = t; }
                }
                tiles[b.first] = arg;
            }
            SetTuning(tpb, tiles);
            const double ms = timeCall(pts, sens, lsensScale, callReps, s);
            if (ms < bestMs) { bestMs = ms; bestTpb = tpb; bestTiles = tiles; }
        }
        // Whole-call refinement: the persistent launch's length is set by how
        // its largest items end, which timing a bucket alone does not see.
        // For the buckets that carry the most work (estimated cost x tiles),
        // try other tile counts one bucket at a time on complete calls and
        // keep each change that makes the call faster by more than 0.5 %.
        SetTuning(bestTpb, bestTiles);
        {
            std::map<std::pair<int, int>, double> work;
            for (auto& c : comps_) work[{c.prog->D, c.prog->P}] += c.prog->weight * (double)pts[c.map].cols;
            std::vector<std::pair<double, std::pair<int, int>>> order;
            for (auto& w : work) order.push_back({-w.second, w.first});
            std::sort(order.begin(), order.end());
            const int kRefineBuckets = 4;
            for (int q = 0; q < (int)order.size() && q < kRefineBuckets; ++q) {
                const auto key = order[q].second;
                const int cur = bestTiles[key];
                for (int t : {std::max(1, cur / 2), cur * 2}) {
                    if (t == cur) continue;
                    auto trial = bestTiles;
                    trial[key] = t;
                    SetTuning(bestTpb, trial);
                    const double ms = timeCall(pts, sens, lsensScale, callReps, s);
                    if (ms < 0.995 * bestMs) { bestMs = ms; bestTiles = trial; }
                }
                SetTuning(bestTpb, bestTiles);
            }
        }
        SetTuning(bestTpb, bestTiles);
        checkStatus(s);
        return bestMs;
    }

private:
    static constexpr int kDefaultTiles = 4;

    // Tables, sort and coefficient gather for one call; builds items_.
    void stage(const StridedMatrix* pts, const StridedMatrix* sens, double lsensScale, const StridedMatrix* outEval,
               const StridedMatrix* outLogDet, double* const* coeffGrad, cudaStream_t s) {
        const int nM = (int)maps_.size(), nC = (int)comps_.size();
        std::vector<long long> N(nM);
        for (int m = 0; m < nM; ++m) {
            const MonotoneMapBase& mp = *maps_[m];
            mp.CheckCoefficients("MapBatch");
            if (pts[m].rows != mp.inputDim) {
                std::ostringstream os;
                os << "MapBatch: pts of map " << m << " has " << pts[m].rows << " rows, expected " << mp.inputDim << ".";
                throw std::invalid_argument(os.str());
            }
            N[m] = pts[m].cols;
            if (N[m] > 0 && !pts[m].data) throw std::invalid_argument("MapBatch: pts without data.");
            if (!sens[m].empty() && (sens[m].rows != mp.outputDim || sens[m].cols != N[m]))
                throw std::invalid_argument("MapBatch: sens must be outputDim x N for every map.");
            if (!outEval[m].empty() && (outEval[m].rows != mp.outputDim || outEval[m].cols != N[m]))
                throw std::invalid_argument("MapBatch: out_eval must be outputDim x N for every map.");
            if (!outLogDet[m].empty() && outLogDet[m].rows * outLogDet[m].cols != N[m])
                throw std::invalid_argument("MapBatch: out_logdet must hold N values for every map.");
            if (N[m] > 0) {
                requireDevice(pts[m].data, "pts", m);
                if (!sens[m].empty()) requireDevice(sens[m].data, "sens", m);
                if (!outEval[m].empty()) requireDevice(outEval[m].data, "out_eval", m);
                if (!outLogDet[m].empty()) requireDevice(outLogDet[m].data, "out_logdet", m);
            }
            requireDevice(coeffGrad[m], "coeff_grad", m);
        }
        // Coefficient gather.
        std::vector<GatherSeg> g;
        int maxSlots = 1;
        for (auto& bc : comps_) {
            const auto& part = maps_[bc.map]->Parts()[bc.part];
            part.owner->CheckCoefficients("MapBatch");
            g.push_back({part.owner->Coeffs() + part.coeffOffset, bc.prog->dSlotTerm, bc.slotOffset, bc.prog->nSlots});
            maxSlots = std::max(maxSlots, bc.prog->nSlots);
        }
        upload(gatherBuf_, g, s);
        cm_.ensure(std::max(1, totalSlots_) * sizeof(double));
        gatherSegKernel<<<dim3((maxSlots + 255) / 256, nC), 256, 0, s>>>(gatherBuf_.as<GatherSeg>(), cm_.as<double>());
        MPGB_CUDA(cudaGetLastError());
        countLaunches(s, 1);

        // Per-component point data, log-det rows and sort segments.
        std::vector<PointIO> io(nC);
        std::vector<long long> ldOff(nC), permOff(nC);
        long long ldTot = 0, permTot = 0;
        for (int k = 0; k < nC; ++k) {
            ldOff[k] = ldTot;
            permOff[k] = permTot;
            ldTot += N[comps_[k].map];
            permTot += N[comps_[k].map];
        }
        logdetRows_.ensure(std::max<long long>(1, ldTot) * sizeof(double));
        perm_.ensure(std::max<long long>(1, permTot) * sizeof(int));
        std::vector<SortSeg> segs;
        std::vector<int> chunkSeg;
        for (int k = 0; k < nC; ++k) {
            const auto& bc = comps_[k];
            const int m = bc.map;
            PointIO& p = io[k];
            p.pts = pts[m].data; p.ptsRs = pts[m].rowStride; p.ptsCs = pts[m].colStride;
            p.N = N[m];
            p.sens = sens[m].empty() ? nullptr : sens[m].data;
            p.sensRs = sens[m].rowStride; p.sensCs = sens[m].colStride;
            p.outEval = outEval[m].empty() ? nullptr : outEval[m].data;
            p.evalRs = outEval[m].rowStride; p.evalCs = outEval[m].colStride;
            p.outLogDet = logdetRows_.as<double>() + ldOff[k];
            p.logDetStride = 1;
            p.perm = perm_.as<int>() + permOff[k];
            p.permStride = 0;
            if (N[m] > 0) {
                const int nCh = (int)((N[m] + kChunk - 1) / kChunk);
                segs.push_back({pts[m].data + (long long)(bc.prog->D - 1) * pts[m].rowStride, pts[m].colStride, N[m],
                                perm_.as<int>() + permOff[k], (int)chunkSeg.size(), nCh});
                for (int q = 0; q < nCh; ++q) chunkSeg.push_back((int)segs.size() - 1);
            }
        }
        upload(ioBuf_, io, s);
        if (!segs.empty()) {
            upload(segBuf_, segs, s);
            upload(chunkSegBuf_, chunkSeg, s);
            hist_.ensure(chunkSeg.size() * kBuckets * sizeof(int));
            segHistKernel<<<(unsigned)chunkSeg.size(), 256, 0, s>>>(segBuf_.as<SortSeg>(), chunkSegBuf_.as<int>(),
                                                                    hist_.as<int>());
            segScanKernel<<<(unsigned)segs.size(), kBuckets, 0, s>>>(segBuf_.as<SortSeg>(), hist_.as<int>());
            segScatterKernel<<<(unsigned)chunkSeg.size(), 32, 0, s>>>(segBuf_.as<SortSeg>(), chunkSegBuf_.as<int>(),
                                                                      hist_.as<int>());
            MPGB_CUDA(cudaGetLastError());
            countLaunches(s, 3);
        }

        // Work items: per component, tiles k, k + nItems, ... (the single-map
        // striding), nItems = ceil(tiles / tiles per item); queue order by
        // decreasing estimated cost.  Partial rows and the reduction order
        // follow the component's own item order.
        struct Cand { WorkItem w; double cost; int order; };
        std::vector<Cand> cand;
        std::vector<long long> rowBase;
        std::vector<ReduceSeg> red;
        long long part = 0;
        for (int k = 0; k < nC; ++k) {
            const auto& bc = comps_[k];
            const long long n = N[bc.map];
            if (n == 0) continue;
            const long long nTiles = (n + tpb_ - 1) / tpb_;
            const long long per = TilesPerItem(bc.prog->D, bc.prog->P);
            const long long nItems = (nTiles + per - 1) / per;
            const long long row0 = (long long)rowBase.size();
            for (long long t = 0; t < nItems; ++t) {
                WorkItem w{k, k + 1, (int)t, (int)((nTiles - t + nItems - 1) / nItems), part, 0, (int)nItems};
                cand.push_back({w, bc.prog->weight * w.nTiles, (int)cand.size()});
                for (int sg = 0; sg < bc.prog->cSegs; ++sg) {
                    rowBase.push_back(part);
                    part += bc.prog->numTerms;
                }
            }
            double* out = coeffGrad[bc.map];
            if (out)
                red.push_back({row0, (int)nItems * bc.prog->cSegs, bc.prog->numTerms,
                               out + maps_[bc.map]->Parts()[bc.part].mapCoeffOffset});
        }
        std::stable_sort(cand.begin(), cand.end(), [](const Cand& a, const Cand& b) { return a.cost > b.cost; });
        items_.clear();
        for (auto& c : cand) items_.push_back(c.w);
        partials_.ensure(std::max<long long>(1, part) * sizeof(double));
        upload(rowBaseBuf_, rowBase, s);
        reduce_ = red;
        // Zero-point maps: their gradients are zero.
        for (int m = 0; m < nM; ++m)
            if (N[m] == 0 && coeffGrad[m])
                MPGB_CUDA(cudaMemsetAsync(coeffGrad[m], 0, maps_[m]->numCoeffs * sizeof(double), s));
        std::vector<LogdetSeg> ld;
        maxN_ = 1;
        for (int m = 0; m < nM; ++m) {
            maxN_ = std::max(maxN_, N[m]);
            if (outLogDet[m].empty() || N[m] == 0) continue;
            int first = -1, cnt = 0;
            for (int k = 0; k < nC; ++k)
                if (comps_[k].map == m) { if (first < 0) first = k; ++cnt; }
            ld.push_back({logdetRows_.as<double>() + ldOff[first], cnt, N[m], outLogDet[m].data,
                          outLogDet[m].rows == 1 ? outLogDet[m].colStride : outLogDet[m].rowStride});
        }
        logdet_ = ld;
        lsensScale_ = lsensScale;
    }

    FusedParams params() const {
        FusedParams p{};
        p.comps = compDesc_.as<CompDesc>();
        p.cm = cm_.as<double>();
        p.N = 0;
        p.flags = kFlagEval | kFlagLogDet | kFlagCoefReduced;
        p.tpb = tpb_;
        p.lsens = nullptr;
        p.lsensScale = lsensScale_;
        p.partials = partials_.as<double>();
        p.statusWord = status_.as<int>();
        p.ioTable = ioBuf_.as<PointIO>();
        p.nugget = opts_.nugget;
        p.dmax = dmax_;
        p.nBmax = nBmax_;
        p.depthMax = depthMax_;
        p.quad = quad_;
        p.bc = bc_;
        return p;
    }

    void runKernel(const std::vector<WorkItem>& items, cudaStream_t s) {
        if (items.empty()) return;
        upload(itemBuf_, items, s);
        counter_.ensure(sizeof(int));
        MPGB_CUDA(cudaMemsetAsync(counter_.p, 0, sizeof(int), s));
        FusedParams p = params();
        p.items = itemBuf_.as<WorkItem>();
        const size_t smem = fusedSmemBytes(tpb_, dmax_, nBmax_, depthMax_, pclass_, false);
        if (smem > 227 * 1024) throw std::invalid_argument("MapBatch: components too large for the shared-memory tile.");
        // Phase A's inputs staged in shared memory for the components that fit
        // kStageCap, when that leaves the blocks per SM unchanged (the batch
        // kernel's register budget: 4 blocks for order classes up to 4, 2 above).
        {
            const size_t base = smem + 1024, with = base + (size_t)stageNeed_ * sizeof(double);
            const size_t lb = pclass_ <= 4 ? 4 : 2;
            auto blocks = [&](size_t b) { return std::min<size_t>(lb, (size_t)smemPerSM_ / b); };
            p.stageDoubles = (stageNeed_ > 0 && with <= 227 * 1024 && blocks(with) == blocks(base)) ? stageNeed_ : 0;
        }
        MPGB_CUDA(launchBatch(basis_, pos_, p, (int)items.size(), pclass_, counter_.as<int>(), s));
    }

    void finishOutputs(cudaStream_t s) {
        if (!reduce_.empty()) {
            upload(reduceBuf_, reduce_, s);
            int maxT = 1;
            for (auto& r : reduce_) maxT = std::max(maxT, r.nTerms);
            reduceSegKernel<<<dim3((maxT + 31) / 32, (unsigned)reduce_.size()), dim3(32, 8), 0, s>>>(
                partials_.as<double>(), rowBaseBuf_.as<long long>(), reduceBuf_.as<ReduceSeg>());
            MPGB_CUDA(cudaGetLastError());
            countLaunches(s, 1);
        }
        if (!logdet_.empty()) {
            upload(logdetBuf_, logdet_, s);
            logdetSegKernel<<<dim3((unsigned)((maxN_ + 255) / 256), (unsigned)logdet_.size()), 256, 0, s>>>(
                logdetBuf_.as<LogdetSeg>());
            MPGB_CUDA(cudaGetLastError());
            countLaunches(s, 1);
        }
    }

    // A whole call with the coefficient adjoint (into scratch), best of reps.
    double timeCall(const StridedMatrix* pts, const StridedMatrix* sens, double lsensScale, int reps,
                    cudaStream_t s) {
        size_t tot = 0;
        for (auto* m : maps_) tot += m->numCoeffs;
        gradScratch_.ensure(std::max<size_t>(1, tot) * sizeof(double));
        std::vector<double*> g(maps_.size());
        size_t off = 0;
        for (size_t m = 0; m < maps_.size(); ++m) {
            g[m] = gradScratch_.as<double>() + off;
            off += maps_[m]->numCoeffs;
        }
        std::vector<StridedMatrix> none(maps_.size());
        auto call = [&] {
            stage(pts, sens, lsensScale, none.data(), none.data(), g.data(), s);
            runKernel(items_, s);
            finishOutputs(s);
        };
        call();  // warm-up
        EventPair ev;
        double best = 1e300;
        for (int r = 0; r < reps; ++r) {
            MPGB_CUDA(cudaEventRecord(ev.a, s));
            call();
            MPGB_CUDA(cudaEventRecord(ev.b, s));
            MPGB_CUDA(cudaEventSynchronize(ev.b));
            best = std::min(best, (double)ev.ms());
        }
        checkStatus(s);
        return best;
    }

    double timeKernel(const std::vector<WorkItem>& items, int reps, cudaStream_t s) {
        runKernel(items, s);  // warm-up
        EventPair ev;
        double best = 1e300;
        for (int r = 0; r < reps; ++r) {
            MPGB_CUDA(cudaEventRecord(ev.a, s));
            runKernel(items, s);
            MPGB_CUDA(cudaEventRecord(ev.b, s));
            MPGB_CUDA(cudaEventSynchronize(ev.b));
            best = std::min(best, (double)ev.ms());
        }
        return best;
    }

    void checkStatus(cudaStream_t s) {
        int st = 0;
        MPGB_CUDA(cudaMemcpyAsync(&st, status_.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        MPGB_CUDA(cudaMemsetAsync(status_.p, 0, sizeof(int), s));
        MPGB_CUDA(cudaStreamSynchronize(s));
        if (st & kStatusInf) throw IntegrandError("MapBatch: MonotoneIntegrand: g(df) overflowed.");
        if (st & kStatusNaN) throw IntegrandError("MapBatch: MonotoneIntegrand: nan was encountered in g(df).");
        if (st & kStatusBudget) throw std::runtime_error("MapBatch: adaptive quadrature exceeded its interval budget.");
    }

    std::vector<std::shared_ptr<ConditionalMapBase>> keep_;
    std::vector<MonotoneMapBase*> maps_;
    std::vector<BatchComp> comps_;
    MapOptions opts_;
    int basis_ = 0, pos_ = 0;
    QuadParams quad_{};
    BasisConsts bc_{};
    int dmax_ = 1, nBmax_ = 0, depthMax_ = 0, pclass_ = 2, totalSlots_ = 0, numSMs_ = 1, stageNeed_ = 0,
        smemPerSM_ = 0;
    int tpb_ = 128;
    std::map<std::pair<int, int>, int> tiles_;
    Buf gradScratch_;  // autotuning: coefficient adjoints of timed calls
    std::vector<WorkItem> items_;
    std::vector<ReduceSeg> reduce_;
    std::vector<LogdetSeg> logdet_;
    long long maxN_ = 1;
    double lsensScale_ = 0.0;
    Buf compDesc_, status_, gatherBuf_, cm_, logdetRows_, perm_, ioBuf_, segBuf_, chunkSegBuf_, hist_, partials_,
        rowBaseBuf_, itemBuf_, counter_, reduceBuf_, logdetBuf_;
};

}  // namespace mpgb

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct mpgb_batch {
    mpgb::MapBatch b;
    explicit mpgb_batch(std::vector<std::shared_ptr<mpgb::ConditionalMapBase>> const& m) : b(m) {}
};

namespace {
template <class F>
int batchGuard(F&& f) {
    try {
        f();
        return MPGB_OK;
    } catch (mpgb::IntegrandError const& e) {
        mpgb::setLastError(e.what());
        return MPGB_ERR_INTEGRAND;
    } catch (mpgb::CudaError const& e) {
        mpgb::setLastError(e.what());
        return MPGB_ERR_CUDA;
    } catch (std::invalid_argument const& e) {
        mpgb::setLastError(e.what());
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        mpgb::setLastError(e.what());
        return MPGB_ERR_RUNTIME;
    }
}

mpgb::StridedMatrix toMat(const mpgb_matrix* a, int i) {
    if (!a) return mpgb::StridedMatrix();
    const mpgb_matrix& m = a[i];
    return mpgb::StridedMatrix(m.data, m.rows, m.cols, m.row_stride, m.col_stride);
}

std::vector<mpgb::StridedMatrix> mats(const mpgb_matrix* a, int n) {
    std::vector<mpgb::StridedMatrix> v;
    for (int i = 0; i < n; ++i) v.push_back(toMat(a, i));
    return v;
}
}  // namespace

extern "C" {

int mpgb_batch_create(mpgb_map* const* maps, int n, mpgb_batch** out) {
    return batchGuard([&] {
        if (!maps || n <= 0 || !out) throw std::invalid_argument("mpgb_batch_create: no maps.");
        std::vector<std::shared_ptr<mpgb::ConditionalMapBase>> v;
        for (int i = 0; i < n; ++i) {
            if (!maps[i] || !maps[i]->obj) throw std::invalid_argument("mpgb_batch_create: null map handle.");
            v.push_back(maps[i]->obj);
        }
        *out = new mpgb_batch(v);
    });
}

int mpgb_batch_destroy(mpgb_batch* b) {
    delete b;
    return MPGB_OK;
}

int mpgb_batch_fwd_adj(mpgb_batch* b, const mpgb_matrix* pts, const mpgb_matrix* sens, double logdet_sens_scale,
                       const mpgb_matrix* out_eval, const mpgb_matrix* out_logdet, double* const* coeff_grad,
                       void* stream) {
    return batchGuard([&] {
        if (!b || !pts) throw std::invalid_argument("mpgb_batch_fwd_adj: null argument.");
        const int n = b->b.NumMaps();
        auto P = mats(pts, n), S = mats(sens, n), E = mats(out_eval, n), L = mats(out_logdet, n);
        std::vector<double*> G(n, nullptr);
        if (coeff_grad)
            for (int i = 0; i < n; ++i) G[i] = coeff_grad[i];
        b->b.FusedForwardAdjoint(P.data(), S.data(), logdet_sens_scale, E.data(), L.data(), G.data(),
                                 (cudaStream_t)stream);
    });
}

int mpgb_batch_autotune(mpgb_batch* b, const mpgb_matrix* pts, const mpgb_matrix* sens, double logdet_sens_scale,
                        int reps, double* best_ms, void* stream) {
    return batchGuard([&] {
        if (!b || !pts) throw std::invalid_argument("mpgb_batch_autotune: null argument.");
        const int n = b->b.NumMaps();
        auto P = mats(pts, n), S = mats(sens, n);
        const double ms = b->b.Autotune(P.data(), S.data(), logdet_sens_scale, reps, (cudaStream_t)stream);
        if (best_ms) *best_ms = ms;
    });
}

int mpgb_batch_tuning(mpgb_batch* b, int* tpb, int max_buckets, int* n_buckets, int* dims, int* orders, int* tiles) {
    return batchGuard([&] {
        if (!b) throw std::invalid_argument("mpgb_batch_tuning: null batch.");
        auto bk = b->b.Buckets();
        if (tpb) *tpb = b->b.Tpb();
        if (n_buckets) *n_buckets = (int)bk.size();
        for (int i = 0; i < (int)bk.size() && i < max_buckets; ++i) {
            if (dims) dims[i] = bk[i].first.first;
            if (orders) orders[i] = bk[i].first.second;
            if (tiles) tiles[i] = bk[i].second;
        }
    });
}

int mpgb_batch_set_tuning(mpgb_batch* b, int tpb, int n_buckets, const int* dims, const int* orders,
                          const int* tiles) {
    return batchGuard([&] {
        if (!b) throw std::invalid_argument("mpgb_batch_set_tuning: null batch.");
        std::map<std::pair<int, int>, int> t;
        for (int i = 0; i < n_buckets; ++i) t[{dims[i], orders[i]}] = tiles[i];
        b->b.SetTuning(tpb, t);
    });
}

}  // extern "C"
