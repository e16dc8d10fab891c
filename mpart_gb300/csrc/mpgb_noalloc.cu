// Fused forward + reduced coefficient adjoint that allocates no memory.
//
// Some callers cannot allocate device memory while they run: code inside a
// custom allocator or memory pool, real-time loops that forbid allocation
// after start-up, and hosts that own the whole device heap themselves.  This
// entry point serves them.  The scratch that mpgb_fused_fwd_adj takes from
// cudaMalloc (launch tables, gathered coefficients, per-item partial sums,
// the status word) lives here in one fixed array in device global memory,
// declared below; the caller passes only inputs and outputs.
//
// Limits and sharing:
//  * the array holds kNoAllocScratchBytes (64 MiB); a call needing more is
//    rejected with MPGB_ERR_INVALID_ARGUMENT and a message giving both sizes;
//  * every GPU that loads the library holds its own copy of the array until
//    the process exits.  With CUDA's lazy module loading (the default) the
//    driver loads the module holding the array, and reserves its memory,
//    when the array's address is first looked up; that look-up is done when
//    a map is created on the device (reserveNoAllocScratch, called by every
//    monotone component's constructor), so the entry point's own calls
//    reserve nothing.  Should that look-up have failed, the first call on
//    the device makes it (and then reserves the array); make that first
//    call during start-up, before any stream capture;
//  * all calls share the array, which keeps the last call's contents, so
//    calls that overlap on the GPU (different streams, or threads) race.
#include <cmath>
#include <cstring>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mpart_gb300.h"
#include "mpgb_launch.h"
#include "mpgb_program.h"

namespace mpgb {
namespace noalloc {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;
constexpr int kTpbNA = 128;

static __device__ __align__(256) unsigned char g_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_base[kMaxDevices] = {nullptr};

// Device address of g_scratch on the current device (looked up once per device).
void* scratchBase() {
    int dev = 0;
    MPGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("no-allocation entry point: device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            std::ostringstream os;
            os << "no-allocation entry point: cudaGetSymbolAddress failed: " << cudaGetErrorString(e);
            throw CudaError(os.str());
        }
        g_base[dev] = p;
    }
    return g_base[dev];
}

}  // namespace noalloc

// Looks up (and so, under lazy module loading, reserves) the scratch array
// of the current device; called when a monotone component is created.  A
// failure is not an error here: the entry point's first call repeats the
// look-up and reports it.
void reserveNoAllocScratch() noexcept {
    try {
        noalloc::scratchBase();
    } catch (...) {
        cudaGetLastError();
    }
}

namespace noalloc {

struct GatherDesc {
    const double* src;
    const int32_t* slotTerm;
    int slotOffset;
    int nSlots;
};

__global__ void gatherNA(const GatherDesc* descs, int nComps, double* cm) {
    const int c = blockIdx.y;
    if (c >= nComps) return;
    const GatherDesc g = descs[c];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < g.nSlots; s += gridDim.x * blockDim.x) {
        const int t = g.slotTerm[s];
        cm[g.slotOffset + s] = (t >= 0) ? g.src[t] : 0.0;
    }
}

// Bump allocator over the static array (offsets only; nothing is allocated).
struct Carve {
    size_t used = 0;
    size_t take(size_t bytes) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + bytes;
        return off;
    }
};

// Device memory of the current device, or managed memory (the kernels run
// on the current device and read these pointers directly).
bool onDevice(const void* p, int dev) {
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}

void run(MonotoneMapBase& map, const mpgb_matrix& pts, const mpgb_matrix& sens, const mpgb_matrix& lsens,
         double lsensScale, const mpgb_matrix& outEval, const mpgb_matrix& outLogDet, double* coeffGrad,
         cudaStream_t stream) {
    map.CheckCoefficients("FusedForwardAdjoint (no allocation)");
    const auto& parts = map.Parts();
    const int nComps = (int)parts.size();
    const long long N = pts.cols;
    if (pts.rows != map.inputDim) throw std::invalid_argument("pts must have inputDim rows");
    if (sens.data && (sens.rows != map.outputDim || sens.cols != N))
        throw std::invalid_argument("sens must be outputDim x N");
    if (lsens.data && lsens.rows * lsens.cols != N) throw std::invalid_argument("logdet_sens must hold N values");
    if (outEval.data && (outEval.rows != map.outputDim || outEval.cols != N))
        throw std::invalid_argument("out_eval must be outputDim x N");
    if (outLogDet.data && outLogDet.rows * outLogDet.cols != N)
        throw std::invalid_argument("out_logdet must hold N values");
    if (outLogDet.data && nComps != 1)
        throw std::invalid_argument("the no-allocation entry point returns log-determinants of one-component maps only");
    int curDev = 0;
    MPGB_CUDA(cudaGetDevice(&curDev));
    if (!onDevice(pts.data, curDev) || !onDevice(sens.data, curDev) || !onDevice(lsens.data, curDev) ||
        !onDevice(outEval.data, curDev) || !onDevice(outLogDet.data, curDev) || !onDevice(coeffGrad, curDev))
        throw std::invalid_argument(
            "the no-allocation entry point takes device pointers of the current device (or managed memory) only");
    const MapOptions& o = map.Options();
    if (!o.contDeriv)
        throw std::invalid_argument("contDeriv = false (discrete derivative) is not provided without allocation.");
    for (int c = 0; c < nComps; ++c)
        if (parts[c].prog->kind != 0)
            throw std::invalid_argument("sigmoid expansions are not provided by the no-allocation entry point.");
    int dev = 0, sms = 0;
    MPGB_CUDA(cudaGetDevice(&dev));
    MPGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned char* base = (unsigned char*)scratchBase();

    // Launch tables on the host (stack / std::vector: host memory only).
    std::vector<CompDesc> comps(nComps);
    std::vector<GatherDesc> gather(nComps);
    std::vector<WorkItem> items;
    std::vector<long long> rowBase;
    std::vector<int> rowOff(nComps + 1, 0);
    int slotOff = 0, pm = 1, dmax = 1, nBmax = 0, depthMax = 0;
    const long long nTiles = (N + kTpbNA - 1) / kTpbNA;
    long long partBase = 0;
    for (int c = 0; c < nComps; ++c) {
        const ComponentProgram& p = *parts[c].prog;
        CompDesc& d = comps[c];
        d = CompDesc{};
        d.D = p.D; d.P = p.P; d.nB = p.nB; d.nNodes = p.nNodes; d.nSlots = p.nSlots; d.nCNodes = p.nCNodes;
        d.maxDepth = p.maxDepth; d.numTerms = p.numTerms; d.outRow = (int)parts[c].outRow;
        d.coeffOffset = (int)parts[c].mapCoeffOffset; d.slotOffset = slotOff; d.cSegs = p.cSegs;
        d.nodeA = p.dNodeA; d.nodeSlot = p.dNodeSlot; d.nodeC = p.dNodeC; d.nodeCRows = p.dNodeCRows;
        d.slotTerm = p.dSlotTerm; d.leadDeg = p.dLeadDeg; d.rowOff = p.dRowOff;
        parts[c].owner->CheckCoefficients("FusedForwardAdjoint (no allocation)");
        gather[c] = {parts[c].owner->Coeffs() + parts[c].coeffOffset, p.dSlotTerm, slotOff, p.nSlots};
        slotOff += p.nSlots;
        pm = std::max(pm, p.P);
        dmax = std::max(dmax, p.D);
        nBmax = std::max(nBmax, p.nB);
        depthMax = std::max(depthMax, p.maxDepth);
        const long long nItemsC = std::max<long long>(1, std::min<long long>(nTiles, (long long)sms * kFusedBlocksPerSM));
        const long long tilesPer = (nTiles + nItemsC - 1) / nItemsC;
        rowOff[c] = (int)rowBase.size();
        for (long long t = 0; t < nTiles; t += tilesPer) {
            WorkItem w{c, c + 1, (int)t, (int)std::min<long long>(tilesPer, nTiles - t), partBase, (int)items.size(), 1};
            for (int sg = 0; sg < p.cSegs; ++sg) {
                rowBase.push_back(partBase);
                partBase += p.numTerms;
            }
            items.push_back(w);
        }
    }
    rowOff[nComps] = (int)rowBase.size();
    const int pmax = instantiatedPmax(pm);
    if (pmax < 0) throw std::invalid_argument("order in the last input too large");

    Carve cv;
    const size_t oStatus = cv.take(sizeof(int));
    const size_t oComps = cv.take(comps.size() * sizeof(CompDesc));
    const size_t oGather = cv.take(gather.size() * sizeof(GatherDesc));
    const size_t oItems = cv.take(std::max<size_t>(1, items.size()) * sizeof(WorkItem));
    const size_t oRows = cv.take(std::max<size_t>(1, rowBase.size()) * sizeof(long long));
    const size_t oCm = cv.take(std::max(1, slotOff) * sizeof(double));
    const size_t oPart = cv.take(std::max<long long>(1, partBase) * sizeof(double));
    if (cv.used > kNoAllocScratchBytes) {
        std::ostringstream os;
        os << "the no-allocation entry point needs " << cv.used << " bytes of scratch for this call but holds "
           << kNoAllocScratchBytes << " bytes; use mpgb_fused_fwd_adj";
        throw std::invalid_argument(os.str());
    }
    int* dStatus = (int*)(base + oStatus);
    MPGB_CUDA(cudaMemsetAsync(dStatus, 0, sizeof(int), stream));
    MPGB_CUDA(cudaMemcpyAsync(base + oComps, comps.data(), comps.size() * sizeof(CompDesc), cudaMemcpyHostToDevice, stream));
    MPGB_CUDA(cudaMemcpyAsync(base + oGather, gather.data(), gather.size() * sizeof(GatherDesc), cudaMemcpyHostToDevice, stream));
    if (!items.empty()) {
        MPGB_CUDA(cudaMemcpyAsync(base + oItems, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, stream));
        MPGB_CUDA(cudaMemcpyAsync(base + oRows, rowBase.data(), rowBase.size() * sizeof(long long), cudaMemcpyHostToDevice, stream));
    }
    double* cm = (double*)(base + oCm);
    int maxSlots = 1;
    for (auto& g : gather) maxSlots = std::max(maxSlots, g.nSlots);
    gatherNA<<<dim3((maxSlots + 255) / 256, nComps), 256, 0, stream>>>((const GatherDesc*)(base + oGather), nComps, cm);
    MPGB_CUDA(cudaGetLastError());
    countLaunches(stream, 1);

    if (coeffGrad && N == 0) MPGB_CUDA(cudaMemsetAsync(coeffGrad, 0, map.numCoeffs * sizeof(double), stream));
    if (N > 0 && (coeffGrad || outEval.data || outLogDet.data)) {
        FusedParams p{};
        p.comps = (const CompDesc*)(base + oComps);
        p.items = (const WorkItem*)(base + oItems);
        p.cm = cm;
        p.N = N;
        p.tpb = kTpbNA;
        p.pts = pts.data; p.ptsRs = pts.row_stride; p.ptsCs = pts.col_stride;
        p.flags = 0;
        // Evaluate integrates without the nugget, the coefficient adjoint with
        // it (MonotoneComponent.h:290, :721): with a nonzero nugget and both
        // asked for, the values come from a second launch.
        const bool valuesApart = o.nugget != 0.0 && outEval.data && coeffGrad;
        if (outEval.data && !valuesApart) {
            p.flags |= kFlagEval;
            p.outEval = outEval.data; p.evalRs = outEval.row_stride; p.evalCs = outEval.col_stride;
        }
        if (outLogDet.data) {
            p.flags |= kFlagLogDet;
            p.outLogDet = outLogDet.data;
            p.logDetStride = (outLogDet.rows == 1) ? outLogDet.col_stride : outLogDet.row_stride;
        }
        int needJ = 0;
        if (coeffGrad) {
            p.flags |= kFlagCoefReduced;
            p.sens = sens.data; p.sensRs = sens.row_stride; p.sensCs = sens.col_stride;
            p.lsens = lsens.data;
            p.lsensStride = lsens.data ? ((lsens.rows == 1) ? lsens.col_stride : lsens.row_stride) : 0;
            p.lsensScale = lsensScale;
            p.partials = (double*)(base + oPart);
            needJ = sens.data ? 1 : 0;
        }
        p.statusWord = dStatus;
        p.nugget = coeffGrad ? o.nugget : 0.0;
        p.dmax = dmax; p.nBmax = nBmax; p.depthMax = depthMax;
        buildLaunchConstants(o, p.quad, p.bc);
        const size_t smem = fusedSmemBytes(p.tpb, p.dmax, p.nBmax, p.depthMax, pmax, false);
        if (smem > 227 * 1024) throw std::invalid_argument("component too large for the shared-memory tile");
        const int basis = o.basisType == BasisTypes::HermiteFunctions ? kBasisHermiteFunctions : kBasisProbHermite;
        const int pos = o.posFuncType == PosFuncTypes::Exp ? kPosExp : kPosSoftPlus;
        if (p.flags) MPGB_CUDA(launchFused(basis, pos, pmax, p, (int)items.size(), needJ, 0, stream));
        if (valuesApart) {
            FusedParams q = p;
            q.flags = kFlagEval;
            q.outEval = outEval.data; q.evalRs = outEval.row_stride; q.evalCs = outEval.col_stride;
            q.nugget = 0.0;
            MPGB_CUDA(launchFused(basis, pos, pmax, q, (int)items.size(), 0, 0, stream));
        }
        if (coeffGrad) {
            const long long* rows = (const long long*)(base + oRows);
            for (int c = 0; c < nComps; ++c)
                MPGB_CUDA(launchReduceRows(p.partials, rows + rowOff[c], rowOff[c + 1] - rowOff[c],
                                           parts[c].prog->numTerms, 1.0, coeffGrad + parts[c].mapCoeffOffset, 0,
                                           stream));
        }
    }
    int st = 0;
    MPGB_CUDA(cudaMemcpyAsync(&st, dStatus, sizeof(int), cudaMemcpyDeviceToHost, stream));
    MPGB_CUDA(cudaStreamSynchronize(stream));
    if (st & kStatusInf)
        throw IntegrandError(
            "FusedForwardAdjoint (no allocation): MonotoneIntegrand: nan was encountered in value of g(df(...)).");
    if (st & kStatusBudget)
        throw std::runtime_error("FusedForwardAdjoint (no allocation): adaptive quadrature exceeded its interval budget.");
}

}  // namespace noalloc
}  // namespace mpgb

extern "C" int mpgb_fused_fwd_adj_noalloc(mpgb_map* map, mpgb_matrix pts, mpgb_matrix sens, mpgb_matrix logdet_sens,
                                          double logdet_sens_scale, mpgb_matrix out_eval, mpgb_matrix out_logdet,
                                          double* coeff_grad, void* stream) {
    using namespace mpgb;
    try {
        if (!map || !map->obj) throw std::invalid_argument("null map handle");
        auto* m = dynamic_cast<MonotoneMapBase*>(map->obj.get());
        if (!m) throw std::invalid_argument("map is not a monotone map");
        noalloc::run(*m, pts, sens, logdet_sens, logdet_sens_scale, out_eval, out_logdet, coeff_grad,
                     (cudaStream_t)stream);
        return MPGB_OK;
    } catch (IntegrandError const& e) {
        setLastError(e.what());
        return MPGB_ERR_INTEGRAND;
    } catch (CudaError const& e) {
        setLastError(e.what());
        return MPGB_ERR_CUDA;
    } catch (std::invalid_argument const& e) {
        setLastError(e.what());
        return MPGB_ERR_INVALID_ARGUMENT;
    } catch (std::exception const& e) {
        setLastError(e.what());
        return MPGB_ERR_RUNTIME;
    }
}
