// Launch-time structures shared by the host planner and the kernels.
#pragma once
#include <stdint.h>
#include "mpgb_device.cuh"

namespace mpgb {

// One monotone component as the kernels see it.  Device arrays are built by
// the host planner from the component's multi-index set (see Program in
// mpgb_host.cu) and live as long as the component object.
struct CompDesc {
    int D;          // input dimension of the component
    int P;          // largest order in the last coordinate
    int nB;         // rows of the per-point basis table (orders >= 1 of the leading coordinates)
    int nNodes;     // prefix-tree nodes (phase A / dense outputs / input gradient), DFS pre-order
    int nSlots;     // dense (node, k) coefficient slots
    int nCNodes;    // prefix nodes that carry terms (reduced coefficient adjoint), sorted by (depth, nk)
    int maxDepth;   // deepest prefix (number of nonzero leading factors)
    int numTerms;   // coefficients of this component
    int outRow;     // output row of this component in the map output
    int coeffOffset;  // offset of its block in the map coefficient vector
    int slotOffset;   // offset of its slots in the map-wide gathered coefficient table
    int cSegs;        // reduced adjoint: point segments per tile = partial rows per work item (divides the block size)
    const uint32_t* nodeA;   // [nNodes] depth | nk<<5 | dim<<10 | brow<<18
    const uint32_t* nodeSlot;  // [nNodes] first slot of the node
    const uint32_t* nodeC;   // [nCNodes] depth | nk<<5 | slot<<10
    const uint16_t* nodeCRows;  // [nCNodes * kMaxDepth] basis rows along the path
    const int32_t* slotTerm; // [nSlots] coefficient index within the component, or -1
    const int32_t* leadDeg;  // [D-1] largest order per leading coordinate
    const int32_t* rowOff;   // [D-1] first basis row of each leading coordinate
    // Sigmoid expansions (kBasisSigmoid launches): the Sigmoid1d parameters of
    // the last input (centers, widths, weights; term k >= 4 sums the entries
    // [sigStart[k-4], sigStart[k-3]) or up to sigN for the last term) and
    // whether the leading products of terms with a last-input factor pass
    // through the rectifier (RectifiedMultivariateExpansion) or not
    // (UnivariateExpansion, one input).
    const double* sigC;
    const double* sigW;
    const double* sigWt;
    const int32_t* sigStart;
    int sigN, sigNStarts;
    int rectify;
    int pad1_;
    const int32_t* nodeCIdx;  // [nNodes] index of the node in nodeC, or -1 (sigmoid rectifier cache)
};

// A block's work: tiles tile0, tile0 + tileStride, ... (nTiles of them) of
// components [c0, c1); tile t covers processing slots [t*TPB, (t+1)*TPB).
// A stride equal to the number of items of the component spreads points that
// were sorted by cost evenly over the items.
struct WorkItem {
    int c0, c1;
    int tile0, nTiles;
    long long partialBase;  // first double of this item's partial rows (cSegs rows of numTerms; reduced adjoint)
    int lossSlot;           // index into the loss partials (KL)
    int tileStride;         // distance between consecutive tiles of the item (>= 1)
    long long rcBase;       // first double of this item's rectifier cache (sigmoid expansions, reduced adjoint)
};

enum FusedFlags : int {
    kFlagEval = 1,          // write T_c(x) to outEval row outRow
    kFlagLogDet = 2,        // sum log d_D T_c over the component range into outLogDet
    kFlagCoefDenseT = 4,    // dense sens-scaled coefficient gradient of T (CoeffGradImpl)
    kFlagCoefDenseL = 8,    // dense coefficient gradient of log-det (LogDeterminantCoeffGradImpl)
    kFlagCoefReduced = 16,  // sum over points of the combined weights into partial rows
    kFlagInput = 32,        // combined input gradient into outInput (GradientImpl / LogDeterminantInputGradImpl)
    kFlagKL = 64,           // sens_c = T_c * sensScale, lsens = lsensScale, loss partials
    kFlagStatusArray = 128, // per-point status words
    // Implicit differentiation of the inverse (one component per launch, in
    // reverse output order): outInput holds the running back-substitution
    // sums acc_j = sum_{m > j} lambda_m dT_m/dx_j on entry; the launch sets
    // lambda = (sens - acc_D) / dT/dx_D, stores it in row D-1, adds
    // lambda dT/dx_j to rows j < D-1 and reduces lambda dT/dc.
    kFlagImplicit = 256,
    kFlagImplicitFirst = 512,  // with kFlagImplicit: the sums start at zero (first launch)
};

// One component's reductions at the end of a KL step: its partial rows
// [rowOff, rowOff + nRows) of rowBase into grad[outOff .. outOff + nTerms) and
// its loss partials [lossOff, lossOff + nLoss) of lossSlots into loss[comp].
struct KLReduceDesc {
    int rowOff, nRows, nTerms, outOff;
    int lossOff, nLoss, comp, pad_;
};

// Point data of one component in a batch of maps (the launch-wide fields of
// FusedParams with the same names, per component).
struct PointIO {
    const double* pts; long long ptsRs, ptsCs;
    long long N;
    const double* sens; long long sensRs, sensCs;
    double* outEval; long long evalRs, evalCs;
    double* outLogDet; long long logDetStride;
    const int* perm; long long permStride;
};

struct FusedParams {
    const CompDesc* comps;
    const WorkItem* items;
    const double* cm;       // gathered coefficients (all components)
    long long N;
    int flags;
    int tpb;
    // inputs
    const double* pts; long long ptsRs, ptsCs;
    const double* sens; long long sensRs, sensCs;   // one row per component (map output row)
    const double* lsens; long long lsensStride;     // log-det sensitivity per point (or null = lsensScale)
    double sensScale, lsensScale;
    // outputs
    double* outEval; long long evalRs, evalCs;
    double* outLogDet; long long logDetStride;
    long long logDetCompStride;  // items of one component c0 write row c0 (0: one row for all)
    double* outDense; long long denseRs, denseCs;   // numCoeffs x N
    double* outInput; long long inputRs, inputCs;   // inputDim x N
    double* partials;
    double* lossPartials;
    int* status; long long statusStride;
    int* statusWord;
    // Optional processing order: point index of slot j for component c is
    // perm[c * permStride + j] (items of one component only).
    const int* perm; long long permStride;
    const PointIO* ioTable;  // batch launches: point data per component (indexed by WorkItem::c0)
    // Sigmoid expansions with a reduced adjoint: R(Phi_m) of phase A kept for
    // the reduction, nCNodes x blockDim doubles per item at WorkItem::rcBase
    // (null: the reduction evaluates the rectifier again).
    double* rcache;
    // Optional: per point and component, the quadrature's interval count / 8
    // at costKey[c * costStride + i] (a sort key: the next call processes the
    // points in order of it).
    double* costKey; long long costStride;
    double nugget;
    int dmax, nBmax, depthMax;
    int negRows;            // kFlagImplicit: rows [0, negRows) of outInput are negated when written
    // Shared-memory staging of phase A's inputs: components with nSlots +
    // nNodes <= stageDoubles read their coefficients and prefix-tree tables
    // from a block-staged copy (0: none; the launch adds stageDoubles to the
    // block's shared memory).
    int stageDoubles;
    QuadParams quad;
    BasisConsts bc;
};

// An interval of the warp-shared adaptive quadrature (inverseWarpKernel):
// [lo, lo + 2^-level] with the integrand at its ends, or (done = 1) an
// accepted interval waiting to be summed, its fine-rule value in hA.
struct QEntry {
    double lo, hA, hB;
    int level, done;
};

struct InverseParams {
    const CompDesc* comps;
    int nComps;
    const double* cm;
    long long N;
    int tpb;
    int extra;               // inputDim - outputDim
    const double* x1; long long x1Rs, x1Cs; int x1Rows; int x1Cols;  // x1Cols == 1 broadcasts
    const double* r; long long rRs, rCs;
    double* out; long long outRs, outCs;
    int* info; long long infoStride;
    int* statusWord;
    double xtol, ytol;
    double nugget;
    int dmax, nBmax, depthMax;
    // Components [compBegin, compEnd) are solved (compEnd 0: to the last);
    // the coordinates of the components before compBegin come from out.
    int compBegin;
    // Two passes per component.  The first takes every point (in perm order
    // when perm is set) with bracketBudget doubling steps; a point that needs
    // more stops, adds one to *deferCount and writes its sort key (from a
    // root estimate) to deferKey[i].  The second (listCount set) takes the
    // *listCount points of perm, the deferred ones sorted by that key, with
    // the full kBracketIts steps.  Restarted with a larger budget a solve
    // repeats the same evaluations, so the results are those of one pass with
    // the full budget.  The second pass's grid covers N points; threads past
    // the count only take part in the warp loops.
    int bracketBudget;
    int compEnd;
    const int* perm;  // the points by increasing expected cost (taken from the end), or null
    const int* listCount;
    double* deferKey;
    int* deferCount;
    // Key pass (keyPass = 1, component compBegin): phase A of every point goes
    // to acoef (row k at acoef + k N) and a root estimate to key.  The solver
    // launches then read the a_k from acoef (when non-null).
    double* acoef;
    double* key;
    int keyPass;
    int method;  // kInverseITP (the reference's solver) or kInverseNewton
    // Queue pass (queuePass = 1, monotone components, component compBegin):
    // a persistent launch whose lanes take the points one at a time from
    // *queue (zero on entry), in perm order from the expensive end, and solve
    // each with the full bracket budget; a_k come from acoef.
    int* queue;
    int queuePass;
    // Queue pass: a point whose solve takes more than nodeBudget integrand
    // nodes, or one of whose quadratures reaches wideQuad intervals, is left
    // to the warp pass: its index goes to deferList[atomicAdd(deferCount, 1)]
    // and its solver state to deferState (nodeBudget 0: no limit).
    int nodeBudget;
    int wideQuad;
    int* deferList;
    int* drained;  // set (to 1) by the first lane that finds the queue empty; zero on entry
    // The solver state of deferred point slot k (k < deferStateCap) at
    // deferState + k * RootSolve::kSaveDoubles; the warp pass continues from
    // it (null, or a slot past the cap: it starts the solve again).
    double* deferState;
    int deferStateCap;
    // Warp pass (warpPass = 1): one group of kWarpGroup lanes per point of
    // deferList (*listCount of them, taken through *queue), the lanes sharing
    // each adaptive quadrature; stack: stackCap entries of scratch per group
    // of the grid.
    QEntry* stack;
    int stackCap;
    int warpPass;
    QuadParams quad;
    BasisConsts bc;
};

}  // namespace mpgb
