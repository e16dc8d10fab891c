// Host-callable launchers of the kernels in mpgb_kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include "mpgb_types.h"

namespace mpgb {

// Smallest instantiated last-coordinate order >= p, or -1.
int instantiatedPmax(int p);

size_t fusedSmemBytes(int tpb, int dmax, int nBmax, int depthMax, int pmax, bool input);

cudaError_t launchFused(int basis, int pos, int pmax, const FusedParams& prm, int nItems, int needJ, int needE,
                        cudaStream_t stream);
cudaError_t launchInverse(int basis, int pos, int pmax, const InverseParams& prm, int nBlocks, cudaStream_t stream);
// Batch of maps: one persistent launch over prm.items (forward, log-det and
// reduced coefficient adjoint; point data in prm.ioTable).  Components of
// last-coordinate order p run the body of order class batchOrderClass(p)
// (2, 4, 6 or 8; -1 above 8); pmaxClass is the largest class in the batch.
int batchOrderClass(int p);
cudaError_t launchBatch(int basis, int pos, const FusedParams& prm, int nItems, int pmaxClass, int* counter,
                        cudaStream_t stream);
cudaError_t launchGather(const int32_t* slotGlobalTerm, int nSlots, const double* coeffs, double* cm,
                         cudaStream_t stream);
cudaError_t launchReduceRows(const double* part, const long long* rowBase, int nRows, int nTerms, double scale,
                             double* out, int accumulate, cudaStream_t stream);
cudaError_t launchSumLoss(const double* lossPart, const int* slots, int n, double scale, double* out,
                          cudaStream_t stream);
// All per-component reductions of a KL step (descs: device array of nComps);
// loss may be null (gradient rows only).
cudaError_t launchKLReduce(const double* part, const long long* rowBase, const KLReduceDesc* descs, int nComps,
                           int maxTerms, double* grad, const double* lossPart, const int* lossSlots, double lossScale,
                           double* loss, cudaStream_t stream);
// Stable counting sort of points by |x_D|: perm[j] = index of the j-th point.
size_t sortScratchInts(long long N);
// nSeg independent sorts in one launch set: keys of segment k at keys + k *
// keySeg, its permutation at perm + k * permSeg; hist holds nSeg *
// sortScratchInts(N) ints.
cudaError_t launchSortByLastSegments(const double* keys, long long stride, long long keySeg, int nSeg, long long N,
                                     int* hist, int* perm, long long permSeg, cudaStream_t stream);
cudaError_t launchSortByLast(const double* xd, long long stride, long long N, int* hist, int* perm,
                             cudaStream_t stream);
cudaError_t launchDfmaPeak(double* out, int blocks, int threads, int iters, cudaStream_t stream);
// Sigmoid1d basis (c.sig* fields, device arrays) at n points x[i * stride]:
// out / d1 / d2 are (maxOrder + 1) x n, row stride n; d1, d2 may be null.
cudaError_t launchSigmoidEval(const CompDesc& c, int maxOrder, const double* x, long long n, long long stride,
                              double* out, double* d1, double* d2, cudaStream_t stream);
// Loss and gradient of the standard-normal reverse KL from dense outputs:
// T, ld (N), dT = dT/dc scaled by T, dL = dlogdet/dc (nTerms x N, row-major).
// Per term j of one component, mean_i (dT[j,i] - dL[j,i])^2 into out[j].
cudaError_t launchDenseKLSquares(const double* dT, const double* dL, int nTerms, long long N, double* out,
                                 cudaStream_t stream);
cudaError_t launchDenseKLReduce(const double* T, const double* ld, const double* dT, const double* dL, int nTerms,
                                long long N, double* loss, double* grad, cudaStream_t stream);

// Count of kernels this library has launched since it was loaded (all
// threads).  Every launch site calls countLaunches after reading its launch
// error; launches into a stream that is being captured are not counted, and
// a graph replay counts the kernel nodes of the graph.
void countLaunches(cudaStream_t stream, long long n);
long long launchCount();

}  // namespace mpgb
