// Explicit instantiations of the fused and inverse kernels.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchFusedP<kBasisProbHermite, kPosExp, 5>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosExp, 5>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosExp, 6>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosExp, 6>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosExp, 8>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosExp, 8>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosExp, 12>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosExp, 12>(const InverseParams&, int, cudaStream_t);

}  // namespace mpgb
