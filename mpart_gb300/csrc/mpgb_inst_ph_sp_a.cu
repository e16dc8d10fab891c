// Explicit instantiations of the fused and inverse kernels.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchFusedP<kBasisProbHermite, kPosSoftPlus, 1>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosSoftPlus, 1>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosSoftPlus, 2>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosSoftPlus, 2>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosSoftPlus, 3>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosSoftPlus, 3>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisProbHermite, kPosSoftPlus, 4>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisProbHermite, kPosSoftPlus, 4>(const InverseParams&, int, cudaStream_t);

}  // namespace mpgb
