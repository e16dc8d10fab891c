// Explicit instantiations of the sigmoid-expansion fused and inverse kernels.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 1>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 1>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 2>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 2>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 3>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 3>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 4>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 4>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 5>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 5>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 6>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 6>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 8>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 8>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosExp, 12>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosExp, 12>(const InverseParams&, int, cudaStream_t);

}  // namespace mpgb
