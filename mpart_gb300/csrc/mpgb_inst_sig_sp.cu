// Explicit instantiations of the sigmoid-expansion fused and inverse kernels.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 1>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 1>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 2>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 2>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 3>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 3>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 4>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 4>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 5>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 5>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 6>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 6>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 8>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 8>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisSigmoid, kPosSoftPlus, 12>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisSigmoid, kPosSoftPlus, 12>(const InverseParams&, int, cudaStream_t);

}  // namespace mpgb
