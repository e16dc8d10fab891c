// Explicit instantiations of the fused and inverse kernels.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchFusedP<kBasisHermiteFunctions, kPosSoftPlus, 1>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisHermiteFunctions, kPosSoftPlus, 1>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisHermiteFunctions, kPosSoftPlus, 2>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisHermiteFunctions, kPosSoftPlus, 2>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisHermiteFunctions, kPosSoftPlus, 3>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisHermiteFunctions, kPosSoftPlus, 3>(const InverseParams&, int, cudaStream_t);
template cudaError_t launchFusedP<kBasisHermiteFunctions, kPosSoftPlus, 4>(const FusedParams&, int, int, int, cudaStream_t);
template cudaError_t launchInverseP<kBasisHermiteFunctions, kPosSoftPlus, 4>(const InverseParams&, int, cudaStream_t);

}  // namespace mpgb
