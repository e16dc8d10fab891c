// Explicit instantiation of the persistent batch kernel.
#include "mpgb_kernels.cuh"

namespace mpgb {

template cudaError_t launchBatchP<kBasisHermiteFunctions, kPosExp>(const FusedParams&, int, int, int*, cudaStream_t);

}  // namespace mpgb
