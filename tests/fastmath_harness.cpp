// Host build of the device exponential and logarithm (mpgb_fastmath.cuh) for
// tests/test_fastmath.py.
#include "../mpart_gb300/csrc/mpgb_fastmath.cuh"

extern "C" void fm_exp(const double* x, double* y, long n) {
    for (long i = 0; i < n; ++i) y[i] = mpgb::fm::expT(x[i]);
}

extern "C" void fm_log1to2(const double* x, double* y, long n) {
    for (long i = 0; i < n; ++i) y[i] = mpgb::fm::log1to2T(x[i]);
}
