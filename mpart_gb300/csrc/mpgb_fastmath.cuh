// Exponential and logarithm for the rectifiers, table-driven after
// P. T. P. Tang, "Table-driven implementation of the exponential function in
// IEEE floating-point arithmetic", ACM TOMS 15(2):144-157, 1989, and "...of
// the logarithm function...", ACM TOMS 16(4):378-400, 1990.  A 64-entry table
// of 2^(j/64) (and a 129-entry table for the logarithm) leaves a reduced
// argument of magnitude <= 2^-7.4 (2^-8), whose series is short: fewer FP64
// instructions than a polynomial over a wider interval.  Both are accurate
// to about one unit in the last place (tests/test_fastmath.py builds them for
// the host and checks them against 40-digit decimal references).
//
// The header compiles for the host too (the test harness builds it with g++).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define __device__
#define __host__
#define __forceinline__ inline
#endif

#include "mpgb_fastmath_tables.h"

namespace mpgb {
namespace fm {

__host__ __device__ __forceinline__ long long bitsOf(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

__host__ __device__ __forceinline__ double fromBits(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

template <class T>
__host__ __device__ __forceinline__ T loadTab(const T* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

// 2^n for -1022 <= n <= 1023.
__host__ __device__ __forceinline__ double pow2i(int n) { return fromBits((long long)(n + 1023) << 52); }

// e^x.  x = (64 n + j) ln2/64 + r with |r| <= ln2/128 (n, j from the nearest
// integer k = 64 n + j to x 64/ln2; ln2/64 split in two so that k times the
// leading part is exact), e^x = 2^n 2^(j/64) (1 + p(r)), p the degree-5 Taylor
// polynomial of e^r - 1 (truncation below 4e-17 relative).  Overflow gives
// +inf beyond log(DBL_MAX), underflow gradual subnormals and then 0.
__host__ __device__ __forceinline__ double expT(double x) {
    constexpr double kMagic = 0x1.8p52;  // rounds to an integer; k in the low word
    const double t = x * kInvLn2x64;
    const double kb = t + kMagic;
    const double kd = kb - kMagic;
    const int k = (int)(unsigned)(bitsOf(kb) & 0xffffffffLL);
    double r = fma(-kd, kLn2x64Hi, x);
    r = fma(-kd, kLn2x64Lo, r);
    double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    q = fma(r, q, 1.0 / 6.0);
    q = fma(r, q, 0.5);
    const double p = fma(r * r, q, r);
    const double s = loadTab(&kExp2Tab[k & 63]);
    const double m = fma(s, p, s);  // in [0.99, 2.01)
    const int n = k >> 6;           // |n| <= 1022 for |x| < 708
    if (fabs(x) < 708.0) return m * pow2i(n);
    // Rare: |x| near or beyond the exponent range, and NaN (k is meaningless
    // beyond |x| = 745, where the result no longer depends on it).
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    // Two steps, so that a subnormal result is rounded once, at the end.
    return (n > 0) ? (m * pow2i(n - 600)) * pow2i(600) : (m * pow2i(n + 600)) * pow2i(-600);
}

// log(y) for y in [1, 2] (the SoftPlus argument 1 + e^-|x|), and NaN for NaN.
// y = 1 + j/128 + f, j the nearest integer to (y - 1) 128: y inv_j = 1 + r
// with |r| <= 2^-8 exactly by one fused multiply-add, inv_j the double nearest
// 1 / (1 + j/128), so log y = log1p(r) - log(inv_j) exactly; log1p(r) by its
// degree-7 series (truncation below 2^-59 relative to r).  j = 0 has inv = 1
// and log = 0, so y near 1 keeps full relative accuracy; y = 2 is j = 128.
__host__ __device__ __forceinline__ double log1to2T(double y) {
    const long long b = bitsOf(y);
    // (y - 1) 128 rounded: mantissa bits 45..51 plus the exponent step at 2.
    const int j = (y >= 2.0) ? 128 : (int)(((b & 0x000fffffffffffffLL) + (1LL << 44)) >> 45);
    const double r = fma(y, loadTab(&kLogInvTab[j]), -1.0);
    double q = fma(r, 1.0 / 7.0, -1.0 / 6.0);
    q = fma(r, q, 1.0 / 5.0);
    q = fma(r, q, -0.25);
    q = fma(r, q, 1.0 / 3.0);
    q = fma(r, q, -0.5);
    const double l1p = fma(r * r, q, r);
    return loadTab(&kLogTab[j]) + l1p;
}

}  // namespace fm
}  // namespace mpgb
