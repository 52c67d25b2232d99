// umag.cuh -- helpers of the per-block maximum of |u|^2 that GET_DT_BLOCK_ACM
// (LIB/EQUATION/ACMnew/module_ACM.f90:617-691) takes over the interior
// (k_misc.cu::dt_kernel), and the divergence guard of the ACM integral
// stage (rhs_ACM.f90:133-146).
//
// The exact maximum of the reference's FP64 expression u*u + v*v (+ w*w) is
// found in two passes so that the FP64 units see only a few points: pass 1
// takes the FP32 maximum m32 of the sums of truncated values (relative error
// below 2^-20 against the exact sums); the point holding the exact maximum
// then has an FP32 value above m32 (1 - 2^-17), and pass 2 evaluates the exact
// FP64 sum only for such points.
#pragma once
#include "exact.cuh"

namespace wg {

// |x| <= 1e12 on the bits (false for nan); the bits through the opaque move
// of exact.cuh, so that the test stays on the integer units
__device__ __forceinline__ bool within_guard(double x) {
    const unsigned long long a = (unsigned long long)dbits(x) & 0x7fffffffffffffffull;
    return a <= 0x426d1a94a2000000ull;   // bits of 1.0e12
}

// float not above |x|, by truncation on the integer units (0 below 2^-126,
// inf from 2^128): |x|(1 - 2^-23) < result <= |x| in the normal range
__device__ __forceinline__ float trunc_abs_f(double x) {
    const unsigned long long b = (unsigned long long)dbits(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -126) return 0.f;
    if (e > 127) return __uint_as_float(0x7f800000u);
    return __uint_as_float(((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}

// pass-2 threshold from the block's FP32 maximum: below 2^-100 the squares
// may be FP32 subnormals without the error bound, and every point is a
// candidate
__device__ __forceinline__ float umag_threshold(float m32) { return m32 < 0x1p-100f ? 0.f : m32 * (1.0f - 0x1p-17f); }

}  // namespace wg
