// exact.cuh -- products with filter taps that are exact powers of two.
//
// Many wavelet taps are +-2^k (CDF4,4: HD(+-6) = -1/512, HD(+-3) = -1/32,
// GD(+-3) = 1/16, GD(0) = 1). For a normal x whose scaled value stays
// normal, x * (+-2^k) is exact: the IEEE product equals x with k added to its
// exponent field (and the sign flipped for a negative tap). Forming it with
// integer operations leaves the FP64 pipe, which bounds the transform
// kernels, to the other taps; zero, subnormal, infinite and NaN inputs and
// results out of the normal range take the FP64 multiply. Results are
// bit-identical to __dmul_rn(x, tap).
#pragma once
#include <cmath>

namespace wg {

// kind 0: general tap, 1: +-2^sh, 2: exactly 1
inline void classify_tap(double c, int &kind, int &sh) {
    kind = 0;
    sh = 0;
    if (c == 1.0) {
        kind = 2;
        return;
    }
    int e = 0;
    const double m = std::frexp(c, &e);
    if (m == 0.5 || m == -0.5) {
        kind = 1;
        sh = e - 1;
    }
}

// x * (+-2^sh) with integer operations only; sgn is the tap's sign bit
// (0 or 1 << 63). Exact for zero and for normal x with a normal result;
// otherwise bad is set and the caller recomputes with the FP64 multiply.
__device__ __forceinline__ double pow2_mul(double x, int sh, long long sgn, bool &bad) {
    const long long b = __double_as_longlong(x);
    const long long a = b & 0x7fffffffffffffffLL;
    const int e0 = (int)(a >> 52), e1 = e0 + sh;
    bad |= a != 0 && (e0 == 0 || e0 == 0x7ff || e1 <= 0 || e1 >= 0x7ff);
    const long long r = a == 0 ? b : b + (long long)sh * (1LL << 52);
    return __longlong_as_double(r ^ sgn);
}

// the same decision per tap at run time (kind 0 general, 1 +-2^sh, 2 one)
__device__ __forceinline__ double tap_mul(double x, double c, int kind, int sh, long long sgn, bool &bad) {
    if (kind == 2) return x;
    if (kind == 1) return pow2_mul(x, sh, sgn, bad);
    return __dmul_rn(x, c);
}

}  // namespace wg
