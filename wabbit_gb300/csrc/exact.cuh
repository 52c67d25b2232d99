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

__device__ __forceinline__ double tap_mul(double x, double c, int kind, int sh) {
    if (kind == 2) return x;
    if (kind == 1) {
        const long long b = __double_as_longlong(x);
        const int e0 = (int)((b >> 52) & 0x7ff), e1 = e0 + sh;
        if (e0 != 0 && e0 != 0x7ff && e1 > 0 && e1 < 0x7ff) {
            long long r = b + (long long)sh * (1LL << 52);
            if (c < 0.0) r ^= (long long)0x8000000000000000ULL;
            return __longlong_as_double(r);
        }
    }
    return __dmul_rn(x, c);
}

}  // namespace wg
