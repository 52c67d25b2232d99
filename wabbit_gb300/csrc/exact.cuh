// exact.cuh -- products with filter taps formed on the integer pipe.
//
// The wavelet and interpolation taps are short dyadic rationals: CDF4,4 has
// HD = (-1/512, 9/256, -1/32, -63/512, 9/32, 87/128, ...), GD and HR are
// +-1/16, +-9/16 and 1. A tap c = +-m 2^sh with an odd integer m < 2^7 times
// a normal x = M 2^(e-1075) (M the 53-bit significand) is the integer product
// P = M m (at most 60 bits) scaled by a power of two; rounding P to 53 bits
// to nearest-even gives the IEEE product bit for bit. For m = 1 (a power of
// two) the product is x with sh added to its exponent field. Forming the
// products with integer operations leaves the FP64 pipe, which bounds the
// transform kernels, to the additions. Zero inputs give a signed zero;
// subnormal, infinite and NaN inputs and results out of the normal range set
// bad, and the caller recomputes with the FP64 multiply. Results are
// bit-identical to __dmul_rn(x, tap).
//
// The functions compile for the host too (tests check them against the
// host's IEEE multiply).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define WG_HD __host__ __device__ __forceinline__
#else
#define WG_HD inline
#endif

namespace wg {

// kind 0: general tap, 1: +-2^sh, 2: exactly 1, 3: +-m 2^sh with m odd in
// [3, 127] (mul = m)
inline void classify_tap(double c, int &kind, int &sh, int &mul) {
    kind = 0;
    sh = 0;
    mul = 1;
    if (c == 1.0) {
        kind = 2;
        return;
    }
    if (c == 0.0 || !std::isfinite(c)) return;
    int e = 0;
    const double fr = std::fabs(std::frexp(c, &e));   // c = +-fr 2^e, fr in [0.5, 1)
    for (int k = 1; k <= 7; k++) {
        const double m = std::ldexp(fr, k);
        if (m != std::floor(m)) continue;
        const int mi = (int)m;
        if (mi == 1) {
            kind = 1;
            sh = e - 1;
        } else if (mi & 1) {
            kind = 3;
            sh = e - k;
            mul = mi;
        }
        return;
    }
}

// the bits of x through an opaque move: tests on the bits of a double that
// the compiler recognises as floating-point compares (x != 0, exponent field
// all ones) would otherwise become FP64 compares on the pipe this code keeps
// free
WG_HD long long dbits(double x) {
#ifdef __CUDA_ARCH__
    long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
#else
    long long b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
#endif
}
WG_HD double dfrom(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, sizeof(x));
    return x;
#endif
}

// x * (+-2^sh) with integer operations only; sgn is the tap's sign bit
// (0 or 1 << 63). Exact for zero and for normal x with a normal result;
// otherwise bad is set and the caller recomputes with the FP64 multiply.
WG_HD double pow2_mul(double x, int sh, long long sgn, bool &bad) {
    const long long b = dbits(x);
    const long long a = b & 0x7fffffffffffffffLL;
    const int e0 = (int)(a >> 52), e1 = e0 + sh;
    // branch-free range test (short-circuit logic here costs more than an
    // FP64 multiply): e0 and e1 in [1, 2046] unless x is zero
    bad |= (a != 0) & (((unsigned)(e0 - 1) > 2045u) | ((unsigned)(e1 - 1) > 2045u));
    const long long r = a == 0 ? b : b + (long long)sh * (1LL << 52);
    return dfrom(r ^ sgn);
}

// x * (+-m 2^sh) for an odd m in [3, 127]: the 53-bit significand times m,
// rounded to nearest-even, with the exponent e + sh + (dropped bits)
WG_HD double short_mul(double x, int m, int sh, long long sgn, bool &bad) {
    const long long b = dbits(x);
    const unsigned long long a = (unsigned long long)b & 0x7fffffffffffffffULL;
    const int e = (int)(a >> 52);
#ifdef __CUDA_ARCH__
    const int k = 32 - __clz(m);                      // bit length of m
#else
    int k = 0;
    while ((m >> k) != 0) k++;
#endif
    const unsigned long long M = (a & 0xfffffffffffffULL) | 0x10000000000000ULL;
    const unsigned long long P = M * (unsigned long long)m;   // in [2^(51+k), 2^(53+k))
    const int q = (P >> (52 + k)) ? k : k - 1;                // bits to drop, >= 1
    const unsigned long long mant = (P + ((1ULL << (q - 1)) - 1) + ((P >> q) & 1)) >> q;   // in [2^52, 2^53]
    const int E = e + sh + q;                                 // biased exponent of mant 2^(E-1075)
    bad |= (a != 0ULL) & (((unsigned)(e - 1) > 2045u) | ((unsigned)(E - 1) > 2044u));   // e in [1, 2046], E in [1, 2045]
    // (E - 1) << 52 plus the significand with its leading bit: a rounding
    // carry to 2^53 moves into the exponent field
    const long long r = a == 0 ? 0 : (long long)(((unsigned long long)(E - 1) << 52) + mant);
    return dfrom(r ^ (b & (long long)0x8000000000000000ULL) ^ sgn);
}

// the same decision per tap at run time (kind 0 general, 1 +-2^sh, 2 one,
// 3 +-mul 2^sh)
WG_HD double tap_mul(double x, double c, int kind, int sh, int mul, long long sgn, bool &bad) {
    if (kind == 2) return x;
    if (kind == 1) return pow2_mul(x, sh, sgn, bad);
    if (kind == 3) return short_mul(x, mul, sh, sgn, bad);
#ifdef __CUDA_ARCH__
    return __dmul_rn(x, c);
#else
    return x * c;
#endif
}

}  // namespace wg
