// df.cuh -- double-float arithmetic on the FP32 units.
//
// A value is held as an unevaluated sum hi + lo of two floats (|lo| <=
// ulp(hi)/2), about 48 significant bits. The operations are the classical
// error-free transformations (Knuth's two-sum, Dekker's two-product with an
// FMA) followed by a renormalisation; their relative error is a few 2^-48.
// They must not be contracted or reassociated: the translation units that
// use them are compiled with -fmad=false, and every FMA below is explicit
// (df_from alone, a single subtraction, has nothing to contract).
#pragma once
#include <cuda_runtime.h>

namespace wg {

struct df2 {
    float hi, lo;
};

__device__ __forceinline__ df2 df_from(double v) {
    const float h = __double2float_rn(v);
    const float l = __double2float_rn(v - (double)h);
    return {h, l};
}

__device__ __forceinline__ double df_to(df2 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df2 quick_two_sum(float a, float b) {
    const float s = a + b;
    const float e = b - (s - a);
    return {s, e};
}

__device__ __forceinline__ df2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    const df2 s = two_sum(a.hi, b.hi);
    const float e = s.lo + (a.lo + b.lo);
    return quick_two_sum(s.hi, e);
}

__device__ __forceinline__ df2 df_neg(df2 a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

// The same operations without the final renormalisation. Their results may
// carry |lo| above ulp(hi)/2 (after cancellation even |lo| > |hi|); every
// operation below accepts such pairs, and the absolute error of a chain stays
// a few 2^-48 of the magnitudes that entered it. df_norm restores the
// canonical form (two_sum, exact for any pair).
__device__ __forceinline__ df2 df_add_nr(df2 a, df2 b) {
    const df2 s = two_sum(a.hi, b.hi);
    return {s.hi, s.lo + (a.lo + b.lo)};
}

__device__ __forceinline__ df2 df_sub_nr(df2 a, df2 b) { return df_add_nr(a, df_neg(b)); }

__device__ __forceinline__ df2 df_mul_nr(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return {p, e};
}

// multiplication by a power of two: exact
__device__ __forceinline__ df2 df_pow2(df2 a, float s) { return {a.hi * s, a.lo * s}; }

__device__ __forceinline__ df2 df_norm(df2 a) { return two_sum(a.hi, a.lo); }

// double -> double-float by bit manipulation on the integer units: hi is v
// truncated to 24 significant bits, lo the remainder truncated to 24 bits
// (|v - hi - lo| < 2^-47 |v|). Zero is exact; magnitudes outside
// [2^-74, 2^128) (where lo or hi would not be a normal float) and inf/nan go
// through the FP64 units.
__device__ __forceinline__ df2 df_split(double v) {
    // the bits through an opaque move: the compiler would otherwise turn the
    // zero and exponent tests below into FP64 compares
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    if ((b << 1) == 0ull) return {__uint_as_float(sign), 0.f};
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -74 || e > 127) return df_from(v);
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    const unsigned r = (unsigned)b & 0x1fffffffu;     // the 29 bits below hi
    if (r == 0u) return {hi, 0.f};
    const int p = 31 - __clz(r);                      // leading one of r, 0..28
    const unsigned m = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
    const float lo = __uint_as_float(sign | ((unsigned)(e - 52 + p + 127) << 23) | (m & 0x7fffffu));
    return {hi, lo};
}

// float -> double (exact) by bit manipulation; zero, subnormal, inf and nan
// inputs go through the conversion unit
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex == 0u || ex == 0xffu) return (double)f;
    const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                                 ((unsigned long long)(ex - 127 + 1023) << 52) |
                                 ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)b);
}

}  // namespace wg
