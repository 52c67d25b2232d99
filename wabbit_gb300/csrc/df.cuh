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

__device__ __forceinline__ df2 df_neg(df2 a) { return {-a.hi, -a.lo}; }

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

// The rare cases of the conversions below (zero, subnormal, inf or nan
// operands) take the FP64 units; they are kept out of line so that the common
// path is a real branch around them and never issues their FP64
// instructions as predicated-off work (the FP64 units of this GPU run a warp
// instruction in tens of cycles).
static __device__ __noinline__ df2 df_from_slow(double v) { return df_from(v); }
static __device__ __noinline__ double df_to_double_slow(float hi, float lo) {
    return __dadd_rn((double)hi, (double)lo);
}

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
    if (e < -74 || e > 127) return df_from_slow(v);
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    const unsigned r = (unsigned)b & 0x1fffffffu;     // the 29 bits below hi
    if (r == 0u) return {hi, 0.f};
    const int p = 31 - __clz(r);                      // leading one of r, 0..28
    const unsigned m = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
    const float lo = __uint_as_float(sign | ((unsigned)(e - 52 + p + 127) << 23) | (m & 0x7fffffu));
    return {hi, lo};
}

// ---------------------------------------------------------------------------
// Anchored double-float values. Every hi part is a multiple of one quantum q
// with |hi| <= 2^20 q at the start of a step (2^22 q leaves room for values
// that double within the step and for interpolated ghost values above their
// coarse data), so a sum of up to four hi parts with factors of one or two
// is an exact FP32 operation, and
// the lo parts (|lo| <= q/2, 24 bits below that) carry the rest. A stencil
// difference A - B or second difference A + B - 2u then costs two FP32
// instructions (hi exact, lo rounded about 2^-43 of the largest value)
// instead of an error-free double-float addition; only the final weighted
// combination of two such differences needs a two-sum.
// ---------------------------------------------------------------------------

// round v's hi part to the quantum of M = 1.5 * 2^23 * q (exact: v.hi - h is
// the rounding residue); M = 0 leaves v as it is
__device__ __forceinline__ df2 anchor(df2 v, float M) {
    const float h = (v.hi + M) - M;
    return {h, (v.hi - h) + v.lo};
}

// M for a state whose largest magnitude has the float bits umax_bits: the
// quantum is 2^-20 of the power of two above the maximum; 0 (no anchoring)
// for a zero state or a quantum outside the normal float range
__host__ __device__ inline float anchor_constant(unsigned umax_bits) {
    const int be = (int)((umax_bits >> 23) & 0xffu);
    if (be == 0 || be == 0xff) return 0.f;
    const int E = be - 127 + 1;               // max|u| < 2^E, q = 2^(E-20)
    if (E - 20 < -126 || E + 3 > 127) return 0.f;
    union { unsigned u; float f; } m;
    m.u = ((unsigned)(E + 3 + 127) << 23) | 0x400000u;   // 1.5 * 2^(E+3) = 1.5 * 2^23 * q
    return m.f;
}

// the double nearest hi + lo of a normalised pair (|lo| <= ulp(hi)/2), formed
// on the integer units: the two significands are aligned in one 53-bit
// integer (at most one bit of lo below the double's last place is cut);
// zero, subnormal, inf or nan hi parts take the FP64 units
__device__ __forceinline__ double df_to_double(df2 x) {
    const unsigned hb = __float_as_uint(x.hi), lb = __float_as_uint(x.lo);
    const int he = (int)((hb >> 23) & 0xffu);
    if (he == 0 || he == 0xff) return df_to_double_slow(x.hi, x.lo);
    long long S = (long long)((hb & 0x7fffffu) | 0x800000u) << 29;   // unit 2^(e(hi) - 52)
    const int le = (int)((lb >> 23) & 0xffu);
    if (le != 0) {
        const int sh = le - he + 29;
        const long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);
        const long long Y = sh >= 0 ? (ml << sh) : (sh > -24 ? (ml >> -sh) : 0LL);
        S = ((hb ^ lb) >> 31) ? S - Y : S + Y;
    }
    int e = he - 127 + 1023;
    if (S < (1LL << 52)) {   // lo of the other sign took the leading bit
        S <<= 1;
        e -= 1;
    }
    const unsigned long long bits = ((unsigned long long)(hb >> 31) << 63) | ((unsigned long long)e << 52) |
                                    ((unsigned long long)S & 0xfffffffffffffULL);
    return __longlong_as_double((long long)bits);
}

}  // namespace wg
