// df.cuh -- double-float arithmetic on the FP32 units.
//
// A value is held as an unevaluated sum hi + lo of two floats (|lo| <=
// ulp(hi)/2), about 48 significant bits. The operations are the classical
// error-free transformations (Knuth's two-sum, Dekker's two-product with an
// FMA) followed by a renormalisation; their relative error is a few 2^-48.
// They must not be contracted or reassociated: the translation units that
// include this header are compiled with -fmad=false, and every FMA below is
// explicit.
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

}  // namespace wg
