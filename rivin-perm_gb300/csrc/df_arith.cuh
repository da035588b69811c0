// Double-float arithmetic on the FP32 pipes: a value is the unevaluated sum
// hi + lo of two FP32 numbers (about 48 significand bits).  Addition is
// Knuth's two-sum followed by a renormalising fast two-sum; multiplication
// forms the exact error of hi*hi with an FMA (Dekker's product with fused
// multiply-add) and adds the cross terms.  Complex values are pairs.
#pragma once

#include <cuda_runtime.h>

namespace pg {

struct df { float hi, lo; };

__device__ __forceinline__ df df_from(double x) {
    df r;
    r.hi = (float)x;
    r.lo = (float)(x - (double)r.hi);
    return r;
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df df_add(df a, df b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    df r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}
__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    df r;
    r.hi = p + e;
    r.lo = e - (r.hi - p);
    return r;
}
// a / b by long division in two FP32 digits (Dekker 1971; the double-float
// quotient of Hida, Li and Bailey's QD library): q1 = a.hi / b.hi from the
// FP32 reciprocal, the remainder a - q1 b with the exact error of q1 b.hi
// from an FMA, then the correction digit q2 = remainder / b.hi.  Relative
// error about 2^-45 for normal operands; b must be well away from zero (the
// callers check it).
__device__ __forceinline__ df df_div(df a, df b) {
    const float r = __frcp_rn(b.hi);
    const float q1 = a.hi * r;
    const float p = q1 * b.hi;
    const float pe = fmaf(q1, b.hi, -p);
    float rem = (a.hi - p) - pe;
    rem = fmaf(-q1, b.lo, rem + a.lo);
    const float q2 = rem * r;
    df res;
    res.hi = q1 + q2;
    res.lo = q2 - (res.hi - q1);
    return res;
}
__device__ __forceinline__ df df_shfl_xor(df a, int off) {
    return df{__shfl_xor_sync(0xffffffffu, a.hi, off), __shfl_xor_sync(0xffffffffu, a.lo, off)};
}
__device__ __forceinline__ void kahan(double &sum, double &comp, double x) {
    const double y = x - comp;
    const double t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

struct dc { df re, im; };

__device__ __forceinline__ dc dc_mul(dc a, dc b) {
    dc r;
    r.re = df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im)));
    r.im = df_add(df_mul(a.re, b.im), df_mul(a.im, b.re));
    return r;
}

}  // namespace pg
