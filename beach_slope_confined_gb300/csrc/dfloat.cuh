// dfloat.cuh -- double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2: about 48 significant bits.  On this GPU the FP32 pipe
// issues about 64 times as many lanes per clock as the FP64 pipe, so a
// double-float operation of 3 to 20 FP32 instructions is cheaper than one FP64
// instruction wherever 48 bits suffice.  The mixed path's PPE assembly uses
// it (ppe.cu): its coefficients come out within ~1e-13 of the FP64 assembly.
//
// The building blocks are the error-free transformations: Knuth's TwoSum
// (the rounding error of a + b, exactly) and the FMA TwoProduct (that of
// a * b).  The operations combine them as in Dekker (1971), "A floating-point
// technique for extending the available precision", and in the double-double
// algorithms of Hida, Li and Bailey (2001), here on FP32 pairs.  Every step is
// an explicitly rounded intrinsic, so the compiler can neither contract nor
// reorder them.
#pragma once

#include "bsc_internal.cuh"

namespace bsc {

struct df2 {
    float hi, lo;
};

// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ df2 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// s + e = a + b exactly, for |a| >= |b| (or a == 0)
__device__ __forceinline__ df2 df_quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df2 df_neg(df2 a) { return {-a.hi, -a.lo}; }

// a + b, with the errors of both halves carried (accurate under cancellation)
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    df2 s = df_two_sum(a.hi, b.hi);
    const df2 t = df_two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = df_quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return df_quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df2 df_sub(df2 a, df2 b) { return df_add(a, df_neg(b)); }

// a + b for an FP32 b: the TwoSum of the high parts, a.lo carried
__device__ __forceinline__ df2 df_add_f(df2 a, float b) {
    df2 s = df_two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return df_quick_two_sum(s.hi, s.lo);
}

// a * b: the exact product of the high parts (TwoProduct by FMA) plus the
// cross terms
__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_quick_two_sum(p, e);
}

// a * a
__device__ __forceinline__ df2 df_sqr(df2 a) {
    const float p = __fmul_rn(a.hi, a.hi);
    float e = __fmaf_rn(a.hi, a.hi, -p);
    e = __fmaf_rn(__fadd_rn(a.hi, a.hi), a.lo, e);
    return df_quick_two_sum(p, e);
}

// 2 a (exact)
__device__ __forceinline__ df2 df_twice(df2 a) { return {__fmul_rn(2.0f, a.hi), __fmul_rn(2.0f, a.lo)}; }

// 1 / a: the FP32 reciprocal y of a.hi and one Newton step y + y (1 - a y),
// whose residual 1 - a y is formed exactly enough from TwoProduct (y is
// within 2^-23 of 1/a, so the step leaves about 2^-46)
__device__ __forceinline__ df2 df_rcp(df2 a) {
    const float y = __frcp_rn(a.hi);
    const float p = __fmul_rn(a.hi, y);
    float e = __fmaf_rn(a.hi, y, -p);  // a.hi y = p + e exactly
    e = __fmaf_rn(a.lo, y, e);         // + a.lo y
    // p lies within an ulp of 1, so 1 - p is exact
    const float r = __fsub_rn(__fsub_rn(1.0f, p), e);
    return df_quick_two_sum(y, __fmul_rn(y, r));
}

// sqrt(a) for a > 0: the FP32 root r0 = a.hi / sqrt(a.hi) from the
// reciprocal root, then one Newton correction r0 + (a - r0^2) / (2 r0) with
// the residual formed exactly enough (r0^2 by TwoProduct; a.hi - r0^2 is
// exact, r0^2 lying within 2^-21 of a.hi): about 2^-44 relative
__device__ __forceinline__ df2 df_sqrt(df2 a) {
    const float y = rsqrtf(a.hi);
    const float r0 = __fmul_rn(a.hi, y);
    const float p = __fmul_rn(r0, r0);
    const float e = __fmaf_rn(r0, r0, -p);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
    return df_quick_two_sum(r0, __fmul_rn(__fmul_rn(res, y), 0.5f));
}

// FP32 -> FP64 on the integer pipe, zero kept exact
__device__ __forceinline__ double f64z(float f) { return f == 0.0f ? 0.0 : f64_of(f); }

// FP64 -> double-float: hi the FP32 rounding (on the integer pipe), lo the
// rounding of the remainder: one FP64 subtraction
__device__ __forceinline__ df2 df_of(double x) {
    const float h = f32_of(x);
    return {h, f32_of(x - f64z(h))};
}

// double-float -> FP64: one FP64 addition
__device__ __forceinline__ double df_to_double(df2 a) { return f64z(a.hi) + f64z(a.lo); }

__device__ __forceinline__ float2 df_pack(df2 a) { return make_float2(a.hi, a.lo); }
__device__ __forceinline__ df2 df_unpack(float2 v) { return {v.x, v.y}; }

// x_i - x_j of two particles from their offsets o to their own cells'
// origins and the cells' column (or row) difference k: (o_i - o_j) + k cs
__device__ __forceinline__ df2 df_pair_offset(df2 oi, float2 oj, int k, df2 cs) {
    df2 d = df_sub(oi, df_unpack(oj));
    if (k == 1) d = df_add(d, cs);
    else if (k == -1) d = df_sub(d, cs);
    else if (k != 0) d = df_add(d, df_mul(cs, df2{(float)k, 0.0f}));
    return d;
}

}  // namespace bsc
