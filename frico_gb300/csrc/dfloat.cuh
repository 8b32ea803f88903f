// Double-float arithmetic on the FP32 pipe: a value is the unevaluated sum
// h + l of two FP32 numbers with |l| <= ulp(h) / 2 (about 48 significant bits).
// Error-free transformations after Knuth (two-sum) and Dekker (two-product,
// here with the FMA); the elementary functions below are written from their
// mathematical definitions:
//   sqrt:   one Newton step from the FP32 square root,  y + (x - y^2) / (2 y)
//   1/x:    one Newton step from the FP32 reciprocal,  y + y (1 - x y)
//   sincos: Cody-Waite reduction by pi/2 (pi/2 split in four parts, the first
//           three with 12 significant bits so that q * part is exact for
//           q < 2^12), then the Taylor series of sin and cos on |r| <= pi/4
//           (terms below 1e-7 summed in FP32, the rest in double-float).
// Accuracy: about 2^-46 relative for +, *, sqrt, 1/x; sincos to about
// 2^-47 absolute plus the argument's own error.
#pragma once

#include <cuda_runtime.h>

namespace frico {

struct dfl {
    float h, l;
};

__device__ __forceinline__ dfl dmk(float h, float l = 0.f) { return dfl{h, l}; }

__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    return dfl{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}

__device__ __forceinline__ dfl quick_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return dfl{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
    dfl s = two_sum(x.h, y.h);
    return quick_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}

__device__ __forceinline__ dfl df_add_f(dfl x, float f) {
    dfl s = two_sum(x.h, f);
    return quick_two_sum(s.h, __fadd_rn(s.l, x.l));
}

__device__ __forceinline__ dfl df_neg(dfl x) { return dfl{-x.h, -x.l}; }

__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ dfl df_mul_f(dfl x, float f) {
    const float p = __fmul_rn(x.h, f);
    float e = __fmaf_rn(x.h, f, -p);
    e = __fmaf_rn(x.l, f, e);
    return quick_two_sum(p, e);
}

// x > 0
__device__ __forceinline__ dfl df_sqrt(dfl x) {
    const float y = sqrtf(x.h);
    const float e = __fadd_rn(__fmaf_rn(-y, y, x.h), x.l);
    return quick_two_sum(y, __fmul_rn(e, __fmul_rn(0.5f, rsqrtf(x.h))));
}

// x != 0
__device__ __forceinline__ dfl df_rcp(dfl x) {
    const float y = __frcp_rn(x.h);
    const float e = __fsub_rn(__fmaf_rn(-x.h, y, 1.0f), __fmul_rn(x.l, y));
    return quick_two_sum(y, __fmul_rn(y, e));
}

// FP64 value as a double-float by integer operations (see split_df in common.cuh)
__device__ __forceinline__ dfl df_from_double(double d, int& bad) {
    dfl r;
    split_df(d, r.h, r.l, bad);
    return r;
}

__device__ __forceinline__ double df_to_double(dfl x) { return f2d_exact(x.h) + f2d_exact(x.l); }

// sin and cos of x (0 <= x.h < 6400: |q| < 2^12); false beyond that range.
__device__ __forceinline__ bool df_sincos(dfl x, dfl& s, dfl& c) {
    // 2/pi and pi/2 = P1 + P2 + P3 + P4 (P1..P3: 12 significant bits each)
    const float kTwoOverPi = 0x1.45f306p-1f;
    const float P1 = 0x1.92p+0f, P2 = 0x1.fb4p-12f, P3 = 0x1.444p-24f, P4 = 0x1.68c234p-39f;
    if (!(x.h >= 0.f && x.h < 6400.f)) return false;
    const float q = rintf(__fmul_rn(x.h, kTwoOverPi));
    dfl r = dmk(__fmaf_rn(-q, P1, x.h));   // exact: q P1 exact, result within a factor 2 of x.h or x.h itself
    r = df_add_f(r, x.l);
    r = df_add_f(r, -__fmul_rn(q, P2));    // exact products
    r = df_add_f(r, -__fmul_rn(q, P3));
    r = df_add_f(r, -__fmul_rn(q, P4));
    const dfl r2 = df_mul(r, r);
    // Taylor coefficients (-1)^k / (2k+1)! and (-1)^k / (2k)!, as (hi, lo) pairs of their exact values
    const float ts = __fmaf_rn(__fmaf_rn(__fmaf_rn(0x1.952c78p-49f, r2.h, -0x1.ae7f3ep-41f), r2.h, 0x1.612462p-33f),
                               r2.h, -0x1.ae6456p-26f);                                   // k = 5..8
    const float tc = __fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(-0x1.682786p-53f, r2.h, 0x1.ae7f3ep-45f), r2.h,
                                                   -0x1.93974ap-37f), r2.h, 0x1.1eed8ep-29f),
                               r2.h, -0x1.27e4fcp-22f);                                   // k = 5..9
    dfl ps = dmk(ts), pc = dmk(tc);
    const dfl cs[5] = {dmk(0x1.71de3ap-19f, 0x1.55b1ccp-45f), dmk(-0x1.a01a02p-13f, 0x1.7f97fap-39f),
                       dmk(0x1.111112p-7f, -0x1.dddddep-32f), dmk(-0x1.555556p-3f, 0x1.555556p-28f),
                       dmk(1.0f)};
    const dfl cc[5] = {dmk(0x1.a01a02p-16f, -0x1.7f97fap-42f), dmk(-0x1.6c16c2p-10f, 0x1.27d27ep-35f),
                       dmk(0x1.555556p-5f, -0x1.555556p-30f), dmk(-0.5f), dmk(1.0f)};
#pragma unroll
    for (int k = 0; k < 5; k++) {
        ps = df_add(df_mul(ps, r2), cs[k]);
        pc = df_add(df_mul(pc, r2), cc[k]);
    }
    ps = df_mul(ps, r);
    switch (int(q) & 3) {
        case 0: s = ps; c = pc; break;
        case 1: s = pc; c = df_neg(ps); break;
        case 2: s = df_neg(ps); c = df_neg(pc); break;
        default: s = df_neg(pc); c = ps; break;
    }
    return true;
}

// complex double-float
struct cdf {
    dfl r, i;
};
__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
    return cdf{df_add(df_mul(a.r, b.r), df_neg(df_mul(a.i, b.i))), df_add(df_mul(a.r, b.i), df_mul(a.i, b.r))};
}
__device__ __forceinline__ cdf cdf_scale(cdf a, dfl s) { return cdf{df_mul(a.r, s), df_mul(a.i, s)}; }
__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return cdf{df_add(a.r, b.r), df_add(a.i, b.i)}; }
__device__ __forceinline__ cdf cdf_sub(cdf a, cdf b) { return cdf{df_add(a.r, df_neg(b.r)), df_add(a.i, df_neg(b.i))}; }
__device__ __forceinline__ cdf cdf_of(float4 q) { return cdf{dmk(q.x, q.y), dmk(q.z, q.w)}; }
__device__ __forceinline__ float4 f4_of(double2 z, int& bad) {
    float4 q;
    split_df(z.x, q.x, q.y, bad);
    split_df(z.y, q.z, q.w, bad);
    return q;
}

}  // namespace frico
