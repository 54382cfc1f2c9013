// wd_df.cuh -- double-float ("df64") arithmetic on the FP32 pipe.
//
// A real value is the unevaluated sum h + l of two floats (h = fl32(x),
// l = fl32(x - h), ~48-bit significand).  Sums use Knuth's error-free
// TwoSum on the high parts; products use the FMA-based exact product
// p + e = xh*yh (e = fma(xh, yh, -p)) plus the two cross terms xh*yl and
// xl*yh, whose own rounding is below 2^-48 of the operands.  The low parts
// are carried unnormalised: errors stay bounded relative to the operands'
// magnitudes, which is what the relative-L2 bar of a Dslash output measures.
// Every step uses explicit _rn intrinsics so the compiler cannot contract or
// reassociate the error-free transformations.
//
// On GB300 the FP64 pipe runs at 1/58 of the FP32 rate, so ~12 FP32
// operations per FP64 multiply-add still win by ~5x.
#pragma once
#include <cuda_runtime.h>

struct dfr {
    float h, l;
};
struct dfc {
    dfr re, im;
};

__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ dfr df_add(dfr a, dfr b)
{
    dfr r;
    float e;
    df_two_sum(a.h, b.h, r.h, e);
    r.l = __fadd_rn(__fadd_rn(a.l, b.l), e);
    return r;
}
__device__ __forceinline__ dfr df_neg(dfr a) { return dfr{-a.h, -a.l}; }
__device__ __forceinline__ dfr df_sub(dfr a, dfr b) { return df_add(a, df_neg(b)); }

// x * y as a fresh accumulator
__device__ __forceinline__ dfr df_mul(dfr x, dfr y)
{
    dfr r;
    r.h = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -r.h);
    e = __fmaf_rn(x.h, y.l, e);
    r.l = __fmaf_rn(x.l, y.h, e);
    return r;
}

// s + x * y
__device__ __forceinline__ dfr df_madd(dfr s, dfr x, dfr y)
{
    const float p = __fmul_rn(x.h, y.h);
    float l = __fmaf_rn(x.h, y.h, -p);
    l = __fmaf_rn(x.h, y.l, l);
    l = __fmaf_rn(x.l, y.h, l);
    l = __fadd_rn(l, s.l);
    float h, e;
    df_two_sum(s.h, p, h, e);
    return dfr{h, __fadd_rn(l, e)};
}

// ------------------------------------------------- complex overload set
__device__ __forceinline__ dfc c_zero(dfc) { return dfc{{0.f, 0.f}, {0.f, 0.f}}; }
__device__ __forceinline__ dfc c_add(dfc a, dfc b) { return dfc{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc c_sub(dfc a, dfc b) { return dfc{df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
__device__ __forceinline__ dfc c_i(dfc a) { return dfc{df_neg(a.im), a.re}; }
// u * h
__device__ __forceinline__ dfc c_mul(dfc u, dfc h)
{
    return dfc{df_madd(df_mul(u.re, h.re), df_neg(u.im), h.im), df_madd(df_mul(u.re, h.im), u.im, h.re)};
}
// acc + u * h
__device__ __forceinline__ dfc c_madd(dfc acc, dfc u, dfc h)
{
    acc.re = df_madd(df_madd(acc.re, u.re, h.re), df_neg(u.im), h.im);
    acc.im = df_madd(df_madd(acc.im, u.re, h.im), u.im, h.re);
    return acc;
}
// conj(u) * h
__device__ __forceinline__ dfc c_mulc(dfc u, dfc h)
{
    return dfc{df_madd(df_mul(u.re, h.re), u.im, h.im), df_madd(df_mul(u.re, h.im), df_neg(u.im), h.re)};
}
// acc + conj(u) * h
__device__ __forceinline__ dfc c_maddc(dfc acc, dfc u, dfc h)
{
    acc.re = df_madd(df_madd(acc.re, u.re, h.re), u.im, h.im);
    acc.im = df_madd(df_madd(acc.im, u.re, h.im), df_neg(u.im), h.re);
    return acc;
}

// Renormalise so that |l| <= ulp(h)/2.  Sums with cancellation leave l large
// relative to h; a product then loses its omitted l*l term and cross-term
// rounding grows with |l/h|, so every stored value is renormalised.
__device__ __forceinline__ dfr df_norm(dfr a)
{
    dfr r;
    df_two_sum(a.h, a.l, r.h, r.l);
    return r;
}

// ------------------------------------------------------------- storage
// A complex df value is stored (normalised) as float4 {re.h, im.h, re.l, im.l}:
// the high parts and the low parts each form an adjacent (re, im) pair, the
// operand shape of the packed FP32 instructions (wd_df2.cuh).
__device__ __forceinline__ dfc df_from_f4(float4 v) { return dfc{{v.x, v.z}, {v.y, v.w}}; }
__device__ __forceinline__ float4 df_to_f4(dfc a)
{
    const dfr re = df_norm(a.re), im = df_norm(a.im);
    return make_float4(re.h, im.h, re.l, im.l);
}

__host__ __device__ __forceinline__ dfr df_split(double x)
{
    const float h = (float)x;
    return dfr{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_value(dfr a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ float4 df_pack(double2 v)
{
    const dfr r = df_split(v.x), i = df_split(v.y);
    return make_float4(r.h, i.h, r.l, i.l);
}
__device__ __forceinline__ double2 df_unpack(float4 v)
{
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}
