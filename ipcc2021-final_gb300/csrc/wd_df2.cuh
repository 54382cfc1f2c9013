// wd_df2.cuh -- double-float arithmetic on (re, im) pairs with the packed
// FP32 instructions of sm_100-family GPUs (add/sub/mul/fma .f32x2: two FP32
// operations per issued instruction, same FP32-pipe throughput).
//
// A complex df value is dfp{h = (re.h, im.h), l = (re.l, im.l)}, the
// storage order of wd_df.cuh, so a 16-byte load yields both pairs in place.
// Every operation performs, lane by lane, exactly the roundings of the scalar
// forms in wd_df.cuh (TwoSum, FMA exact products, the same operand order),
// so a kernel written with these gives bit-identical results to its scalar
// twin with about half the arithmetic instructions.
#pragma once
#include "wd_df.cuh"

__device__ __forceinline__ unsigned long long wd_f2u(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 wd_u2f(unsigned long long a)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a));
    return r;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(wd_f2u(a)), "l"(wd_f2u(b)));
    return wd_u2f(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(wd_f2u(a)), "l"(wd_f2u(b)));
    return wd_u2f(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(wd_f2u(a)), "l"(wd_f2u(b)));
    return wd_u2f(d);
}
// a * b + c, one rounding per lane
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(wd_f2u(a)), "l"(wd_f2u(b)), "l"(wd_f2u(c)));
    return wd_u2f(d);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

struct dfp {
    float2 h, l;
};

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e)
{
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

// df_add per lane
__device__ __forceinline__ dfp df_add2(const dfp &a, const dfp &b)
{
    dfp r;
    float2 e;
    two_sum2(a.h, b.h, r.h, e);
    r.l = add2(add2(a.l, b.l), e);
    return r;
}
__device__ __forceinline__ dfp df_neg2(const dfp &a) { return dfp{neg2(a.h), neg2(a.l)}; }

// df_mul per lane: x * y as a fresh accumulator
__device__ __forceinline__ dfp df_mul2(const dfp &x, const dfp &y)
{
    dfp r;
    r.h = mul2(x.h, y.h);
    float2 e = fma2(x.h, y.h, neg2(r.h));
    e = fma2(x.h, y.l, e);
    r.l = fma2(x.l, y.h, e);
    return r;
}

// df_madd per lane: s + x * y
__device__ __forceinline__ dfp df_madd2(const dfp &s, const dfp &x, const dfp &y)
{
    const float2 p = mul2(x.h, y.h);
    float2 l = fma2(x.h, y.h, neg2(p));
    l = fma2(x.h, y.l, l);
    l = fma2(x.l, y.h, l);
    l = add2(l, s.l);
    float2 h, e;
    two_sum2(s.h, p, h, e);
    return dfp{h, add2(l, e)};
}

__device__ __forceinline__ dfp df_norm2(const dfp &a)
{
    dfp r;
    two_sum2(a.h, a.l, r.h, r.l);
    return r;
}

// ---------------------------------------------- complex overloads on pairs
__device__ __forceinline__ dfp c_zero(dfp) { return dfp{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
__device__ __forceinline__ dfp c_add(const dfp &a, const dfp &b) { return df_add2(a, b); }
__device__ __forceinline__ dfp c_sub(const dfp &a, const dfp &b) { return df_add2(a, df_neg2(b)); }
// i a = (-a.im, a.re)
__device__ __forceinline__ dfp c_i(const dfp &a)
{
    return dfp{make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)};
}
// lane views of a complex u: (u.re, u.re), (-u.im, u.im), (u.im, -u.im); swap = (im, re)
__device__ __forceinline__ dfp dup_re(const dfp &u) { return dfp{make_float2(u.h.x, u.h.x), make_float2(u.l.x, u.l.x)}; }
__device__ __forceinline__ dfp nim_im(const dfp &u) { return dfp{make_float2(-u.h.y, u.h.y), make_float2(-u.l.y, u.l.y)}; }
__device__ __forceinline__ dfp im_nim(const dfp &u) { return dfp{make_float2(u.h.y, -u.h.y), make_float2(u.l.y, -u.l.y)}; }
__device__ __forceinline__ dfp swap_ri(const dfp &h) { return dfp{make_float2(h.h.y, h.h.x), make_float2(h.l.y, h.l.x)}; }

// u * h, acc + u * h, conj(u) * h, acc + conj(u) * h: the lane-wise
// equivalents of wd_df.cuh's c_mul / c_madd / c_mulc / c_maddc
__device__ __forceinline__ dfp c_mul(const dfp &u, const dfp &h)
{
    return df_madd2(df_mul2(dup_re(u), h), nim_im(u), swap_ri(h));
}
__device__ __forceinline__ dfp c_madd(const dfp &acc, const dfp &u, const dfp &h)
{
    return df_madd2(df_madd2(acc, dup_re(u), h), nim_im(u), swap_ri(h));
}
__device__ __forceinline__ dfp c_mulc(const dfp &u, const dfp &h)
{
    return df_madd2(df_mul2(dup_re(u), h), im_nim(u), swap_ri(h));
}
__device__ __forceinline__ dfp c_maddc(const dfp &acc, const dfp &u, const dfp &h)
{
    return df_madd2(df_madd2(acc, dup_re(u), h), im_nim(u), swap_ri(h));
}

__device__ __forceinline__ dfp dfp_from_f4(float4 v) { return dfp{make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 dfp_to_f4(const dfp &a)
{
    const dfp n = df_norm2(a);
    return make_float4(n.h.x, n.h.y, n.l.x, n.l.y);
}
