// wd_complex.cuh -- complex arithmetic for the hopping kernels, one overload
// set per arithmetic type, so the spin/colour algebra in wd_hop.cuh is
// written once.
#pragma once
#include <cuda_runtime.h>

// ------------------------------------------------------------ FP64 (double2)
__device__ __forceinline__ double2 c_zero(double2) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double2 c_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 c_sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 c_i(double2 a) { return make_double2(-a.y, a.x); }
__device__ __forceinline__ double2 c_neg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ double2 c_scale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// u * h
__device__ __forceinline__ double2 c_mul(double2 u, double2 h)
{
    return make_double2(fma(-u.y, h.y, u.x * h.x), fma(u.y, h.x, u.x * h.y));
}
// acc + u * h
__device__ __forceinline__ double2 c_madd(double2 acc, double2 u, double2 h)
{
    acc.x = fma(u.x, h.x, acc.x);
    acc.x = fma(-u.y, h.y, acc.x);
    acc.y = fma(u.x, h.y, acc.y);
    acc.y = fma(u.y, h.x, acc.y);
    return acc;
}
// conj(u) * h
__device__ __forceinline__ double2 c_mulc(double2 u, double2 h)
{
    return make_double2(fma(u.y, h.y, u.x * h.x), fma(-u.y, h.x, u.x * h.y));
}
// acc + conj(u) * h
__device__ __forceinline__ double2 c_maddc(double2 acc, double2 u, double2 h)
{
    acc.x = fma(u.x, h.x, acc.x);
    acc.x = fma(u.y, h.y, acc.x);
    acc.y = fma(u.x, h.y, acc.y);
    acc.y = fma(-u.y, h.x, acc.y);
    return acc;
}
// alpha * a + beta * b (epilogue)
__device__ __forceinline__ double2 c_axpby(double alpha, double2 a, double beta, double2 b)
{
    return make_double2(fma(alpha, a.x, beta * b.x), fma(alpha, a.y, beta * b.y));
}
__device__ __forceinline__ double2 c_to_d2(double2 a) { return a; }

// ------------------------------------------------------------- FP32 (float2)
__device__ __forceinline__ float2 c_zero(float2) { return make_float2(0.f, 0.f); }
__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_i(float2 a) { return make_float2(-a.y, a.x); }
__device__ __forceinline__ float2 c_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 c_mul(float2 u, float2 h)
{
    return make_float2(fmaf(-u.y, h.y, u.x * h.x), fmaf(u.y, h.x, u.x * h.y));
}
__device__ __forceinline__ float2 c_madd(float2 acc, float2 u, float2 h)
{
    acc.x = fmaf(u.x, h.x, acc.x);
    acc.x = fmaf(-u.y, h.y, acc.x);
    acc.y = fmaf(u.x, h.y, acc.y);
    acc.y = fmaf(u.y, h.x, acc.y);
    return acc;
}
__device__ __forceinline__ float2 c_mulc(float2 u, float2 h)
{
    return make_float2(fmaf(u.y, h.y, u.x * h.x), fmaf(-u.y, h.x, u.x * h.y));
}
__device__ __forceinline__ float2 c_maddc(float2 acc, float2 u, float2 h)
{
    acc.x = fmaf(u.x, h.x, acc.x);
    acc.x = fmaf(u.y, h.y, acc.x);
    acc.y = fmaf(u.x, h.y, acc.y);
    acc.y = fmaf(-u.y, h.x, acc.y);
    return acc;
}
__device__ __forceinline__ float2 c_axpby(float alpha, float2 a, float beta, float2 b)
{
    return make_float2(fmaf(alpha, a.x, beta * b.x), fmaf(alpha, a.y, beta * b.y));
}
__device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
