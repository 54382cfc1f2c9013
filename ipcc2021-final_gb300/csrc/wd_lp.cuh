// wd_lp.cuh -- low-precision storage used by the mixed-precision solvers.
//
// FP32 spinor: 6 planes of float4 per parity, plane j = complex components
//   (2j, 2j+1) as {re, im, re, im}: 96 B/site in six 16-byte loads.
// FP16 spinor: 3 planes of uint4 (8 halves = 4 complex) per parity plus one
//   FP32 scale per site: value = half * scale, scale = max |real| of the
//   site, so every stored half lies in [-1, 1]: 48 + 4 B/site.
// Links (both): 12-real compression, rows 0 and 1 of the SU(3) matrix;
//   row 2 = conj(row0 x row1) is rebuilt in registers (exact for SU(3)).
//   FP32: 3 planes of float4 = 48 B/link.  FP16 (entries bounded by 1, no
//   scale): one uint4 plane (complex 0..3) + one uint2 plane (4..5) = 24 B.
#pragma once
#include <cuda_fp16.h>
#include "wd_internal.cuh"
#include "wd_complex.cuh"
#include "wd_async.cuh"

__device__ __forceinline__ float2 h2f(__half2 h) { return __half22float2(h); }
__device__ __forceinline__ __half2 f2h(float2 f) { return __float22half2_rn(f); }

__device__ __forceinline__ void unpack4(uint4 u, float2 *v)
{
    v[0] = h2f(*reinterpret_cast<__half2 *>(&u.x));
    v[1] = h2f(*reinterpret_cast<__half2 *>(&u.y));
    v[2] = h2f(*reinterpret_cast<__half2 *>(&u.z));
    v[3] = h2f(*reinterpret_cast<__half2 *>(&u.w));
}
__device__ __forceinline__ uint4 pack4(const float2 *v)
{
    uint4 u;
    __half2 h;
    h = f2h(v[0]); u.x = *reinterpret_cast<unsigned *>(&h);
    h = f2h(v[1]); u.y = *reinterpret_cast<unsigned *>(&h);
    h = f2h(v[2]); u.z = *reinterpret_cast<unsigned *>(&h);
    h = f2h(v[3]); u.w = *reinterpret_cast<unsigned *>(&h);
    return u;
}

// ---------------------------------------------------------- spinor sites
struct SpF32 {
    static constexpr bool kScaled = false;
    float4 *p;
    int Vh;
    __device__ __forceinline__ void load(int s, float2 *v) const
    {
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const float4 f = __ldg(p + (size_t)j * Vh + s);
            v[2 * j] = make_float2(f.x, f.y);
            v[2 * j + 1] = make_float2(f.z, f.w);
        }
    }
    __device__ __forceinline__ void store(int s, const float2 *v) const
    {
#pragma unroll
        for (int j = 0; j < 6; ++j)
            p[(size_t)j * Vh + s] = make_float4(v[2 * j].x, v[2 * j].y, v[2 * j + 1].x, v[2 * j + 1].y);
    }
};

struct SpF16 {
    static constexpr bool kScaled = true;
    uint4 *p;
    float *scale;
    int Vh;
    // unscaled components; returns the site's scale
    __device__ __forceinline__ float load_raw(int s, float2 *v) const
    {
#pragma unroll
        for (int j = 0; j < 3; ++j) unpack4(__ldg(p + (size_t)j * Vh + s), v + 4 * j);
        return __ldg(scale + s);
    }
    __device__ __forceinline__ void load(int s, float2 *v) const
    {
        const float sc = load_raw(s, v);
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = make_float2(v[c].x * sc, v[c].y * sc);
    }
    __device__ __forceinline__ void store(int s, const float2 *v) const
    {
        float m = 0.f;
#pragma unroll
        for (int c = 0; c < 12; ++c) m = fmaxf(m, fmaxf(fabsf(v[c].x), fabsf(v[c].y)));
        const float inv = m > 0.f ? 1.0f / m : 0.f;
        float2 w[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) w[c] = make_float2(v[c].x * inv, v[c].y * inv);
#pragma unroll
        for (int j = 0; j < 3; ++j) p[(size_t)j * Vh + s] = pack4(w + 4 * j);
        scale[s] = m;
    }
    // shared-memory slot of T threads for the staged kernel (cp.async):
    // stage() copies site s for thread t (raw halves and the scale)
    template <int T>
    struct Slot {
        uint4 v[3][T];
        float sc[T];
    };
    template <int T>
    __device__ __forceinline__ void stage(int s, Slot<T> &S, int t) const
    {
#pragma unroll
        for (int j = 0; j < 3; ++j) wd_cp_async_ca<16>(&S.v[j][t], p + (size_t)j * Vh + s);
        wd_cp_async_ca<4>(&S.sc[t], scale + s);
    }
};

inline SpF32 sp_f32(WdVec v, int Vh) { return SpF32{(float4 *)v.p, Vh}; }
inline SpF16 sp_f16(WdVec v, int Vh) { return SpF16{(uint4 *)v.p, v.scale, Vh}; }

// ------------------------------------------------------------ links (12-real)
__device__ __forceinline__ void su3_row2(float2 *U)
{
    // U[6..8] = conj(row0 x row1), with explicit FMAs (c_mul) so every kernel
    // that rebuilds a link rounds it identically
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a = (k + 1) % 3, b = (k + 2) % 3;
        const float2 p = c_mul(U[a], U[3 + b]);
        const float2 q = c_mul(U[b], U[3 + a]);
        U[6 + k] = make_float2(p.x - q.x, q.y - p.y);
    }
}

struct LinkF32 {
    const float4 *g;  // [mu][par][3][Vh]
    int Vh;
    __device__ __forceinline__ void load(int mu, int par, int s, float2 *U) const
    {
        const float4 *b = g + (size_t)((mu * 2 + par) * 3) * Vh + s;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float4 f = __ldg(b + (size_t)j * Vh);
            U[2 * j] = make_float2(f.x, f.y);
            U[2 * j + 1] = make_float2(f.z, f.w);
        }
        su3_row2(U);
    }
};

struct LinkF16 {
    const uint4 *a;  // [mu][par][Vh] complex 0..3
    const uint2 *b;  // [mu][par][Vh] complex 4..5
    int Vh;
    __device__ __forceinline__ void load(int mu, int par, int s, float2 *U) const
    {
        const size_t i = (size_t)(mu * 2 + par) * Vh + s;
        unpack4(__ldg(a + i), U);
        const uint2 v = __ldg(b + i);
        U[4] = h2f(*reinterpret_cast<const __half2 *>(&v.x));
        U[5] = h2f(*reinterpret_cast<const __half2 *>(&v.y));
        su3_row2(U);
    }
    // staged copies: the 16-byte part L2-only (each link entry is read once
    // per application; cp.async.cg takes 16 bytes only), the 8-byte part via L1
    template <int T>
    struct Slot {
        uint4 a[T];
        uint2 b[T];
    };
    template <int T>
    __device__ __forceinline__ void stage(int mu, int par, int s, Slot<T> &S, int t) const
    {
        const size_t i = (size_t)(mu * 2 + par) * Vh + s;
        wd_cp_async_cg16(&S.a[t], a + i);
        wd_cp_async_ca<8>(&S.b[t], b + i);
    }
};
