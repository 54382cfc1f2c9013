// wd_h16m.cuh -- the FP16 hopping arithmetic on FP16 operands.
//
// The storage of wd_lp.cuh (FP16 spinors with a per-site scale, 12-real FP16
// links), computed without converting operands to FP32 first:
//   * the spin projection h = P psi in half2 arithmetic (one rounding to FP16
//     per component, the precision of the stored spinor itself);
//   * the SU(3) products W h by mixed-precision FMAs (fma.rn.f32.f16: the
//     product of two FP16 values is exact in FP32 and is accumulated in FP32),
//     so neither the links nor the projected spinor are converted;
//   * row 2 of the link, conj(row0 x row1), from the same mixed FMAs, rounded
//     once to FP16;
//   * the accumulation over the eight directions, with the neighbour's scale,
//     in FP32 as in the FP32-arithmetic kernel.
// Sums that carry a minus sign are accumulated in two FP32 chains and
// subtracted once, so no FP16 operand needs negating.
#pragma once
#include <cuda_fp16.h>
#include "wd_hop.cuh"
#include "wd_lp.cuh"
#include "wd_lp_staged.cuh"

__device__ __forceinline__ unsigned wd_h2u(__half2 h) { return *reinterpret_cast<unsigned *>(&h); }

// a.{x,y} * b.{x,y} + c with a single FP32 rounding (a, b: half2 bit patterns)
#define WD_FMAH(NAME, AS, BS)                                                                              \
    __device__ __forceinline__ float NAME(unsigned a, unsigned b, float c)                                 \
    {                                                                                                      \
        float d;                                                                                           \
        asm("{.reg .f16 a0, a1, b0, b1;\n\tmov.b32 {a0, a1}, %1;\n\tmov.b32 {b0, b1}, %2;\n\t"             \
            "fma.rn.f32.f16 %0, " AS ", " BS ", %3;\n\t}"                                                  \
            : "=f"(d)                                                                                      \
            : "r"(a), "r"(b), "f"(c));                                                                     \
        return d;                                                                                          \
    }
WD_FMAH(wd_fmah_xx, "a0", "b0")
WD_FMAH(wd_fmah_xy, "a0", "b1")
WD_FMAH(wd_fmah_yx, "a1", "b0")
WD_FMAH(wd_fmah_yy, "a1", "b1")
#undef WD_FMAH

// a + SG i z in half2: (x, y) -> (-SG y, SG x) + a
template <int SG>
__device__ __forceinline__ __half2 h16_add_i(__half2 a, __half2 z)
{
    const __half2 k = __floats2half2_rn((float)-SG, (float)SG);
    return __hfma2(__lowhigh2highlow(z), k, a);
}
template <int SG>
__device__ __forceinline__ __half2 h16_add(__half2 a, __half2 z)
{
    if constexpr (SG > 0) return __hadd2(a, z);
    else return __hsub2(a, z);
}

// spin projection of one colour (the table of wd_proj1), in half2
template <int MU, int SG>
__device__ __forceinline__ void h16_proj1(__half2 s0, __half2 s1, __half2 s2, __half2 s3, __half2 &h0, __half2 &h1)
{
    if constexpr (MU == 0) {
        h0 = h16_add_i<SG>(s0, s3);
        h1 = h16_add_i<SG>(s1, s2);
    } else if constexpr (MU == 1) {
        h0 = h16_add<-SG>(s0, s3);
        h1 = h16_add<SG>(s1, s2);
    } else if constexpr (MU == 2) {
        h0 = h16_add_i<SG>(s0, s2);
        h1 = h16_add_i<-SG>(s1, s3);
    } else {
        h0 = h16_add<SG>(s0, s2);
        h1 = h16_add<SG>(s1, s3);
    }
}

// row 2 of a 12-real link: conj(row0 x row1), rounded to FP16 (U: half2 bits)
__device__ __forceinline__ void h16_row2(unsigned *U)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a = (k + 1) % 3, b = (k + 2) % 3;
        const unsigned ua = U[a], ub = U[b], va = U[3 + a], vb = U[3 + b];
        const float P = wd_fmah_yy(ub, va, wd_fmah_xx(ua, vb, 0.f));
        const float Q = wd_fmah_xx(ub, va, wd_fmah_yy(ua, vb, 0.f));
        const float R = wd_fmah_yx(ub, va, wd_fmah_xy(ub, va, 0.f));
        const float S = wd_fmah_yx(ua, vb, wd_fmah_xy(ua, vb, 0.f));
        U[6 + k] = wd_h2u(__floats2half2_rn(P - Q, R - S));
    }
}

// t = W h for one row a: forward W = U[a][.], backward W = conj(U[.][a])
template <bool FWD>
__device__ __forceinline__ float2 h16_row(const unsigned *U, int a, const unsigned *h)
{
    if constexpr (FWD) {
        const unsigned u0 = U[a * 3], u1 = U[a * 3 + 1], u2 = U[a * 3 + 2];
        const float p = wd_fmah_xx(u2, h[2], wd_fmah_xx(u1, h[1], wd_fmah_xx(u0, h[0], 0.f)));
        const float m = wd_fmah_yy(u2, h[2], wd_fmah_yy(u1, h[1], wd_fmah_yy(u0, h[0], 0.f)));
        float im = wd_fmah_yx(u0, h[0], wd_fmah_xy(u0, h[0], 0.f));
        im = wd_fmah_yx(u1, h[1], wd_fmah_xy(u1, h[1], im));
        im = wd_fmah_yx(u2, h[2], wd_fmah_xy(u2, h[2], im));
        return make_float2(p - m, im);
    } else {
        const unsigned u0 = U[a], u1 = U[3 + a], u2 = U[6 + a];
        float re = wd_fmah_yy(u0, h[0], wd_fmah_xx(u0, h[0], 0.f));
        re = wd_fmah_yy(u1, h[1], wd_fmah_xx(u1, h[1], re));
        re = wd_fmah_yy(u2, h[2], wd_fmah_xx(u2, h[2], re));
        const float p = wd_fmah_xy(u2, h[2], wd_fmah_xy(u1, h[1], wd_fmah_xy(u0, h[0], 0.f)));
        const float m = wd_fmah_yx(u2, h[2], wd_fmah_yx(u1, h[1], wd_fmah_yx(u0, h[0], 0.f)));
        return make_float2(re, p - m);
    }
}

// the terms of one of the eight neighbours: sp = its 12 components (half2
// bits, index spin*3 + colour), sc its scale, U the link (rows 0, 1; row 2
// is filled here, or, ROW2 = false, already filled by the caller)
template <int MU, bool FWD, bool DAG, bool ROW2 = true>
__device__ __forceinline__ void h16_dir_terms(const unsigned *sp, float sc, unsigned *U, float2 *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    unsigned h0[3], h1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        __half2 a, b;
        h16_proj1<MU, SG>(*reinterpret_cast<const __half2 *>(&sp[k]), *reinterpret_cast<const __half2 *>(&sp[3 + k]),
                          *reinterpret_cast<const __half2 *>(&sp[6 + k]),
                          *reinterpret_cast<const __half2 *>(&sp[9 + k]), a, b);
        h0[k] = wd_h2u(a);
        h1[k] = wd_h2u(b);
    }
    if constexpr (ROW2) h16_row2(U);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float2 t0 = h16_row<FWD>(U, a, h0), t1 = h16_row<FWD>(U, a, h1);
        wd_recon1_scaled<MU, SG>(t0, t1, sc, acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
    }
}

template <int D, bool DAG, class P, class S>
__device__ __forceinline__ void h16_compute_dir(const P &p, const S &st, int slot, float2 *acc)
{
    const int t = threadIdx.x;
    unsigned sp[12], U[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const uint4 v = st.sp[slot].v[j][t];
        sp[4 * j] = v.x, sp[4 * j + 1] = v.y, sp[4 * j + 2] = v.z, sp[4 * j + 3] = v.w;
    }
    const float sc = st.sp[slot].sc[t];
    const uint4 la = st.lk[slot].a[t];
    const uint2 lb = st.lk[slot].b[t];
    U[0] = la.x, U[1] = la.y, U[2] = la.z, U[3] = la.w, U[4] = lb.x, U[5] = lb.y;
    h16_dir_terms<D / 2, (D % 2) == 0, DAG>(sp, sc, U, acc);
}

template <int D, bool DAG, class P, class S>
__device__ __forceinline__ void h16_step(const P &p, int s, const WdSite &c, S &st, float2 *acc)
{
    if constexpr (D + 1 < 8) lp_stage_dir<D + 1>(p, s, c, st, (D + 1) & 1);
    wd_cp_async_commit();  // possibly empty: one group per step keeps the count
    wd_cp_async_wait<1>();
    h16_compute_dir<D, DAG>(p, st, D & 1, acc);
}

// acc = sum over the eight neighbours of FP16 output site s, operands staged
// as in lp_hop_site_staged
template <bool DAG, class P, class S>
__device__ __forceinline__ void h16_hop_site_staged(const P &p, int s, float2 *acc, S &st)
{
    const WdSite c = wd_site(p.g, s, p.cb);
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = make_float2(0.f, 0.f);
    lp_stage_dir<0>(p, s, c, st, 0);
    wd_cp_async_commit();
    h16_step<0, DAG>(p, s, c, st, acc);
    h16_step<1, DAG>(p, s, c, st, acc);
    h16_step<2, DAG>(p, s, c, st, acc);
    h16_step<3, DAG>(p, s, c, st, acc);
    h16_step<4, DAG>(p, s, c, st, acc);
    h16_step<5, DAG>(p, s, c, st, acc);
    h16_step<6, DAG>(p, s, c, st, acc);
    h16_step<7, DAG>(p, s, c, st, acc);
}

// Register-loading form (the batched kernel): the operands of direction D
// loaded straight from global memory.  P supplies g, cb, in (SpF16) and link
// (LinkF16).
template <int D, bool DAG, class P>
__device__ __forceinline__ void h16_dir(const P &p, int s, const WdSite &c, float2 *acc)
{
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    const int nb = wd_neighbour(p.g, s, c, MU, FWD);
    const size_t Vh = p.g.Vh;
    unsigned sp[12], U[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const uint4 v = __ldg(p.in.p + (size_t)j * Vh + nb);
        sp[4 * j] = v.x, sp[4 * j + 1] = v.y, sp[4 * j + 2] = v.z, sp[4 * j + 3] = v.w;
    }
    const float sc = __ldg(p.in.scale + nb);
    // forward: U_mu(x) stored at this site (parity cb); backward: U_mu(x - mu) at the neighbour
    const size_t i = (size_t)(MU * 2 + (FWD ? p.cb : 1 - p.cb)) * Vh + (FWD ? s : nb);
    const uint4 la = __ldg(p.link.a + i);
    const uint2 lb = __ldg(p.link.b + i);
    U[0] = la.x, U[1] = la.y, U[2] = la.z, U[3] = la.w, U[4] = lb.x, U[5] = lb.y;
    h16_dir_terms<MU, FWD, DAG>(sp, sc, U, acc);
}

template <bool DAG, class P>
__device__ __forceinline__ void h16_hop_site(const P &p, int s, float2 *acc)
{
    const WdSite c = wd_site(p.g, s, p.cb);
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = make_float2(0.f, 0.f);
    h16_dir<0, DAG>(p, s, c, acc);
    h16_dir<1, DAG>(p, s, c, acc);
    h16_dir<2, DAG>(p, s, c, acc);
    h16_dir<3, DAG>(p, s, c, acc);
    h16_dir<4, DAG>(p, s, c, acc);
    h16_dir<5, DAG>(p, s, c, acc);
    h16_dir<6, DAG>(p, s, c, acc);
    h16_dir<7, DAG>(p, s, c, acc);
}

// Shared-row-2 form (the batched kernel, several systems over the same 32
// sites): row 2 of the link of direction D at this thread's site is read
// from r2[D][k][lane], filled once per block by h16_fill_row2, instead of
// being rebuilt by every system.  Same arithmetic and rounding as h16_dir.
template <int D, bool DAG, class P>
__device__ __forceinline__ void h16_dir_r2(const P &p, int s, const WdSite &c, const unsigned (*r2)[3][32],
                                           int lane, float2 *acc)
{
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    const int nb = wd_neighbour(p.g, s, c, MU, FWD);
    const size_t Vh = p.g.Vh;
    unsigned sp[12], U[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const uint4 v = __ldg(p.in.p + (size_t)j * Vh + nb);
        sp[4 * j] = v.x, sp[4 * j + 1] = v.y, sp[4 * j + 2] = v.z, sp[4 * j + 3] = v.w;
    }
    const float sc = __ldg(p.in.scale + nb);
    const size_t i = (size_t)(MU * 2 + (FWD ? p.cb : 1 - p.cb)) * Vh + (FWD ? s : nb);
    const uint4 la = __ldg(p.link.a + i);
    const uint2 lb = __ldg(p.link.b + i);
    U[0] = la.x, U[1] = la.y, U[2] = la.z, U[3] = la.w, U[4] = lb.x, U[5] = lb.y;
    U[6] = r2[D][0][lane], U[7] = r2[D][1][lane], U[8] = r2[D][2][lane];
    h16_dir_terms<MU, FWD, DAG, false>(sp, sc, U, acc);
}

template <bool DAG, class P>
__device__ __forceinline__ void h16_hop_site_r2(const P &p, int s, const unsigned (*r2)[3][32], int lane,
                                                float2 *acc)
{
    const WdSite c = wd_site(p.g, s, p.cb);
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = make_float2(0.f, 0.f);
    h16_dir_r2<0, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<1, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<2, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<3, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<4, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<5, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<6, DAG>(p, s, c, r2, lane, acc);
    h16_dir_r2<7, DAG>(p, s, c, r2, lane, acc);
}

// Row 2 of the link of direction D at site s (parity cb output), rebuilt as
// h16_dir_terms rebuilds it, into r2[D][k][lane].
template <int D>
__device__ __forceinline__ void h16_fill_row2_dir(const WdGeom &g, int cb, const LinkF16 &link, int s,
                                                  const WdSite &c, unsigned (*r2)[3][32], int lane)
{
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    const size_t i = (size_t)(MU * 2 + (FWD ? cb : 1 - cb)) * g.Vh + (FWD ? s : wd_neighbour(g, s, c, MU, false));
    const uint4 la = __ldg(link.a + i);
    const uint2 lb = __ldg(link.b + i);
    unsigned U[9] = {la.x, la.y, la.z, la.w, lb.x, lb.y, 0u, 0u, 0u};
    h16_row2(U);
    r2[D][0][lane] = U[6], r2[D][1][lane] = U[7], r2[D][2][lane] = U[8];
}

// Fill the block's row-2 table for the site of each lane: warp w of NW takes
// directions w, w + NW, ...
template <int NW>
__device__ __forceinline__ void h16_fill_row2(const WdGeom &g, int cb, const LinkF16 &link, int s,
                                              unsigned (*r2)[3][32], int warp, int lane)
{
    const WdSite c = wd_site(g, s, cb);
#pragma unroll
    for (int d = 0; d < 8; ++d)
        if (d % NW == warp) {
            switch (d) {
            case 0: h16_fill_row2_dir<0>(g, cb, link, s, c, r2, lane); break;
            case 1: h16_fill_row2_dir<1>(g, cb, link, s, c, r2, lane); break;
            case 2: h16_fill_row2_dir<2>(g, cb, link, s, c, r2, lane); break;
            case 3: h16_fill_row2_dir<3>(g, cb, link, s, c, r2, lane); break;
            case 4: h16_fill_row2_dir<4>(g, cb, link, s, c, r2, lane); break;
            case 5: h16_fill_row2_dir<5>(g, cb, link, s, c, r2, lane); break;
            case 6: h16_fill_row2_dir<6>(g, cb, link, s, c, r2, lane); break;
            default: h16_fill_row2_dir<7>(g, cb, link, s, c, r2, lane); break;
            }
        }
}
