// wd_dslash_df.cu -- double-float (df64) hopping kernel.
//
// Same algorithm and memory traffic as the FP64 kernel (1536 B per output
// site: every complex number is a 16-byte float4 {re.h, im.h, re.l, im.l}),
// with the arithmetic moved from the FP64 pipe to the FP32 pipe
// (wd_df.cuh): ~8.5k FP32 operations per site instead of ~790 FP64 ones.
// Results agree with FP64 to ~1e-14 relative L2 (storage rounding 2^-49,
// arithmetic ~2^-48 per operation).
//
// Colour-split mapping: three threads share an output site, one per colour
// c.  Each loads only spin components (k, c) of the neighbour and row c (or
// column c, backward) of the link, projects its colour, and receives the
// other two colours of the half-spinor from its partners by warp shuffles.
// Loads stay non-redundant, registers fall from ~144 to ~90 per thread and
// three times as many threads are in flight to hide memory latency.  A warp
// holds 10 sites (lanes 0-9 colour 0, 10-19 colour 1, 20-29 colour 2).
#include "wd_hop.cuh"
#include "wd_df.cuh"
#include "wd_df2.cuh"
#include "wd_kernels.h"
#include <type_traits>
#include "wd_tune.h"

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSitesPerWarp = 10;

struct SplitDF {
    WdGeom g;
    int cb;
    const float4 *__restrict__ in;
    const float4 *__restrict__ gauge;
    const float4 *__restrict__ x;
    float4 *__restrict__ out;
    dfr alpha, beta;
};

__device__ __forceinline__ dfc shfl_dfc(const dfc &v, int src)
{
    return dfc{{__shfl_sync(kFull, v.re.h, src), __shfl_sync(kFull, v.re.l, src)},
               {__shfl_sync(kFull, v.im.h, src), __shfl_sync(kFull, v.im.l, src)}};
}

__device__ __forceinline__ dfc ld(const float4 *p, size_t i, bool on)
{
    return on ? df_from_f4(p[i]) : c_zero(dfc());
}

template <int MU, bool FWD, bool DAG>
__device__ __forceinline__ void split_dir(const SplitDF &p, int s, const WdSite &cs, int col, int c1, int c2,
                                          int src1, int src2, bool on, dfc *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    const size_t Vh = p.g.Vh;
    const int nb = wd_neighbour(p.g, s, cs, MU, FWD);
    dfc h0, h1;
    {
        const dfc s0 = ld(p.in, (0 + col) * Vh + nb, on), s1 = ld(p.in, (3 + col) * Vh + nb, on);
        const dfc s2 = ld(p.in, (6 + col) * Vh + nb, on), s3 = ld(p.in, (9 + col) * Vh + nb, on);
        wd_proj1<MU, SG>(s0, s1, s2, s3, h0, h1);
    }
    // W[col][b] for b = col, c1, c2: forward row col of U_mu(x); backward
    // conj of column col of U_mu(x - mu)
    const float4 *gb = p.gauge + (size_t)((MU * 2 + (FWD ? p.cb : 1 - p.cb)) * 9) * Vh + (FWD ? s : nb);
    dfc wa, wb, wc;
    if constexpr (FWD) {
        wa = ld(gb, (size_t)(col * 3 + col) * Vh, on);
        wb = ld(gb, (size_t)(col * 3 + c1) * Vh, on);
        wc = ld(gb, (size_t)(col * 3 + c2) * Vh, on);
    } else {
        wa = ld(gb, (size_t)(col * 3 + col) * Vh, on);
        wb = ld(gb, (size_t)(c1 * 3 + col) * Vh, on);
        wc = ld(gb, (size_t)(c2 * 3 + col) * Vh, on);
    }
    const dfc h0b = shfl_dfc(h0, src1), h1b = shfl_dfc(h1, src1);
    const dfc h0c = shfl_dfc(h0, src2), h1c = shfl_dfc(h1, src2);
    dfc t0, t1;
    if constexpr (FWD) {
        t0 = c_madd(c_madd(c_mul(wa, h0), wb, h0b), wc, h0c);
        t1 = c_madd(c_madd(c_mul(wa, h1), wb, h1b), wc, h1c);
    } else {
        t0 = c_maddc(c_maddc(c_mulc(wa, h0), wb, h0b), wc, h0c);
        t1 = c_maddc(c_maddc(c_mulc(wa, h1), wb, h1b), wc, h1c);
    }
    wd_recon1<MU, SG>(t0, t1, acc[0], acc[1], acc[2], acc[3]);
}

// Software-pipelined form: the loads of the next direction are issued
// before the arithmetic of the current one, so two directions' memory
// latency overlap in every warp (more registers, fewer warps).
struct DirLoad {
    dfc s[4];  // spin components (k, col) of the neighbour
    dfc w[3];  // W[col][col], W[col][c1], W[col][c2] as stored (conjugated on use backward)
};

struct SplitCtx {
    int s, col, c1, c2, src1, src2;
    bool on;
    WdSite cs;
};

template <int MU, bool FWD>
__device__ __forceinline__ void split_load(const SplitDF &p, const SplitCtx &x, DirLoad &L)
{
    const size_t Vh = p.g.Vh;
    const int nb = wd_neighbour(p.g, x.s, x.cs, MU, FWD);
#pragma unroll
    for (int k = 0; k < 4; ++k) L.s[k] = ld(p.in, (size_t)(k * 3 + x.col) * Vh + nb, x.on);
    const float4 *gb = p.gauge + (size_t)((MU * 2 + (FWD ? p.cb : 1 - p.cb)) * 9) * Vh + (FWD ? x.s : nb);
    if constexpr (FWD) {
        L.w[0] = ld(gb, (size_t)(x.col * 3 + x.col) * Vh, x.on);
        L.w[1] = ld(gb, (size_t)(x.col * 3 + x.c1) * Vh, x.on);
        L.w[2] = ld(gb, (size_t)(x.col * 3 + x.c2) * Vh, x.on);
    } else {
        L.w[0] = ld(gb, (size_t)(x.col * 3 + x.col) * Vh, x.on);
        L.w[1] = ld(gb, (size_t)(x.c1 * 3 + x.col) * Vh, x.on);
        L.w[2] = ld(gb, (size_t)(x.c2 * 3 + x.col) * Vh, x.on);
    }
}

template <int MU, bool FWD, bool DAG>
__device__ __forceinline__ void split_compute(const SplitCtx &x, const DirLoad &L, dfc *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    dfc h0, h1;
    wd_proj1<MU, SG>(L.s[0], L.s[1], L.s[2], L.s[3], h0, h1);
    const dfc h0b = shfl_dfc(h0, x.src1), h1b = shfl_dfc(h1, x.src1);
    const dfc h0c = shfl_dfc(h0, x.src2), h1c = shfl_dfc(h1, x.src2);
    dfc t0, t1;
    if constexpr (FWD) {
        t0 = c_madd(c_madd(c_mul(L.w[0], h0), L.w[1], h0b), L.w[2], h0c);
        t1 = c_madd(c_madd(c_mul(L.w[0], h1), L.w[1], h1b), L.w[2], h1c);
    } else {
        t0 = c_maddc(c_maddc(c_mulc(L.w[0], h0), L.w[1], h0b), L.w[2], h0c);
        t1 = c_maddc(c_maddc(c_mulc(L.w[0], h1), L.w[1], h1b), L.w[2], h1c);
    }
    wd_recon1<MU, SG>(t0, t1, acc[0], acc[1], acc[2], acc[3]);
}

// L2 prefetch of one direction's operands (the addresses split_load reads):
// no registers held, so the next direction's requests are in flight while
// the current one computes.
__device__ __forceinline__ void pf_l2(const float4 *a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }

template <int MU, bool FWD>
__device__ __forceinline__ void split_prefetch(const SplitDF &p, const SplitCtx &x)
{
    if (!x.on) return;
    const size_t Vh = p.g.Vh;
    const int nb = wd_neighbour(p.g, x.s, x.cs, MU, FWD);
#pragma unroll
    for (int k = 0; k < 4; ++k) pf_l2(p.in + (size_t)(k * 3 + x.col) * Vh + nb);
    const float4 *gb = p.gauge + (size_t)((MU * 2 + (FWD ? p.cb : 1 - p.cb)) * 9) * Vh + (FWD ? x.s : nb);
    if constexpr (FWD) {
        pf_l2(gb + (size_t)(x.col * 3 + x.col) * Vh);
        pf_l2(gb + (size_t)(x.col * 3 + x.c1) * Vh);
        pf_l2(gb + (size_t)(x.col * 3 + x.c2) * Vh);
    } else {
        pf_l2(gb + (size_t)(x.col * 3 + x.col) * Vh);
        pf_l2(gb + (size_t)(x.c1 * 3 + x.col) * Vh);
        pf_l2(gb + (size_t)(x.c2 * 3 + x.col) * Vh);
    }
}

template <bool DAG, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_hop_df_pipe(const SplitDF p)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cq = lane / kSitesPerWarp;
    const int ls = lane - cq * kSitesPerWarp;
    const int s_raw = (blockIdx.x * WARPS + warp) * kSitesPerWarp + ls;
    SplitCtx x;
    x.on = cq < 3 && s_raw < p.g.Vh;
    x.col = cq < 3 ? cq : 0;
    x.s = x.on ? s_raw : 0;
    x.c1 = x.col == 2 ? 0 : x.col + 1;
    x.c2 = x.col == 0 ? 2 : x.col - 1;
    x.src1 = ls + kSitesPerWarp * x.c1;
    x.src2 = ls + kSitesPerWarp * x.c2;
    x.cs = wd_site(p.g, x.s, p.cb);
    dfc acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = c_zero(dfc());
    DirLoad A, B;
    split_load<0, true>(p, x, A);
    split_load<0, false>(p, x, B);
    split_compute<0, true, DAG>(x, A, acc);
    split_load<1, true>(p, x, A);
    split_compute<0, false, DAG>(x, B, acc);
    split_load<1, false>(p, x, B);
    split_compute<1, true, DAG>(x, A, acc);
    split_load<2, true>(p, x, A);
    split_compute<1, false, DAG>(x, B, acc);
    split_load<2, false>(p, x, B);
    split_compute<2, true, DAG>(x, A, acc);
    split_load<3, true>(p, x, A);
    split_compute<2, false, DAG>(x, B, acc);
    split_load<3, false>(p, x, B);
    split_compute<3, true, DAG>(x, A, acc);
    split_compute<3, false, DAG>(x, B, acc);
    if (!x.on) return;
    const size_t Vh = p.g.Vh;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t i = (size_t)(k * 3 + x.col) * Vh + x.s;
        dfc r{df_mul(p.alpha, acc[k].re), df_mul(p.alpha, acc[k].im)};
        if (p.x) {
            const dfc v = df_from_f4(p.x[i]);
            r.re = df_madd(r.re, p.beta, v.re);
            r.im = df_madd(r.im, p.beta, v.im);
        }
        p.out[i] = df_to_f4(r);
    }
}

// Packed form (wd_df2.cuh): the same colour-split, software-pipelined
// kernel with every double-float operation issued on (re, im) pairs -- half
// the arithmetic instructions for the same FP32-pipe work, bit-identical
// results.
struct DirLoadP {
    dfp s[4];
    dfp w[3];
};

__device__ __forceinline__ dfp ldp(const float4 *p, size_t i, bool on)
{
    return on ? dfp_from_f4(p[i]) : c_zero(dfp());
}

__device__ __forceinline__ dfp shfl_dfp(const dfp &v, int src)
{
    return dfp{make_float2(__shfl_sync(kFull, v.h.x, src), __shfl_sync(kFull, v.h.y, src)),
               make_float2(__shfl_sync(kFull, v.l.x, src), __shfl_sync(kFull, v.l.y, src))};
}

template <int MU, bool FWD>
__device__ __forceinline__ void pair_load(const SplitDF &p, const SplitCtx &x, DirLoadP &L)
{
    const size_t Vh = p.g.Vh;
    const int nb = wd_neighbour(p.g, x.s, x.cs, MU, FWD);
#pragma unroll
    for (int k = 0; k < 4; ++k) L.s[k] = ldp(p.in, (size_t)(k * 3 + x.col) * Vh + nb, x.on);
    const float4 *gb = p.gauge + (size_t)((MU * 2 + (FWD ? p.cb : 1 - p.cb)) * 9) * Vh + (FWD ? x.s : nb);
    if constexpr (FWD) {
        L.w[0] = ldp(gb, (size_t)(x.col * 3 + x.col) * Vh, x.on);
        L.w[1] = ldp(gb, (size_t)(x.col * 3 + x.c1) * Vh, x.on);
        L.w[2] = ldp(gb, (size_t)(x.col * 3 + x.c2) * Vh, x.on);
    } else {
        L.w[0] = ldp(gb, (size_t)(x.col * 3 + x.col) * Vh, x.on);
        L.w[1] = ldp(gb, (size_t)(x.c1 * 3 + x.col) * Vh, x.on);
        L.w[2] = ldp(gb, (size_t)(x.c2 * 3 + x.col) * Vh, x.on);
    }
}

template <int MU, bool FWD, bool DAG>
__device__ __forceinline__ void pair_compute(const SplitCtx &x, const DirLoadP &L, dfp *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    dfp h0, h1;
    wd_proj1<MU, SG>(L.s[0], L.s[1], L.s[2], L.s[3], h0, h1);
    const dfp h0b = shfl_dfp(h0, x.src1), h1b = shfl_dfp(h1, x.src1);
    const dfp h0c = shfl_dfp(h0, x.src2), h1c = shfl_dfp(h1, x.src2);
    dfp t0, t1;
    if constexpr (FWD) {
        t0 = c_madd(c_madd(c_mul(L.w[0], h0), L.w[1], h0b), L.w[2], h0c);
        t1 = c_madd(c_madd(c_mul(L.w[0], h1), L.w[1], h1b), L.w[2], h1c);
    } else {
        t0 = c_maddc(c_maddc(c_mulc(L.w[0], h0), L.w[1], h0b), L.w[2], h0c);
        t1 = c_maddc(c_maddc(c_mulc(L.w[0], h1), L.w[1], h1b), L.w[2], h1c);
    }
    wd_recon1<MU, SG>(t0, t1, acc[0], acc[1], acc[2], acc[3]);
}

template <int MU, bool FWD, bool DAG>
__device__ __forceinline__ void pair_dir(const SplitDF &p, const SplitCtx &x, dfp *acc)
{
    DirLoadP L;
    pair_load<MU, FWD>(p, x, L);
    pair_compute<MU, FWD, DAG>(x, L, acc);
}

// PIPE: loads of the next direction issued before the current one's
// arithmetic (in registers); otherwise PF prefetches the next direction into
// L2 instead (no registers held)
template <bool DAG, int WARPS, bool PIPE, bool PF = false>
__device__ __forceinline__ void hop_df_pair_body(const SplitDF &p)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cq = lane / kSitesPerWarp;
    const int ls = lane - cq * kSitesPerWarp;
    const int s_raw = (blockIdx.x * WARPS + warp) * kSitesPerWarp + ls;
    SplitCtx x;
    x.on = cq < 3 && s_raw < p.g.Vh;
    x.col = cq < 3 ? cq : 0;
    x.s = x.on ? s_raw : 0;
    x.c1 = x.col == 2 ? 0 : x.col + 1;
    x.c2 = x.col == 0 ? 2 : x.col - 1;
    x.src1 = ls + kSitesPerWarp * x.c1;
    x.src2 = ls + kSitesPerWarp * x.c2;
    x.cs = wd_site(p.g, x.s, p.cb);
    dfp acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = c_zero(dfp());
    if constexpr (PIPE) {
        DirLoadP A, B;
        pair_load<0, true>(p, x, A);
        pair_load<0, false>(p, x, B);
        pair_compute<0, true, DAG>(x, A, acc);
        pair_load<1, true>(p, x, A);
        pair_compute<0, false, DAG>(x, B, acc);
        pair_load<1, false>(p, x, B);
        pair_compute<1, true, DAG>(x, A, acc);
        pair_load<2, true>(p, x, A);
        pair_compute<1, false, DAG>(x, B, acc);
        pair_load<2, false>(p, x, B);
        pair_compute<2, true, DAG>(x, A, acc);
        pair_load<3, true>(p, x, A);
        pair_compute<2, false, DAG>(x, B, acc);
        pair_load<3, false>(p, x, B);
        pair_compute<3, true, DAG>(x, A, acc);
        pair_compute<3, false, DAG>(x, B, acc);
    } else {
        if constexpr (PF) split_prefetch<0, false>(p, x);
        pair_dir<0, true, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<1, true>(p, x);
        pair_dir<0, false, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<1, false>(p, x);
        pair_dir<1, true, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<2, true>(p, x);
        pair_dir<1, false, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<2, false>(p, x);
        pair_dir<2, true, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<3, true>(p, x);
        pair_dir<2, false, DAG>(p, x, acc);
        if constexpr (PF) split_prefetch<3, false>(p, x);
        pair_dir<3, true, DAG>(p, x, acc);
        pair_dir<3, false, DAG>(p, x, acc);
    }
    if (!x.on) return;
    const size_t Vh = p.g.Vh;
    const dfp al{make_float2(p.alpha.h, p.alpha.h), make_float2(p.alpha.l, p.alpha.l)};
    const dfp be{make_float2(p.beta.h, p.beta.h), make_float2(p.beta.l, p.beta.l)};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t i = (size_t)(k * 3 + x.col) * Vh + x.s;
        dfp r = df_mul2(al, acc[k]);
        if (p.x) r = df_madd2(r, be, dfp_from_f4(p.x[i]));
        p.out[i] = dfp_to_f4(r);
    }
}

template <bool DAG, int WARPS, bool PIPE, bool PF = false>
__global__ void __launch_bounds__(32 * WARPS) k_hop_df_pair(const SplitDF p)
{
    hop_df_pair_body<DAG, WARPS, PIPE, PF>(p);
}

template <bool DAG, int WARPS, int MINB>
__global__ void __launch_bounds__(32 * WARPS, MINB) k_hop_df_split(const SplitDF p)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cq = lane / kSitesPerWarp;          // 0..2, 3 for the two idle lanes
    const int ls = lane - cq * kSitesPerWarp;     // site within the warp
    const int s_raw = (blockIdx.x * WARPS + warp) * kSitesPerWarp + ls;
    const bool on = cq < 3 && s_raw < p.g.Vh;
    const int col = cq < 3 ? cq : 0;
    const int s = on ? s_raw : 0;                 // idle lanes compute on site 0 and store nothing
    const int c1 = col == 2 ? 0 : col + 1, c2 = col == 0 ? 2 : col - 1;
    const int src1 = ls + kSitesPerWarp * c1, src2 = ls + kSitesPerWarp * c2;
    const WdSite cs = wd_site(p.g, s, p.cb);
    dfc acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = c_zero(dfc());
    split_dir<0, true, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<0, false, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<1, true, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<1, false, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<2, true, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<2, false, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<3, true, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    split_dir<3, false, DAG>(p, s, cs, col, c1, c2, src1, src2, on, acc);
    if (!on) return;
    const size_t Vh = p.g.Vh;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t i = (size_t)(k * 3 + col) * Vh + s;
        dfc r{df_mul(p.alpha, acc[k].re), df_mul(p.alpha, acc[k].im)};
        if (p.x) {
            const dfc v = df_from_f4(p.x[i]);
            r.re = df_madd(r.re, p.beta, v.re);
            r.im = df_madd(r.im, p.beta, v.im);
        }
        p.out[i] = df_to_f4(r);
    }
}

__global__ void k_f64_to_df(const double2 *__restrict__ in, float4 *__restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = df_pack(in[i]);
}

__global__ void k_df_to_f64(const float4 *__restrict__ in, double2 *__restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = df_unpack(in[i]);
}

int conv_blocks(int64_t n)
{
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

}  // namespace

wd_status wd_hop_df(wd_context *ctx, const wd_lattice *lat, const float4 *in_block, float4 *out_block,
                    const float4 *x_block, int cb, int dag, double alpha, double beta)
{
    wd_status st = wd_lattice_gauge_df(ctx, lat);
    if (st != WD_OK) return st;
    SplitDF p;
    p.g = lat->g;
    p.cb = cb;
    p.in = in_block;
    p.gauge = lat->gauge_df;
    p.x = x_block;
    p.out = out_block;
    p.alpha = df_split(alpha);
    p.beta = df_split(beta);
    auto run = [&](auto warps, auto minb) -> wd_status {
        constexpr int W = decltype(warps)::value, M = decltype(minb)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        if (dag) k_hop_df_split<true, W, M><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        else k_hop_df_split<false, W, M><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    auto run_pipe = [&](auto warps) -> wd_status {
        constexpr int W = decltype(warps)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        if (dag) k_hop_df_pipe<true, W><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        else k_hop_df_pipe<false, W><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    auto run_pair = [&](auto warps, auto pf) -> wd_status {
        constexpr int W = decltype(warps)::value;
        constexpr bool PF = decltype(pf)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        if (dag) k_hop_df_pair<true, W, false, PF><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        else k_hop_df_pair<false, W, false, PF><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    // variants (ncu at 24^3x48 on GB300 in brackets): software-pipelined with 2
    // and 4 warps per block [0.150 ms, 123.5 M warp instructions, 55 % FMA
    // pipe, 68 % issue]; colour-split at <= 80 registers (6 blocks of 4 warps
    // per SM); packed (re, im) pairs, 2 warps [0.163 ms: 87.7 M instructions
    // but 6.6 long-scoreboard stalls per issue]; packed pairs with an L2
    // prefetch of the next direction [0.153 ms, 100.9 M, stalls 3.5].  Every
    // form tried lands at ~55 % of the FMA pipe.  Dropped: the unbounded
    // colour-split form (242 registers, 0.225 ms), the register-prefetching
    // packed form (0.180 ms), L2 prefetch on the scalar form (0.161 ms), the
    // pipelined form capped at 80 or 72 registers (550-830 bytes of spills;
    // 0.205 and 0.244 ms).
    using F = std::false_type;
    using T = std::true_type;
    using W2 = std::integral_constant<int, 2>;
    return wd_tune_launch(ctx, "hop_df64", lat->g.Vh, 5, [&](int v) -> wd_status {
        if (v == 1) return run_pipe(std::integral_constant<int, 4>());
        if (v == 2) return run(std::integral_constant<int, 4>(), std::integral_constant<int, 6>());
        if (v == 3) return run_pair(W2(), F());
        if (v == 4) return run_pair(W2(), T());
        return run_pipe(W2());
    });
}

wd_status wd_convert_f64_to_df(wd_context *ctx, const double2 *in, float4 *out, int64_t n)
{
    k_f64_to_df<<<conv_blocks(n), 256, 0, ctx->stream>>>(in, out, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_convert_df_to_f64(wd_context *ctx, const float4 *in, double2 *out, int64_t n)
{
    k_df_to_f64<<<conv_blocks(n), 256, 0, ctx->stream>>>(in, out, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// df copy of the resident links, built on first use (wd_lattice_invalidate_derived drops it).
wd_status wd_lattice_gauge_df(wd_context *ctx, const wd_lattice *lat_c)
{
    wd_lattice *lat = const_cast<wd_lattice *>(lat_c);
    if (lat->gauge_df) return WD_OK;
    const int64_t n = lat->volume * 4 * 9;
    WD_CUDA(ctx, cudaMalloc(&lat->gauge_df, n * sizeof(float4)));
    return wd_convert_f64_to_df(ctx, lat->gauge, lat->gauge_df, n);
}
