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
//
// Three kernels, bit-identical to each other:
//   k_hop_df_staged  each thread copies the next direction's seven operands
//                    into shared memory with cp.async while it computes the
//                    current one with the packed (re, im) arithmetic of
//                    wd_df2.cuh (half the instructions);
//   k_hop_df_grouped the same staging and arithmetic with a colour per warp:
//                    three warps share 32 sites and exchange half-spinors
//                    through shared memory, so no lane idles (the fastest on
//                    GB300);
//   k_hop_df_pipe    scalar arithmetic, the next direction's operands loaded
//                    into registers ahead of use.
#include "wd_hop.cuh"
#include "wd_df.cuh"
#include "wd_df2.cuh"
#include "wd_async.cuh"
#include "wd_kernels.h"
#include "wd_reduce.cuh"
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

// this thread's site, colour and shuffle partners (colour-split mapping)
template <int WARPS>
__device__ __forceinline__ SplitCtx split_ctx(const SplitDF &p)
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
    return x;
}

template <bool DAG, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_hop_df_pipe(const SplitDF p)
{
    const SplitCtx x = split_ctx<WARPS>(p);
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

// Packed arithmetic (wd_df2.cuh): every double-float operation issued on
// (re, im) pairs -- half the arithmetic instructions for the same FP32-pipe
// work, lane by lane the roundings of the scalar form.
struct DirLoadP {
    dfp s[4];
    dfp w[3];
};

__device__ __forceinline__ dfp shfl_dfp(const dfp &v, int src)
{
    return dfp{make_float2(__shfl_sync(kFull, v.h.x, src), __shfl_sync(kFull, v.h.y, src)),
               make_float2(__shfl_sync(kFull, v.l.x, src), __shfl_sync(kFull, v.l.y, src))};
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

// out = alpha acc (+ beta x) for this thread's colour of its site
__device__ __forceinline__ void pair_epilogue(const SplitDF &p, const SplitCtx &x, const dfp *acc)
{
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

// Staged packed form: each thread copies its own operands of the next LOOK
// directions into shared memory with cp.async (no registers held while the
// copies are in flight), then computes the current direction from shared
// memory with the packed arithmetic (pair_compute: bit-identical to the other
// forms).  A thread reads back only what it copied itself, so no block
// barrier is needed: cp.async.wait_group makes a thread's completed copies
// visible to it.  NS >= LOOK + 1 slots per thread; a slot is refilled
// NS - LOOK directions after it was read.  Every address copied is one the
// register-loading forms read (idle lanes use site 0), so all are in bounds.
constexpr int kOps = 7;  // float4 operands per thread and direction: 4 spinor components, 3 link entries

// spinors through L1 (each is read by eight output sites), links L2-only
// (each entry is read once per application)
__device__ __forceinline__ void cp_async16(float4 *smem, const float4 *gmem) { wd_cp_async_ca<16>(smem, gmem); }
template <bool L2ONLY>
__device__ __forceinline__ void cp_async16_link(float4 *smem, const float4 *gmem)
{
    if constexpr (L2ONLY) wd_cp_async_cg16(smem, gmem);
    else wd_cp_async_ca<16>(smem, gmem);
}

// direction D = 2 mu + (0 forward, 1 backward): copy its operands into slot
template <int D, bool LCG>
__device__ __forceinline__ void stage_issue(const SplitDF &p, const SplitCtx &x, float4 *slot, int stride)
{
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    const size_t Vh = p.g.Vh;
    const int nb = wd_neighbour(p.g, x.s, x.cs, MU, FWD);
#pragma unroll
    for (int k = 0; k < 4; ++k) cp_async16(slot + k * stride, p.in + (size_t)(k * 3 + x.col) * Vh + nb);
    const float4 *gb = p.gauge + (size_t)((MU * 2 + (FWD ? p.cb : 1 - p.cb)) * 9) * Vh + (FWD ? x.s : nb);
    if constexpr (FWD) {
        cp_async16_link<LCG>(slot + 4 * stride, gb + (size_t)(x.col * 3 + x.col) * Vh);
        cp_async16_link<LCG>(slot + 5 * stride, gb + (size_t)(x.col * 3 + x.c1) * Vh);
        cp_async16_link<LCG>(slot + 6 * stride, gb + (size_t)(x.col * 3 + x.c2) * Vh);
    } else {
        cp_async16_link<LCG>(slot + 4 * stride, gb + (size_t)(x.col * 3 + x.col) * Vh);
        cp_async16_link<LCG>(slot + 5 * stride, gb + (size_t)(x.c1 * 3 + x.col) * Vh);
        cp_async16_link<LCG>(slot + 6 * stride, gb + (size_t)(x.c2 * 3 + x.col) * Vh);
    }
}

template <int D, bool DAG>
__device__ __forceinline__ void stage_compute(const SplitCtx &x, const float4 *slot, int stride, dfp *acc)
{
    DirLoadP L;
#pragma unroll
    for (int k = 0; k < 4; ++k) L.s[k] = dfp_from_f4(slot[k * stride]);
#pragma unroll
    for (int k = 0; k < 3; ++k) L.w[k] = dfp_from_f4(slot[(4 + k) * stride]);
    pair_compute<D / 2, (D % 2) == 0, DAG>(x, L, acc);
}

template <int D, bool DAG, int LOOK, int NS, bool LCG>
__device__ __forceinline__ void stage_step(const SplitDF &p, const SplitCtx &x, float4 *base, int stride, dfp *acc)
{
    if constexpr (D + LOOK < 8) stage_issue<D + LOOK, LCG>(p, x, base + ((D + LOOK) % NS) * kOps * stride, stride);
    wd_cp_async_commit();  // possibly empty: one group per step keeps the count
    wd_cp_async_wait<LOOK>();
    stage_compute<D, DAG>(x, base + (D % NS) * kOps * stride, stride, acc);
}

// this thread's colour of the hopping sum at its site (staged, packed)
template <bool DAG, int WARPS, int LOOK, int NS, bool LCG>
__device__ __forceinline__ void df_staged_site(const SplitDF &p, const SplitCtx &x, dfp *acc)
{
    static_assert(LOOK >= 1 && NS >= LOOK + 1, "slot count");
    __shared__ float4 slots[NS * kOps * 32 * WARPS];
    constexpr int stride = 32 * WARPS;
    float4 *base = slots + threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = c_zero(dfp());
    stage_issue<0, LCG>(p, x, base, stride);
    wd_cp_async_commit();
    if constexpr (LOOK >= 2) {
        stage_issue<1, LCG>(p, x, base + (1 % NS) * kOps * stride, stride);
        wd_cp_async_commit();
    }
    stage_step<0, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<1, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<2, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<3, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<4, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<5, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<6, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
    stage_step<7, DAG, LOOK, NS, LCG>(p, x, base, stride, acc);
}

template <bool DAG, int WARPS, int LOOK, int NS, bool LCG>
__global__ void __launch_bounds__(32 * WARPS) k_hop_df_staged(const SplitDF p)
{
    const SplitCtx x = split_ctx<WARPS>(p);
    dfp acc[4];
    df_staged_site<DAG, WARPS, LOOK, NS, LCG>(p, x, acc);
    pair_epilogue(p, x, acc);
}

// Grouped colour split: three warps per 32 sites, warp w of a group holding
// colour w of each of its 32 sites, so every lane works (the 10-sites-a-warp
// split leaves lanes 30-31 idle: 1/16 of the FP32 pipe, which bounds this
// kernel).  The projected half-spinors go to the partner colours through
// shared memory instead of by warp shuffles: one named barrier per direction
// and group, two buffers alternating by direction, so a buffer is rewritten
// only after every partner has passed the next direction's barrier (and so
// has finished reading it).  Operands are staged as in df_staged_site and the
// arithmetic is pair_compute's, in the same order: bit-identical results.
template <int GROUPS>
__device__ __forceinline__ SplitCtx group_ctx(const SplitDF &p)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = warp / 3;
    const int s_raw = (blockIdx.x * GROUPS + grp) * 32 + lane;
    SplitCtx x;
    x.on = s_raw < p.g.Vh;
    x.col = warp - 3 * grp;
    x.s = x.on ? s_raw : 0;
    x.c1 = x.col == 2 ? 0 : x.col + 1;
    x.c2 = x.col == 0 ? 2 : x.col - 1;
    x.src1 = (3 * grp + x.c1) * 32 + lane;  // partner threads in the block
    x.src2 = (3 * grp + x.c2) * 32 + lane;
    x.cs = wd_site(p.g, x.s, p.cb);
    return x;
}

__device__ __forceinline__ float4 dfp_raw(const dfp &v) { return make_float4(v.h.x, v.h.y, v.l.x, v.l.y); }
__device__ __forceinline__ dfp dfp_unraw(float4 v) { return dfp{make_float2(v.x, v.y), make_float2(v.z, v.w)}; }

// xb: this direction's exchange buffer, h0 of every thread then h1 (T threads)
template <int MU, bool FWD, bool DAG, int T>
__device__ __forceinline__ void group_compute(const SplitCtx &x, const DirLoadP &L, float4 *xb, dfp *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    dfp h0, h1;
    wd_proj1<MU, SG>(L.s[0], L.s[1], L.s[2], L.s[3], h0, h1);
    xb[threadIdx.x] = dfp_raw(h0);
    xb[T + threadIdx.x] = dfp_raw(h1);
    asm volatile("bar.sync %0, 96;" ::"r"(1 + (int)(threadIdx.x >> 5) / 3) : "memory");
    const dfp h0b = dfp_unraw(xb[x.src1]), h1b = dfp_unraw(xb[T + x.src1]);
    const dfp h0c = dfp_unraw(xb[x.src2]), h1c = dfp_unraw(xb[T + x.src2]);
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

template <int D, bool DAG, int T, bool LCG>
__device__ __forceinline__ void group_step(const SplitDF &p, const SplitCtx &x, float4 *base, float4 *xch, dfp *acc)
{
    constexpr int NS = 2;
    if constexpr (D + 1 < 8) stage_issue<D + 1, LCG>(p, x, base + ((D + 1) % NS) * kOps * T, T);
    wd_cp_async_commit();  // possibly empty: one group per step keeps the count
    wd_cp_async_wait<1>();
    DirLoadP L;
    const float4 *slot = base + (D % NS) * kOps * T;
#pragma unroll
    for (int k = 0; k < 4; ++k) L.s[k] = dfp_from_f4(slot[k * T]);
#pragma unroll
    for (int k = 0; k < 3; ++k) L.w[k] = dfp_from_f4(slot[(4 + k) * T]);
    group_compute<D / 2, (D % 2) == 0, DAG, T>(x, L, xch + (D & 1) * 2 * T, acc);
}

// this thread's colour of the hopping sum at its site (grouped split)
template <bool DAG, int GROUPS, bool LCG>
__device__ __forceinline__ void df_group_site(const SplitDF &p, const SplitCtx &x, dfp *acc)
{
    constexpr int T = 96 * GROUPS;
    __shared__ float4 slots[2 * kOps * T];
    __shared__ float4 xch[2 * 2 * T];
    float4 *base = slots + threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = c_zero(dfp());
    stage_issue<0, LCG>(p, x, base, T);
    wd_cp_async_commit();
    group_step<0, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<1, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<2, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<3, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<4, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<5, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<6, DAG, T, LCG>(p, x, base, xch, acc);
    group_step<7, DAG, T, LCG>(p, x, base, xch, acc);
}

// GROUPS groups a block, registers capped for MINB blocks per SM
template <bool DAG, int GROUPS, bool LCG, int MINB>
__global__ void __launch_bounds__(96 * GROUPS, MINB) k_hop_df_grouped(const SplitDF p)
{
    const SplitCtx x = group_ctx<GROUPS>(p);
    dfp acc[4];
    df_group_site<DAG, GROUPS, LCG>(p, x, acc);
    pair_epilogue(p, x, acc);
}

// The reliable update's second Schur hop fused with the true residual
// (wd_hop_hi_residual): s = bhat - (alpha acc + beta x) in double-float,
// rounded to FP32 into s32 (plane c/2, half c&1 of the float4 for component
// c), |s32|^2 reduced over the grid into *result.
struct ResSinkDF {
    const float4 *bhat;
    float4 *s32;
    double *partial;
    unsigned *counter;
    double *result;
};

// WARPS warps of the 10-sites-a-warp split, or (GROUPED) WARPS / 3 groups of
// the grouped split
template <int WARPS, bool LCG, bool GROUPED = false, int MINB = 0>
__global__ void __launch_bounds__(32 * WARPS, MINB) k_hop_df_res(const SplitDF p, const ResSinkDF r)
{
    const SplitCtx x = GROUPED ? group_ctx<WARPS / 3>(p) : split_ctx<WARPS>(p);
    dfp acc[4];
    if constexpr (GROUPED) df_group_site<false, WARPS / 3, LCG>(p, x, acc);
    else df_staged_site<false, WARPS, 1, 2, LCG>(p, x, acc);
    float n = 0.f;
    if (x.on) {
        const size_t Vh = p.g.Vh;
        const dfp al{make_float2(p.alpha.h, p.alpha.h), make_float2(p.alpha.l, p.alpha.l)};
        const dfp be{make_float2(p.beta.h, p.beta.h), make_float2(p.beta.l, p.beta.l)};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = k * 3 + x.col;
            const size_t i = (size_t)c * Vh + x.s;
            const dfp o = df_madd2(df_mul2(al, acc[k]), be, dfp_from_f4(p.x[i]));
            const dfp sd = df_add2(dfp_from_f4(r.bhat[i]), df_neg2(o));
            const float2 v = make_float2(__fadd_rn(sd.h.x, sd.l.x), __fadd_rn(sd.h.y, sd.l.y));
            reinterpret_cast<float2 *>(r.s32 + (size_t)(c >> 1) * Vh + x.s)[c & 1] = v;
            n = fmaf(v.x, v.x, fmaf(v.y, v.y, n));
        }
    }
    double tot;
    if (wd_grid_sum<32 * WARPS>((double)n, r.partial, r.counter, &tot)) *r.result = tot;
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
    auto run_pipe = [&](auto warps) -> wd_status {
        constexpr int W = decltype(warps)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        if (dag) k_hop_df_pipe<true, W><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        else k_hop_df_pipe<false, W><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    auto run_staged = [&](auto warps, auto lcg) -> wd_status {
        constexpr int W = decltype(warps)::value;
        constexpr bool LCG = decltype(lcg)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        if (dag) k_hop_df_staged<true, W, 1, 2, LCG><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        else k_hop_df_staged<false, W, 1, 2, LCG><<<blocks, 32 * W, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    // Variants, D_eo on GB300 at 32^3x64 / 24^3x48 (CUDA events, best of 3x50):
    //   0  staged, 4 warps, links copied L2-only   378.5 / 123.0 us
    //   1  staged, 2 warps, links copied L2-only   383.2 / 123.3 us
    //   2  staged, 2 warps, links through L1       386.2 / 127.0 us
    //   3  register-pipelined scalar, 2 warps      459.9 / 150.1 us
    //   4  register-pipelined scalar, 4 warps      459.0 / 149.5 us
    //   5  grouped split, 2 groups, 4 blocks/SM    345.8 us (1.741 ms at 48^3x96 against 1.900 for 0)
    // Dropped (same lattices): the grouped split with 1 group (389 us), 2
    // groups without the register cap (96 registers, 353 us) or 4 groups
    // (414 us), with a split-phase exchange on mbarriers (arrive, own
    // colour's term, bounded wait: 375 us, the polling costs more issue slots
    // than the barrier stalls it removes), and with the half-spinors passed
    // through the thread's just-read staging slot so that 5 blocks fit an SM
    // (64 registers, 80 bytes spilled, the next copies issued behind each
    // barrier: 383 us); the staged form two directions ahead in three
    // slots (413 / 135 us with L2-only links, 584 / 196 us through L1: the
    // larger shared-memory footprint leaves less L1 for the neighbour
    // spinors); staged with registers capped at 80 or 72 (420 and 635 us,
    // spills); packed pairs loading into registers (504 us; 6.6
    // long-scoreboard stalls per issue), with an L2 prefetch of the next
    // direction (507 us); colour-split at <= 80 registers (478 us); the
    // unbounded colour-split form (242 registers); the register-prefetching
    // packed form; the scalar pipelined form capped at 80 or 72 registers
    // (550-830 bytes of spills, 639 and 778 us).
    // the grouped split: 2 groups (192 threads), registers capped for 4 blocks per SM
    auto run_grouped = [&]() -> wd_status {
        const int blocks = (lat->g.Vh + 63) / 64;
        if (dag) k_hop_df_grouped<true, 2, true, 4><<<blocks, 192, 0, ctx->stream>>>(p);
        else k_hop_df_grouped<false, 2, true, 4><<<blocks, 192, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    using F = std::false_type;
    using T = std::true_type;
    using W2 = std::integral_constant<int, 2>;
    using W4 = std::integral_constant<int, 4>;
    return wd_tune_launch(ctx, "hop_df64", lat->g.Vh, 6, [&](int v) -> wd_status {
        if (v == 1) return run_staged(W2(), T());
        if (v == 2) return run_staged(W2(), F());
        if (v == 3) return run_pipe(W2());
        if (v == 4) return run_pipe(W4());
        if (v == 5) return run_grouped();
        return run_staged(W4(), T());
    });
}

wd_status wd_hop_df_residual(wd_context *ctx, const wd_lattice *lat, const float4 *in_block, const float4 *x_block,
                             const float4 *bhat, float4 *s32, double mass, double *partial, unsigned *counter,
                             double *result)
{
    wd_status st = wd_lattice_gauge_df(ctx, lat);
    if (st != WD_OK) return st;
    const double a = 4.0 + mass;
    SplitDF p;
    p.g = lat->g;
    p.cb = 0;
    p.in = in_block;
    p.gauge = lat->gauge_df;
    p.x = x_block;
    p.out = nullptr;
    p.alpha = df_split(-0.25 / a);
    p.beta = df_split(a);
    const ResSinkDF r{bhat, s32, partial, counter, result};
    auto run = [&](auto warps, auto lcg) -> wd_status {
        constexpr int W = decltype(warps)::value;
        const int sites_per_block = kSitesPerWarp * W;
        const int blocks = (lat->g.Vh + sites_per_block - 1) / sites_per_block;
        k_hop_df_res<W, decltype(lcg)::value><<<blocks, 32 * W, 0, ctx->stream>>>(p, r);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    // the plain double-float hop's tuned shape (its register-pipelined
    // variants 3 and 4 take variant 0's)
    const int v = wd_tune_choice(ctx, "hop_df64", lat->g.Vh);
    if (v == 5) {  // the grouped split (2 groups, 4 blocks per SM)
        k_hop_df_res<6, true, true, 4><<<(lat->g.Vh + 63) / 64, 192, 0, ctx->stream>>>(p, r);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    if (v == 1) return run(std::integral_constant<int, 2>(), std::true_type());
    if (v == 2) return run(std::integral_constant<int, 2>(), std::false_type());
    return run(std::integral_constant<int, 4>(), std::true_type());
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
