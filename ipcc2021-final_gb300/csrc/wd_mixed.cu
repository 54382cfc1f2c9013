// wd_mixed.cu -- mixed-precision even-odd CG with reliable updates.
//
// The CG on Mhat^dag Mhat x_e = Mhat^dag bhat_e (Mhat = a - D_eo D_oe/(4a))
// iterates in low precision: search direction and operator outputs in the
// kernel storage (FP32, or FP16 with per-site scale; 12-real links), the
// iterated residual r_s and the solution increment x_s in FP32, with
// per-site double-float partial sums reduced in FP64.  Whenever the
// low-precision residual has dropped by delta (default 0.1) since the last
// update, or has reached the estimated target, a reliable update
// (Sleijpen & van der Vorst) recomputes the residual in high precision (FP64,
// or double-float when prec_reliable = WD_PREC_DF64):
//   x_e += x_s;  s = bhat - Mhat x_e;  r_s = Mhat^dag s (FP32);  x_s <- 0
// |s| is the true residual |b - M x| of the full system, so convergence is
// decided on the recomputed high-precision residual, never on the iterated one.
#include <algorithm>
#include <chrono>
#include <cmath>
#include "wd_df.cuh"
#include "wd_lp.cuh"
#include "wd_reduce.cuh"
#include "wd_solver.h"

namespace {

// high-precision (FP64 or double-float) block access in FP64 registers
struct HF64 {
    double2 *p;
    int Vh;
    __device__ double2 load(int c, int s) const { return p[(size_t)c * Vh + s]; }
    __device__ void store(int c, int s, double2 v) const { p[(size_t)c * Vh + s] = v; }
    __device__ float2 load_f32(int c, int s) const
    {
        const double2 d = load(c, s);
        return make_float2((float)d.x, (float)d.y);
    }
    __device__ void add_f32(int c, int s, float2 v) const
    {
        double2 d = load(c, s);
        d.x += (double)v.x;
        d.y += (double)v.y;
        store(c, s, d);
    }
};
// double-float: the FP32 views and the accumulation stay on the FP32 pipe
// (TwoSum, no FP64 conversions)
struct HDF {
    float4 *p;
    int Vh;
    __device__ double2 load(int c, int s) const { return df_unpack(p[(size_t)c * Vh + s]); }
    __device__ void store(int c, int s, double2 v) const { p[(size_t)c * Vh + s] = df_pack(v); }
    __device__ float2 load_f32(int c, int s) const
    {
        const float4 v = p[(size_t)c * Vh + s];  // {re.h, im.h, re.l, im.l}
        return make_float2(__fadd_rn(v.x, v.z), __fadd_rn(v.y, v.w));
    }
    __device__ void add_f32(int c, int s, float2 v) const
    {
        const dfc d = df_from_f4(p[(size_t)c * Vh + s]);
        p[(size_t)c * Vh + s] = df_to_f4(dfc{df_add(d.re, dfr{v.x, 0.f}), df_add(d.im, dfr{v.y, 0.f})});
    }
};

__device__ __forceinline__ dfr df_sq_acc(dfr acc, float2 v)
{
    return df_madd(df_madd(acc, dfr{v.x, 0.f}, dfr{v.x, 0.f}), dfr{v.y, 0.f}, dfr{v.y, 0.f});
}

#define SITE_STRIDE(s, Vh) for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < (Vh); s += gridDim.x * blockDim.x)

// p = r_s + beta p
template <class SpL>
__global__ void k_mx_xpay(SpF32 rs, float beta, SpL p, int Vh)
{
    SITE_STRIDE(s, Vh)
    {
        float2 rv[12], pv[12];
        rs.load(s, rv);
        p.load(s, pv);
#pragma unroll
        for (int c = 0; c < 12; ++c) pv[c] = make_float2(fmaf(beta, pv[c].x, rv[c].x), fmaf(beta, pv[c].y, rv[c].y));
        p.store(s, pv);
    }
}

// p = r_s + beta p with beta from the device scalars; a no-op while a
// reliable update is due (d->stop != 0)
template <class SpL>
__global__ void k_mx_xpay_dev(SpF32 rs, const WdMxDev *d, SpL p, int Vh)
{
    if (d->stop) return;
    const float beta = d->beta;
    SITE_STRIDE(s, Vh)
    {
        float2 rv[12], pv[12];
        rs.load(s, rv);
        p.load(s, pv);
#pragma unroll
        for (int c = 0; c < 12; ++c) pv[c] = make_float2(fmaf(beta, pv[c].x, rv[c].x), fmaf(beta, pv[c].y, rv[c].y));
        p.store(s, pv);
    }
}

template <class SpL>
__global__ void __launch_bounds__(WD_RED_THREADS) k_mx_norm2(SpL t, int Vh, double2 *partial)
{
    dfr acc{0.f, 0.f};
    SITE_STRIDE(s, Vh)
    {
        float2 v[12];
        t.load(s, v);
#pragma unroll
        for (int c = 0; c < 12; ++c) acc = df_sq_acc(acc, v[c]);
    }
    wd_block_partial(df_value(acc), 0.0, partial);
}

// high precision -> low precision (two outputs: FP32 r_s and kernel-storage p)
template <class H, class SpL>
__global__ void k_mx_from_h(H in, SpF32 a, SpL b, int Vh)
{
    SITE_STRIDE(s, Vh)
    {
        float2 v[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = in.load_f32(c, s);
        a.store(s, v);
        b.store(s, v);
    }
}

// high precision -> FP32
template <class H>
__global__ void k_mx_to_f32(H in, SpF32 a, int Vh)
{
    SITE_STRIDE(s, Vh)
    {
        float2 v[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = in.load_f32(c, s);
        a.store(s, v);
    }
}

// FP32 -> kernel storage
template <class SpL>
__global__ void k_mx_f32_to(SpF32 a, SpL b, int Vh)
{
    SITE_STRIDE(s, Vh)
    {
        float2 v[12];
        a.load(s, v);
        b.store(s, v);
    }
}

// x_H += x_s; x_s = 0
template <class H>
__global__ void k_mx_accum(SpF32 xs, H x, int Vh)
{
    SITE_STRIDE(s, Vh)
    {
        float2 v[12];
        xs.load(s, v);
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            x.add_f32(c, s, v[c]);
            v[c] = make_float2(0.f, 0.f);
        }
        xs.store(s, v);
    }
}

// Reduction kernels always run the fixed grid of WD_RED_BLOCKS blocks (idle
// blocks write zero partials): wd_red_finish folds exactly that many.
inline int site_grid(int) { return WD_RED_BLOCKS; }

// Typed launchers over (kernel storage L) x (high precision H)
struct Mixed {
    wd_context *ctx;
    int Vh;
    wd_precision L, H;

    wd_status xpay(WdVec rs, float beta, WdVec p) const
    {
        if (L == WD_PREC_F32) k_mx_xpay<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(rs, Vh), beta, sp_f32(p, Vh), Vh);
        else k_mx_xpay<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(rs, Vh), beta, sp_f16(p, Vh), Vh);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    wd_status xpay_dev(WdVec rs, const WdMxDev *d, WdVec p) const
    {
        if (L == WD_PREC_F32) k_mx_xpay_dev<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(rs, Vh), d, sp_f32(p, Vh), Vh);
        else k_mx_xpay_dev<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(rs, Vh), d, sp_f16(p, Vh), Vh);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    wd_status from_h(WdVec h, WdVec rs, WdVec p) const
    {
        const int g = site_grid(Vh);
        if (H == WD_PREC_F64) {
            const HF64 in{(double2 *)h.p, Vh};
            if (L == WD_PREC_F32) k_mx_from_h<<<g, WD_RED_THREADS, 0, ctx->stream>>>(in, sp_f32(rs, Vh), sp_f32(p, Vh), Vh);
            else k_mx_from_h<<<g, WD_RED_THREADS, 0, ctx->stream>>>(in, sp_f32(rs, Vh), sp_f16(p, Vh), Vh);
        } else {
            const HDF in{(float4 *)h.p, Vh};
            if (L == WD_PREC_F32) k_mx_from_h<<<g, WD_RED_THREADS, 0, ctx->stream>>>(in, sp_f32(rs, Vh), sp_f32(p, Vh), Vh);
            else k_mx_from_h<<<g, WD_RED_THREADS, 0, ctx->stream>>>(in, sp_f32(rs, Vh), sp_f16(p, Vh), Vh);
        }
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    wd_status to_f32(WdVec h, WdVec a) const
    {
        const int g = site_grid(Vh);
        if (H == WD_PREC_F64) k_mx_to_f32<<<g, WD_RED_THREADS, 0, ctx->stream>>>(HF64{(double2 *)h.p, Vh}, sp_f32(a, Vh), Vh);
        else k_mx_to_f32<<<g, WD_RED_THREADS, 0, ctx->stream>>>(HDF{(float4 *)h.p, Vh}, sp_f32(a, Vh), Vh);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    wd_status f32_to(WdVec a, WdVec p) const
    {
        if (L == WD_PREC_F32) {
            WD_CUDA(ctx, cudaMemcpyAsync(p.p, a.p, (size_t)12 * Vh * sizeof(float2), cudaMemcpyDeviceToDevice, ctx->stream));
            return WD_OK;
        }
        k_mx_f32_to<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(a, Vh), sp_f16(p, Vh), Vh);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
    wd_status norm2_f32(WdVec t, int slot) const
    {
        k_mx_norm2<<<site_grid(Vh), WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(t, Vh), Vh, (double2 *)ctx->red_partial);
        WD_LAUNCHED(ctx);
        return wd_red_finish(ctx, slot);
    }
    wd_status accum(WdVec xs, WdVec xh) const
    {
        const int g = site_grid(Vh);
        if (H == WD_PREC_F64) k_mx_accum<<<g, WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(xs, Vh), HF64{(double2 *)xh.p, Vh}, Vh);
        else k_mx_accum<<<g, WD_RED_THREADS, 0, ctx->stream>>>(sp_f32(xs, Vh), HDF{(float4 *)xh.p, Vh}, Vh);
        WD_LAUNCHED(ctx);
        return WD_OK;
    }
};

inline WdVec par_half(WdVec v, int par, int Vh) { return wd_offset(v, (int64_t)par * 12 * Vh, (int64_t)par * Vh); }

// out (odd) = D_oe in (or D_oe^dag), a no-op while *stop != 0
wd_status hop_oe_gated(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, int dag, const int *stop)
{
    if (in.prec == WD_PREC_F32) return wd_hop_f32(ctx, lat, in, out, nullptr, 1, dag, 1.0, 0.0, stop);
    return wd_hop_f16(ctx, lat, in, out, nullptr, 1, dag, 1.0, 0.0, stop);
}

// a block from the context's work-buffer cache, returned on scope exit
struct DevBlock {
    wd_context *ctx = nullptr;
    void *p = nullptr;
    ~DevBlock()
    {
        if (p) wd_dev_free(ctx, p);
    }
    wd_status alloc(wd_context *c, size_t bytes)
    {
        ctx = c;
        return wd_dev_alloc(c, &p, bytes);
    }
};

}  // namespace

wd_status wd_mx_accum(wd_context *ctx, int Vh, wd_precision H, WdVec xs, WdVec xh)
{
    return Mixed{ctx, Vh, WD_PREC_F32, H}.accum(xs, xh);
}

wd_status wd_mx_from_h(wd_context *ctx, int Vh, wd_precision L, wd_precision H, WdVec h, WdVec rs, WdVec p)
{
    return Mixed{ctx, Vh, L, H}.from_h(h, rs, p);
}

// Reliable update shared by the solo and batched mixed solvers:
//   x_e += x_s, x_s = 0            (high precision)
//   s = bhat - Mhat x_e, ss = |s|^2 (high precision: the true residual)
//   r_s = Mhat^dag s, rr = |r_s|^2  (FP32: s rounded to FP32, FP32 12-real links)
//   p <- r_s in kernel storage      (on a restart)
// Only s decides convergence.  r_s seeds the low-precision iteration, which
// keeps r_s in FP32 anyway, so an FP32 Mhat^dag adds an error of the same
// order as the rounding of a high-precision r to FP32, relative to the
// current residual -- and costs a quarter of a double-float application.
// scratch_h: one high-precision half-lattice buffer, used as two FP32 ones.
wd_status wd_mx_xpay(wd_context *ctx, int Vh, wd_precision L, WdVec rs, double beta, WdVec p)
{
    return Mixed{ctx, Vh, L, WD_PREC_F64}.xpay(rs, (float)beta, p);
}

wd_status wd_mx_reliable(wd_context *ctx, const wd_lattice *lat, double mass, wd_precision L, wd_precision H,
                         const WdMxReliable &v, const WdVec *p_restart, double *rr, double *ss)
{
    double2 *res = (double2 *)ctx->red_partial + WD_RED_BLOCKS;
    wd_status e = wd_mx_reliable_enqueue(ctx, lat, mass, L, H, v, p_restart, &res[0].x, &res[1].x);
    if (e != WD_OK) return e;
    double2 red[2];
    if ((e = wd_red_fetch(ctx, 2, red)) != WD_OK) return e;
    *rr = red[0].x;
    *ss = red[1].x;
    return WD_OK;
}

size_t wd_mx_reliable_scratch_doubles(int Vh) { return (size_t)Vh / 16 + 3; }

wd_status wd_mx_reliable_enqueue(wd_context *ctx, const wd_lattice *lat, double mass, wd_precision L, wd_precision H,
                                 const WdMxReliable &v, const WdVec *p_restart, double *rr_dev, double *ss_dev,
                                 double *scratch)
{
    const int Vh = lat->g.Vh;
    const int64_t nh = (int64_t)12 * Vh;
    const Mixed mx{ctx, Vh, L, H};
    WdVec s32, tmp32;
    s32.prec = tmp32.prec = WD_PREC_F32;
    s32.p = v.scratch_h.p;
    tmp32.p = (char *)v.scratch_h.p + (size_t)nh * sizeof(float2);
    // block partials of the two reductions, then their two counters: the
    // caller's scratch, or a block from the work-buffer cache
    const size_t nparts = wd_mx_reliable_scratch_doubles(Vh) - 1;
    DevBlock blk;
    wd_status e;
    if (!scratch && (e = blk.alloc(ctx, (nparts + 1) * sizeof(double))) != WD_OK) return e;
    double *partial = scratch ? scratch : (double *)blk.p;
    unsigned *count = (unsigned *)(partial + nparts);
    WD_CUDA(ctx, cudaMemsetAsync(count, 0, 2 * sizeof(unsigned), ctx->stream));
    if ((e = mx.accum(v.xs, v.x_e)) != WD_OK) return e;
    // s = bhat - Mhat x_e (high precision, rounded to FP32 as stored), |s|^2 -> slot + 1
    if ((e = wd_hop_v(ctx, lat, v.x_e, v.tmp_oh, nullptr, 1, 0, 1.0, 0.0)) != WD_OK) return e;
    if ((e = wd_hop_hi_residual(ctx, lat, v.tmp_oh, v.x_e, v.bhat, s32, mass, partial, count, ss_dev)) != WD_OK)
        return e;
    // r_s = Mhat^dag s (FP32), |r_s|^2 -> slot
    if ((e = wd_hop_v(ctx, lat, s32, tmp32, nullptr, 1, 1, 1.0, 0.0)) != WD_OK) return e;
    if ((e = wd_hop_f32_norm(ctx, lat, tmp32, v.rs, s32, mass, 1, partial, count + 1, rr_dev)) != WD_OK)
        return e;
    return p_restart ? mx.f32_to(v.rs, *p_restart) : WD_OK;
}

wd_status wd_solve_cg_eo_mixed(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x,
                               const wd_solver_params *prm, wd_solver_stats *stats)
{
    const int Vh = lat->g.Vh;
    const int64_t nh = (int64_t)12 * Vh, n = 2 * nh;
    const double m = prm->mass, a = 4.0 + m;
    const double delta = prm->delta > 0 && prm->delta < 1 ? prm->delta : 0.1;
    const wd_precision H = prm->prec_reliable == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
    const Mixed mx{ctx, Vh, prm->prec, H};
    wd_status st;

    // high-precision vectors: full source and solution, even-parity work blocks
    WdVecBuf hs, hx, bhat, r_h, tmp_oh;
    WdVecBuf p, t, tmp_ol, rs, xs;
    WdVecBuf *hbufs[] = {&bhat, &r_h, &tmp_oh};
    for (WdVecBuf *b : hbufs)
        if ((st = wd_vec_alloc(ctx, *b, H, nh)) != WD_OK) return st;
    WdVecBuf *lbufs[] = {&p, &t, &tmp_ol};
    for (WdVecBuf *b : lbufs)
        if ((st = wd_vec_alloc(ctx, *b, prm->prec, nh)) != WD_OK) return st;
    if ((st = wd_vec_alloc(ctx, rs, WD_PREC_F32, nh)) != WD_OK) return st;
    if ((st = wd_vec_alloc(ctx, xs, WD_PREC_F32, nh)) != WD_OK) return st;
    WdVec vsrc{(void *)src}, vx{(void *)x};
    if (H == WD_PREC_DF64) {
        if ((st = wd_vec_alloc(ctx, hs, H, n)) != WD_OK) return st;
        if ((st = wd_vec_alloc(ctx, hx, H, n)) != WD_OK) return st;
        if ((st = wd_convert_f64_to_df(ctx, src, (float4 *)hs.v.p, n)) != WD_OK) return st;
        // without an initial guess x_e is zeroed below and x_o is written at the end
        if (prm->use_initial_guess && (st = wd_convert_f64_to_df(ctx, x, (float4 *)hx.v.p, n)) != WD_OK) return st;
        vsrc = hs.v;
        vx = hx.v;
    }
    const WdVec b_e = par_half(vsrc, 0, Vh), b_o = par_half(vsrc, 1, Vh);
    const WdVec x_e = par_half(vx, 0, Vh), x_o = par_half(vx, 1, Vh);

    if ((st = wd_hop_v(ctx, lat, b_o, bhat.v, &b_e, 0, 0, 0.5 / a, 1.0)) != WD_OK) return st;
    if (!prm->use_initial_guess && (st = wd_v_zero(ctx, x_e, nh)) != WD_OK) return st;
    if ((st = wd_v_zero(ctx, xs.v, nh)) != WD_OK) return st;
    double2 red[2];
    if ((st = wd_red_norm2(ctx, src, n, 1)) != WD_OK) return st;
    if ((st = wd_red_fetch(ctx, 2, red)) != WD_OK) return st;
    const double norm_b = red[1].x > 0 ? std::sqrt(red[1].x) : 1.0;

    // reliable update: x_e += x_s; s = bhat - Mhat x_e; r_s = Mhat^dag s (p <- r_s only on a restart)
    double rr = 0, ss = 0;
    const WdMxReliable rv{xs.v, x_e, bhat.v, tmp_oh.v, r_h.v, rs.v};
    auto reliable = [&](bool reset_p) -> wd_status {
        return wd_mx_reliable(ctx, lat, m, prm->prec, H, rv, reset_p ? &p.v : nullptr, &rr, &ss);
    };

    if ((st = reliable(true)) != WD_OK) return st;
    double true_res = std::sqrt(ss) / norm_b;
    double ratio = ss > 0 ? std::sqrt(rr / ss) : 1.0;
    double target = prm->tol * norm_b * ratio * 0.5;
    int iters = 0;
    bool converged = true_res <= prm->tol;

    // The iterations run on device scalars (WdMxDev): alpha and beta are
    // formed by the reducing hops' last blocks, and the last block of each
    // |r_s|^2 reduction decides whether a reliable update is due.  The host
    // queues the number of iterations the previous residual-reduction cycle
    // took, then reads the scalars once: iterations queued past the one that
    // asked for an update are no-ops.
    DevBlock dev_blk, part_blk;
    if ((st = dev_blk.alloc(ctx, sizeof(WdMxDev))) != WD_OK) return st;
    if ((st = part_blk.alloc(ctx, sizeof(double) * ((size_t)Vh / 64 + 2))) != WD_OK) return st;
    WdMxDev *dev = (WdMxDev *)dev_blk.p;
    double *partial = (double *)part_blk.p;
    WdMxDev *sc = (WdMxDev *)ctx->state_host;
    *sc = WdMxDev{};
    sc->rr = sc->rr_max = rr;
    sc->target2 = target * target;
    sc->delta2 = delta * delta;
    WD_CUDA(ctx, cudaMemcpyAsync(dev, sc, sizeof(WdMxDev), cudaMemcpyHostToDevice, ctx->stream));
    int cycle = 4, since = 0;
    while (!converged && iters < prm->max_iter) {
        const int k = std::min(std::max(1, cycle - since), prm->max_iter - iters);
        for (int i = 0; i < k; ++i) {
            // t = Mhat p with |t|^2 -> alpha; q = Mhat^dag t applied as the update; p = r_s + beta p
            if ((st = hop_oe_gated(ctx, lat, p.v, tmp_ol.v, 0, &dev->stop)) != WD_OK) return st;
            if ((st = wd_hop_lp_norm(ctx, lat, tmp_ol.v, t.v, p.v, m, dev, partial)) != WD_OK) return st;
            if ((st = hop_oe_gated(ctx, lat, t.v, tmp_ol.v, 1, &dev->stop)) != WD_OK) return st;
            if ((st = wd_hop_lp_update(ctx, lat, tmp_ol.v, t.v, p.v, rs.v, xs.v, m, dev, partial)) != WD_OK)
                return st;
            if ((st = mx.xpay_dev(rs.v, dev, p.v)) != WD_OK) return st;
        }
        WD_CUDA(ctx, cudaMemcpyAsync(sc, dev, sizeof(WdMxDev), cudaMemcpyDeviceToHost, ctx->stream));
        WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        since += sc->iters - iters;
        iters = sc->iters;
        if (sc->stop == 2) {
            stats->iterations = iters;
            return wd_fail(ctx, WD_ERR_NAN, "mixed CG residual is not finite");
        }
        if (sc->stop != 1) continue;
        // reliable update after this iteration
        const double rr_old = sc->rr, rr_new = sc->rr_new;
        if ((st = reliable(false)) != WD_OK) return st;
        stats->reliable_updates++;
        true_res = std::sqrt(ss) / norm_b;
        if (true_res <= prm->tol) {
            converged = true;
            break;
        }
        if (std::sqrt(rr_new) <= target) {
            ratio = ss > 0 ? std::sqrt(rr / ss) : ratio;
            target = std::fmin(target * 0.5, prm->tol * norm_b * ratio * 0.5);
        }
        // continue from the recomputed residual: beta = |r_s|^2 / previous |r_s|^2
        if ((st = mx.xpay(rs.v, (float)(rr / rr_old), p.v)) != WD_OK) return st;
        sc->rr = sc->rr_max = rr;
        sc->target2 = target * target;
        sc->stop = 0;
        WD_CUDA(ctx, cudaMemcpyAsync(dev, sc, sizeof(WdMxDev), cudaMemcpyHostToDevice, ctx->stream));
        cycle = since;
        since = 0;
    }
    if (!converged && (st = mx.accum(xs.v, x_e)) != WD_OK) return st;
    // x_o = (b_o + D_oe x_e / 2) / a, then back to FP64
    if ((st = wd_hop_v(ctx, lat, x_e, x_o, &b_o, 1, 0, 0.5 / a, 1.0 / a)) != WD_OK) return st;
    if (H == WD_PREC_DF64 && (st = wd_convert_df_to_f64(ctx, (const float4 *)hx.v.p, x, n)) != WD_OK) return st;
    stats->iterations = iters;
    stats->residual = true_res;
    stats->converged = converged;
    return WD_OK;
}
