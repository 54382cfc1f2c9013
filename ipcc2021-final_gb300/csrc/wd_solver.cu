// wd_solver.cu -- conjugate-gradient solvers on resident fields.
//
// WD_SOLVER_CGNR_REF follows the reference CGinvert (src/invert.cpp:25-121)
// step for step: CG on M^dag M x = M^dag b over the whole lattice, complex
// alpha = (r,r)/(p,q), beta = (r,r)_new/(r,r)_old, stop on the absolute
// normal residual |r| < tol.  WD_SOLVER_CG_EO solves the same system through
// the even-odd Schur complement Mhat = a - D_eo D_oe/(4a) (a = 4+m), which
// needs half the hopping applications per iteration and converges in fewer
// iterations; it stops on the relative true residual |b - M x|/|b|.
//
// Both run in FP64 or in double-float (prec = WD_PREC_DF64: the same
// recurrences on float-pair vectors, ~5x faster on GB300's narrow FP64
// pipe).  Mixed precision (FP32 / FP16 inner) lives in wd_mixed.cu.
#include <chrono>
#include <cmath>
#include <vector>
#include "wd_kernels.h"
#include "wd_solver.h"

// ---------------------------------------------------------------- buffers
wd_status wd_vec_alloc(wd_context *ctx, WdVecBuf &b, wd_precision prec, int64_t n_complex)
{
    b.release();
    size_t bytes = (size_t)n_complex * wd_entry_bytes(prec);
    if (prec == WD_PREC_F16) bytes += (size_t)(n_complex / 12) * sizeof(float);
    wd_status st = wd_dev_alloc(ctx, &b.v.p, bytes);
    if (st != WD_OK) return st;
    b.ctx = ctx;
    b.v.prec = prec;
    b.v.scale = prec == WD_PREC_F16 ? (float *)((char *)b.v.p + (size_t)n_complex * wd_entry_bytes(prec)) : nullptr;
    return WD_OK;
}

void WdVecBuf::release()
{
    if (ctx) wd_dev_free(ctx, v.p);
    v = WdVec{};
    ctx = nullptr;
}

// half of a full-lattice vector (parity 0 or 1)
static inline WdVec par_half(WdVec v, int par, int Vh) { return wd_offset(v, (int64_t)par * 12 * Vh, (int64_t)par * Vh); }

// ---------------------------------------------------------------- operators
wd_status wd_apply_M_v(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, double mass, int dag)
{
    const int Vh = lat->g.Vh;
    for (int cb = 0; cb < 2; ++cb) {
        const WdVec x = par_half(in, cb, Vh);
        wd_status st = wd_hop_v(ctx, lat, par_half(in, 1 - cb, Vh), par_half(out, cb, Vh), &x, cb, dag, -0.5, 4.0 + mass);
        if (st != WD_OK) return st;
    }
    return WD_OK;
}

// Schur operator on even blocks: out = a v - D_eo D_oe v / (4a) (dag: with D^dag = Mhat^dag).
wd_status wd_apply_Mhat_v(wd_context *ctx, const wd_lattice *lat, WdVec v, WdVec out, WdVec tmp_o, double mass,
                          int dag)
{
    const double a = 4.0 + mass;
    wd_status st = wd_hop_v(ctx, lat, v, tmp_o, nullptr, 1, dag, 1.0, 0.0);
    if (st != WD_OK) return st;
    return wd_hop_v(ctx, lat, tmp_o, out, &v, 0, dag, -0.25 / a, a);
}

// |b - M x| / |b| recomputed in FP64 (b, x, tmp: FP64 full-lattice arrays).
wd_status wd_true_residual(wd_context *ctx, const wd_lattice *lat, const double2 *b, const double2 *x, double2 *tmp,
                           double mass, double *rel)
{
    const int64_t n = lat->volume * 12;
    WdVec vx{(void *)x}, vt{(void *)tmp};
    wd_status st = wd_apply_M_v(ctx, lat, vx, vt, mass, 0);
    if (st != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, b, make_double2(-1.0, 0.0), tmp, tmp, n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, tmp, n, 0)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, b, n, 1)) != WD_OK) return st;
    double2 r[2];
    if ((st = wd_red_fetch(ctx, 2, r)) != WD_OK) return st;
    *rel = r[1].x > 0 ? std::sqrt(r[0].x / r[1].x) : std::sqrt(r[0].x);
    return WD_OK;
}

static double2 cdiv(double2 a, double2 b)
{
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

static wd_status fetch1(wd_context *ctx, double2 *v) { return wd_red_fetch(ctx, 1, v); }

// ------------------------------------------------------- reference CGNR
// src/invert.cpp:25-121 on full-lattice vectors of one storage (FP64 or df).
static wd_status cgnr_ref_core(wd_context *ctx, const wd_lattice *lat, WdVec src, WdVec x,
                               const wd_solver_params *prm, wd_solver_stats *stats)
{
    const int64_t n = lat->volume * 12;
    const double m = prm->mass;
    WdVecBuf b[5];
    for (auto &v : b) {
        wd_status s = wd_vec_alloc(ctx, v, src.prec, n);
        if (s != WD_OK) return s;
    }
    WdVec r0 = b[0].v, q = b[1].v, qq = b[2].v, p = b[3].v, Mdb = b[4].v;
    wd_status st;
    // Mdb = M^dag src; r0 = Mdb - M^dag M x   (src/invert.cpp:41-58)
    if ((st = wd_apply_M_v(ctx, lat, src, Mdb, m, 1)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, x, qq, m, 0)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, qq, r0, m, 1)) != WD_OK) return st;
    if ((st = wd_v_xpayz(ctx, Mdb, make_double2(-1.0, 0.0), r0, r0, n)) != WD_OK) return st;
    if ((st = wd_v_norm2(ctx, r0, n, 0)) != WD_OK) return st;
    double2 red;
    if ((st = fetch1(ctx, &red)) != WD_OK) return st;
    double rr = red.x, r1 = rr, rsd = std::sqrt(rr);
    int iters = 0;
    bool converged = false;
    for (int f = 1; f < prm->max_iter; ++f) {
        if (f == 1) {
            if ((st = wd_v_copy(ctx, p, r0, n)) != WD_OK) return st;
        } else {
            // beta = (r,r)/r1; p = r + beta p   (src/invert.cpp:67-76)
            if ((st = wd_v_axpby(ctx, make_double2(1.0, 0.0), r0, make_double2(rr / r1, 0.0), p, n)) != WD_OK)
                return st;
        }
        if ((st = wd_apply_M_v(ctx, lat, p, qq, m, 0)) != WD_OK) return st;
        if ((st = wd_apply_M_v(ctx, lat, qq, q, m, 1)) != WD_OK) return st;
        r1 = rr;
        if ((st = wd_v_dot(ctx, p, q, n, 0)) != WD_OK) return st;
        if ((st = fetch1(ctx, &red)) != WD_OK) return st;
        const double2 alpha = cdiv(make_double2(r1, 0.0), red);
        // dest += alpha p; r0 -= alpha q; |r0|^2   (src/invert.cpp:84-107)
        if ((st = wd_v_cg_update(ctx, alpha, p, q, x, r0, n, 0)) != WD_OK) return st;
        if ((st = fetch1(ctx, &red)) != WD_OK) return st;
        rr = red.x;
        rsd = std::sqrt(rr);
        iters = f;
        if (!std::isfinite(rsd)) {
            stats->iterations = iters;
            return wd_fail(ctx, WD_ERR_NAN, "CG residual is not finite");
        }
        if (rsd < prm->tol) {
            converged = true;
            break;
        }
    }
    stats->iterations = iters;
    stats->residual = rsd;
    stats->converged = converged;
    return WD_OK;
}

// ----------------------------------------------------- even-odd Schur CG
static wd_status cg_eo_core(wd_context *ctx, const wd_lattice *lat, WdVec src, WdVec x, const wd_solver_params *prm,
                            wd_solver_stats *stats)
{
    const int Vh = lat->g.Vh;
    const int64_t nh = (int64_t)12 * Vh;
    const double m = prm->mass, a = 4.0 + m;
    WdVecBuf b[7];
    for (auto &v : b) {
        wd_status s = wd_vec_alloc(ctx, v, src.prec, nh);
        if (s != WD_OK) return s;
    }
    WdVec bhat = b[0].v, r = b[1].v, p = b[2].v, t = b[3].v, q = b[4].v, tmp_o = b[5].v, s_e = b[6].v;
    const WdVec b_e = par_half(src, 0, Vh), b_o = par_half(src, 1, Vh);
    WdVec x_e = par_half(x, 0, Vh), x_o = par_half(x, 1, Vh);
    wd_status st;

    // bhat_e = b_e + D_eo b_o / (2a)
    if ((st = wd_hop_v(ctx, lat, b_o, bhat, &b_e, 0, 0, 0.5 / a, 1.0)) != WD_OK) return st;
    if (!prm->use_initial_guess && (st = wd_v_zero(ctx, x_e, nh)) != WD_OK) return st;
    double2 red[2];
    if ((st = wd_v_norm2(ctx, src, 2 * nh, 1)) != WD_OK) return st;
    if ((st = wd_red_fetch(ctx, 2, red)) != WD_OK) return st;
    const double norm_b = std::sqrt(red[1].x) > 0 ? std::sqrt(red[1].x) : 1.0;

    // s = bhat - Mhat x (its norm is the full-system true residual |b - M x|
    // once x_o = (b_o + D_oe x_e / 2)/a), r = Mhat^dag s
    double ss = 0.0;
    auto residuals = [&](double *rr) -> wd_status {
        wd_status e = wd_apply_Mhat_v(ctx, lat, x_e, t, tmp_o, m, 0);
        if (e != WD_OK) return e;
        if ((e = wd_v_xpayz(ctx, bhat, make_double2(-1.0, 0.0), t, s_e, nh)) != WD_OK) return e;
        if ((e = wd_apply_Mhat_v(ctx, lat, s_e, r, tmp_o, m, 1)) != WD_OK) return e;
        if ((e = wd_v_norm2(ctx, r, nh, 0)) != WD_OK) return e;
        if ((e = wd_v_norm2(ctx, s_e, nh, 1)) != WD_OK) return e;
        double2 v[2];
        if ((e = wd_red_fetch(ctx, 2, v)) != WD_OK) return e;
        *rr = v[0].x;
        ss = v[1].x;
        return WD_OK;
    };

    double rr;
    if ((st = residuals(&rr)) != WD_OK) return st;
    if ((st = wd_v_copy(ctx, p, r, nh)) != WD_OK) return st;
    // normal-residual target from the observed ratio |r| / |s|
    double ratio = ss > 0 ? std::sqrt(rr / ss) : 1.0;
    double target = prm->tol * norm_b * ratio * 0.5;
    double true_res = std::sqrt(ss) / norm_b;
    int iters = 0;
    bool converged = true_res <= prm->tol;
    while (!converged && iters < prm->max_iter) {
        // t = Mhat p, q = Mhat^dag t, alpha = rr / |t|^2
        if ((st = wd_apply_Mhat_v(ctx, lat, p, t, tmp_o, m, 0)) != WD_OK) return st;
        if ((st = wd_apply_Mhat_v(ctx, lat, t, q, tmp_o, m, 1)) != WD_OK) return st;
        if ((st = wd_v_norm2(ctx, t, nh, 0)) != WD_OK) return st;
        if ((st = fetch1(ctx, red)) != WD_OK) return st;
        const double alpha = rr / red[0].x;
        if ((st = wd_v_cg_update_real(ctx, alpha, p, q, x_e, r, nh, 0)) != WD_OK) return st;
        if ((st = fetch1(ctx, red)) != WD_OK) return st;
        double rr_new = red[0].x;
        ++iters;
        if (!std::isfinite(rr_new)) {
            stats->iterations = iters;
            return wd_fail(ctx, WD_ERR_NAN, "CG residual is not finite");
        }
        if (std::sqrt(rr_new) <= target) {
            // check the true residual; replace r by the recomputed one
            if ((st = residuals(&rr_new)) != WD_OK) return st;
            stats->reliable_updates++;
            true_res = std::sqrt(ss) / norm_b;
            if (true_res <= prm->tol) {
                converged = true;
                rr = rr_new;
                break;
            }
            ratio = ss > 0 ? std::sqrt(rr_new / ss) : ratio;
            target = std::fmin(target * 0.5, prm->tol * norm_b * ratio * 0.5);
        }
        const double beta = rr_new / rr;
        rr = rr_new;
        if ((st = wd_v_xpby(ctx, r, beta, p, nh)) != WD_OK) return st;
    }
    // x_o = (b_o + D_oe x_e / 2) / a
    if ((st = wd_hop_v(ctx, lat, x_e, x_o, &b_o, 1, 0, 0.5 / a, 1.0 / a)) != WD_OK) return st;
    stats->iterations = iters;
    stats->residual = true_res;
    stats->converged = converged;
    return WD_OK;
}

// Runs a solver core in the requested arithmetic on FP64 fields.
template <class Core>
static wd_status run_in(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x, wd_precision prec,
                        Core core)
{
    WdVec vs{(void *)src}, vx{(void *)x};
    if (prec == WD_PREC_F64) return core(vs, vx);
    const int64_t n = lat->volume * 12;
    WdVecBuf ds, dx;
    wd_status st = wd_vec_alloc(ctx, ds, WD_PREC_DF64, n);
    if (st == WD_OK) st = wd_vec_alloc(ctx, dx, WD_PREC_DF64, n);
    if (st == WD_OK) st = wd_convert_f64_to_df(ctx, src, (float4 *)ds.v.p, n);
    if (st == WD_OK) st = wd_convert_f64_to_df(ctx, x, (float4 *)dx.v.p, n);
    if (st == WD_OK) st = core(ds.v, dx.v);
    if (st == WD_OK) st = wd_convert_df_to_f64(ctx, (const float4 *)dx.v.p, x, n);
    return st;
}

extern "C" void wd_solver_params_default(wd_solver_params *p)
{
    if (!p) return;
    p->kind = WD_SOLVER_CG_EO;
    p->mass = 0.1;
    p->tol = 1e-10;
    p->max_iter = 1000;
    p->prec = WD_PREC_F64;
    p->delta = 0.1;
    p->use_initial_guess = 0;
    p->prec_reliable = WD_PREC_F64;
}

extern "C" wd_status wd_solve(wd_context *ctx, const wd_lattice *lat, const wd_field *src, wd_field *dest,
                              const wd_solver_params *params, wd_solver_stats *stats)
{
    if (!ctx || !lat || !src || !dest || !params) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (src == dest) return wd_fail(ctx, WD_ERR_BAD_ARG, "source and solution must be different fields");
    if (src->lat->volume != lat->volume || dest->lat->volume != lat->volume)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "field does not belong to this lattice size");
    if (src->storage != WD_PREC_F64 || dest->storage != WD_PREC_F64)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "solver fields must be FP64 (prec selects the arithmetic)");
    if (params->max_iter < 1 || !(params->tol > 0)) return wd_fail(ctx, WD_ERR_BAD_ARG, "bad tolerance or max_iter");
    if (params->prec < WD_PREC_F64 || params->prec > WD_PREC_F16)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "unknown precision");
    wd_solver_stats local;
    if (!stats) stats = &local;
    *stats = wd_solver_stats{};
    const auto t0 = std::chrono::steady_clock::now();
    wd_status st;
    const bool mixed = params->prec == WD_PREC_F32 || params->prec == WD_PREC_F16;
    switch (params->kind) {
    case WD_SOLVER_CGNR_REF:
        if (mixed) return wd_fail(ctx, WD_ERR_BAD_ARG, "the reference CG runs in FP64 or double-float only");
        st = run_in(ctx, lat, src->d, dest->d, params->prec,
                    [&](WdVec s, WdVec x) { return cgnr_ref_core(ctx, lat, s, x, params, stats); });
        break;
    case WD_SOLVER_CG_EO:
        if (mixed)
            st = wd_solve_cg_eo_mixed(ctx, lat, src->d, dest->d, params, stats);
        else
            st = run_in(ctx, lat, src->d, dest->d, params->prec,
                        [&](WdVec s, WdVec x) { return cg_eo_core(ctx, lat, s, x, params, stats); });
        break;
    default: return wd_fail(ctx, WD_ERR_BAD_ARG, "unknown solver kind");
    }
    if (st != WD_OK) return st;
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // the FP64 true residual |b - M x|/|b| of whatever the solver returned
    // (a check of the result, after the timed solve)
    WdVecBuf tmp;
    if ((st = wd_vec_alloc(ctx, tmp, WD_PREC_F64, lat->volume * 12)) != WD_OK) return st;
    st = wd_true_residual(ctx, lat, src->d, dest->d, (double2 *)tmp.v.p, params->mass, &stats->true_residual);
    if (st != WD_OK) return st;
    return stats->converged ? WD_OK : WD_ERR_NOT_CONVERGED;
}

extern "C" wd_status wd_check(wd_context *ctx, const wd_lattice *lat, const wd_field *b, const wd_field *x,
                              double mass, double out[12])
{
    if (!ctx || !lat || !b || !x || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (b->storage != WD_PREC_F64 || x->storage != WD_PREC_F64)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "check needs FP64 fields");
    const int64_t n = lat->volume * 12;
    WdVecBuf bufs[6];
    for (auto &v : bufs) {
        wd_status s = wd_vec_alloc(ctx, v, WD_PREC_F64, n);
        if (s != WD_OK) return s;
    }
    const WdVec vb = wd_whole(b), vx = wd_whole(x);
    const WdVec Mb = bufs[0].v, Mdb = bufs[1].v, MMb = bufs[2].v, Mx = bufs[3].v, MMx = bufs[4].v, tmp = bufs[5].v;
    auto d2 = [](WdVec v) { return (double2 *)v.p; };
    wd_status st;
    // the sequence of src/check.cpp:37-60
    if ((st = wd_apply_M_v(ctx, lat, vb, Mb, mass, 0)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, vb, Mdb, mass, 1)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, Mb, MMb, mass, 1)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, vx, Mx, mass, 0)) != WD_OK) return st;
    if ((st = wd_apply_M_v(ctx, lat, Mx, MMx, mass, 1)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, b->d, n, 0)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, x->d, n, 1)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, d2(Mb), d2(Mb), n, 2)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, b->d, d2(MMb), n, 3)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, d2(Mx), d2(Mx), n, 4)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, x->d, d2(MMx), n, 5)) != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, d2(Mx), make_double2(-1.0, 0.0), b->d, d2(tmp), n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, d2(tmp), n, 6)) != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, d2(MMx), make_double2(-1.0, 0.0), d2(Mdb), d2(tmp), n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, d2(tmp), n, 7)) != WD_OK) return st;
    double2 r[8];
    if ((st = wd_red_fetch(ctx, 8, r)) != WD_OK) return st;
    out[0] = std::sqrt(r[0].x);
    out[1] = std::sqrt(r[1].x);
    out[2] = r[2].x, out[3] = r[2].y;
    out[4] = r[3].x, out[5] = r[3].y;
    out[6] = r[4].x, out[7] = r[4].y;
    out[8] = r[5].x, out[9] = r[5].y;
    out[10] = std::sqrt(r[6].x);
    out[11] = std::sqrt(r[7].x);
    return WD_OK;
}
