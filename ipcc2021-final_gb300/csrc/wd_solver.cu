// wd_solver.cu -- conjugate-gradient solvers on resident fields.
//
// WD_SOLVER_CGNR_REF follows the reference CGinvert (src/invert.cpp:25-121)
// step for step: CG on M^dag M x = M^dag b over the whole lattice, complex
// alpha = (r,r)/(p,q), beta = (r,r)_new/(r,r)_old, stop on the absolute
// normal residual |r| < tol.  WD_SOLVER_CG_EO solves the same system through
// the even-odd Schur complement Mhat = a - D_eo D_oe/(4a) (a = 4+m), which
// needs half the hopping applications per iteration and converges in fewer
// iterations; it stops on the relative true residual |b - M x|/|b|.
#include <chrono>
#include <cmath>
#include <vector>
#include "wd_kernels.h"
#include "wd_solver.h"

namespace {

struct DevBuf {
    double2 *p = nullptr;
    ~DevBuf() { cudaFree(p); }
};

wd_status alloc_bufs(wd_context *ctx, std::vector<DevBuf> &bufs, size_t n_complex)
{
    for (auto &b : bufs) WD_CUDA(ctx, cudaMalloc(&b.p, n_complex * sizeof(double2)));
    return WD_OK;
}

double2 cdiv(double2 a, double2 b)
{
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

}  // namespace

// M (dag=0) or M^dag (dag=1) on full-lattice double2 arrays.
wd_status wd_apply_M(wd_context *ctx, const wd_lattice *lat, const double2 *in, double2 *out, double mass,
                     int dag, wd_precision prec)
{
    const size_t blk = (size_t)12 * lat->g.Vh;
    for (int cb = 0; cb < 2; ++cb) {
        wd_status st = wd_hop(ctx, lat, in + (1 - cb) * blk, out + cb * blk, in + cb * blk, cb, dag, -0.5,
                              4.0 + mass, prec);
        if (st != WD_OK) return st;
    }
    return WD_OK;
}

// Schur operator on even-parity blocks: out = a v - D_eo D_oe v / (4a)
// (dag: the same with D^dag, which is Mhat^dag).  tmp_o is an odd-parity block.
wd_status wd_apply_Mhat(wd_context *ctx, const wd_lattice *lat, const double2 *v, double2 *out,
                        double2 *tmp_o, double mass, int dag, wd_precision prec)
{
    const double a = 4.0 + mass;
    wd_status st = wd_hop(ctx, lat, v, tmp_o, nullptr, 1, dag, 1.0, 0.0, prec);
    if (st != WD_OK) return st;
    return wd_hop(ctx, lat, tmp_o, out, v, 0, dag, -0.25 / a, a, prec);
}

// |b - M x| / |b| recomputed in FP64.
wd_status wd_true_residual(wd_context *ctx, const wd_lattice *lat, const double2 *b, const double2 *x,
                           double2 *tmp, double mass, double *rel)
{
    const int64_t n = lat->volume * 12;
    wd_status st = wd_apply_M(ctx, lat, x, tmp, mass, 0, WD_PREC_F64);
    if (st != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, b, make_double2(-1.0, 0.0), tmp, tmp, n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, tmp, n, 0)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, b, n, 1)) != WD_OK) return st;
    double2 r[2];
    if ((st = wd_red_fetch(ctx, 2, r)) != WD_OK) return st;
    *rel = r[1].x > 0 ? std::sqrt(r[0].x / r[1].x) : std::sqrt(r[0].x);
    return WD_OK;
}

static wd_status solve_cgnr_ref(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x,
                                const wd_solver_params *prm, wd_solver_stats *stats)
{
    const int64_t n = lat->volume * 12;
    const double m = prm->mass;
    const wd_precision prec = prm->prec == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
    std::vector<DevBuf> b(5);
    wd_status st = alloc_bufs(ctx, b, n);
    if (st != WD_OK) return st;
    double2 *r0 = b[0].p, *q = b[1].p, *qq = b[2].p, *p = b[3].p, *Mdb = b[4].p;

    // Mdb = M^dag src; r0 = Mdb - M^dag M x   (src/invert.cpp:41-58)
    if ((st = wd_apply_M(ctx, lat, src, Mdb, m, 1, prec)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, x, qq, m, 0, prec)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, qq, r0, m, 1, prec)) != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, Mdb, make_double2(-1.0, 0.0), r0, r0, n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, r0, n, 0)) != WD_OK) return st;
    double2 red[2];
    if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
    double rr = red[0].x, r1 = rr, rsd = std::sqrt(rr);
    int iters = 0;
    bool converged = false;
    for (int f = 1; f < prm->max_iter; ++f) {
        if (f == 1) {
            WD_CUDA(ctx, cudaMemcpyAsync(p, r0, n * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
        } else {
            // beta = (r,r)/r1; p = r + beta p   (src/invert.cpp:67-76)
            const double beta = rr / r1;
            if ((st = wd_blas_axpby(ctx, make_double2(1.0, 0.0), r0, make_double2(beta, 0.0), p, n)) != WD_OK)
                return st;
        }
        if ((st = wd_apply_M(ctx, lat, p, qq, m, 0, prec)) != WD_OK) return st;
        if ((st = wd_apply_M(ctx, lat, qq, q, m, 1, prec)) != WD_OK) return st;
        r1 = rr;
        if ((st = wd_red_dot(ctx, p, q, n, 0)) != WD_OK) return st;
        if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
        const double2 alpha = cdiv(make_double2(r1, 0.0), red[0]);
        // dest += alpha p; r0 -= alpha q; |r0|^2   (src/invert.cpp:84-107)
        if ((st = wd_blas_cg_update(ctx, alpha, p, q, x, r0, n, 0)) != WD_OK) return st;
        if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
        rr = red[0].x;
        rsd = std::sqrt(rr);
        iters = f;
        if (!std::isfinite(rsd)) {
            stats->iterations = iters;
            stats->residual = rsd;
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

static wd_status solve_cg_eo(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x,
                             const wd_solver_params *prm, wd_solver_stats *stats)
{
    const int Vh = lat->g.Vh;
    const size_t blk = (size_t)12 * Vh;
    const int64_t nh = (int64_t)blk;
    const double m = prm->mass, a = 4.0 + m;
    const wd_precision prec = prm->prec == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
    std::vector<DevBuf> b(6);
    wd_status st = alloc_bufs(ctx, b, blk);
    if (st != WD_OK) return st;
    double2 *bhat = b[0].p, *r = b[1].p, *p = b[2].p, *t = b[3].p, *q = b[4].p, *tmp_o = b[5].p;
    const double2 *b_e = src, *b_o = src + blk;
    double2 *x_e = x, *x_o = x + blk;

    // bhat_e = b_e + D_eo b_o / (2a)
    if ((st = wd_hop(ctx, lat, b_o, bhat, b_e, 0, 0, 0.5 / a, 1.0, prec)) != WD_OK) return st;
    if (!prm->use_initial_guess) WD_CUDA(ctx, cudaMemsetAsync(x_e, 0, blk * sizeof(double2), ctx->stream));

    // r = Mhat^dag (bhat - Mhat x); returns |r|^2 and |Mhat^dag bhat|^2 on request
    auto normal_residual = [&](double *rr) -> wd_status {
        wd_status s = wd_apply_Mhat(ctx, lat, x_e, t, tmp_o, m, 0, prec);
        if (s != WD_OK) return s;
        if ((s = wd_blas_xpayz(ctx, bhat, make_double2(-1.0, 0.0), t, t, nh)) != WD_OK) return s;
        if ((s = wd_apply_Mhat(ctx, lat, t, r, tmp_o, m, 1, prec)) != WD_OK) return s;
        if ((s = wd_red_norm2(ctx, r, nh, 0)) != WD_OK) return s;
        double2 v;
        if ((s = wd_red_fetch(ctx, 1, &v)) != WD_OK) return s;
        *rr = v.x;
        return WD_OK;
    };

    // reference scale for the normal residual: |Mhat^dag bhat|
    if ((st = wd_apply_Mhat(ctx, lat, bhat, q, tmp_o, m, 1, prec)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, q, nh, 0)) != WD_OK) return st;
    double2 red[2];
    if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
    const double norm_mb = std::sqrt(red[0].x);

    double rr;
    if ((st = normal_residual(&rr)) != WD_OK) return st;
    WD_CUDA(ctx, cudaMemcpyAsync(p, r, blk * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
    double target = prm->tol * norm_mb;
    int iters = 0, checks = 0;
    bool converged = false;
    double true_res = INFINITY;
    while (iters < prm->max_iter) {
        if (std::sqrt(rr) <= target || rr == 0.0) {
            // reconstruct x_o and measure the true residual of the full system
            if ((st = wd_hop(ctx, lat, x_e, x_o, b_o, 1, 0, 0.5 / a, 1.0 / a, WD_PREC_F64)) != WD_OK) return st;
            double2 *full_tmp = nullptr;
            WD_CUDA(ctx, cudaMallocAsync((void **)&full_tmp, 2 * blk * sizeof(double2), ctx->stream));
            st = wd_true_residual(ctx, lat, src, x, full_tmp, m, &true_res);
            cudaFreeAsync(full_tmp, ctx->stream);
            if (st != WD_OK) return st;
            ++checks;
            if (true_res <= prm->tol || rr == 0.0) {
                converged = true;
                break;
            }
            // tighten the normal-residual target and replace r by the true one
            target *= std::fmax(0.05, 0.5 * prm->tol / true_res);
            if ((st = normal_residual(&rr)) != WD_OK) return st;
            stats->reliable_updates++;
            if (std::sqrt(rr) <= target) continue;
        }
        // t = Mhat p, q = Mhat^dag t, alpha = rr / |t|^2
        if ((st = wd_apply_Mhat(ctx, lat, p, t, tmp_o, m, 0, prec)) != WD_OK) return st;
        if ((st = wd_apply_Mhat(ctx, lat, t, q, tmp_o, m, 1, prec)) != WD_OK) return st;
        if ((st = wd_red_norm2(ctx, t, nh, 0)) != WD_OK) return st;
        if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
        const double alpha = rr / red[0].x;
        if ((st = wd_blas_cg_update(ctx, make_double2(alpha, 0.0), p, q, x_e, r, nh, 0)) != WD_OK) return st;
        if ((st = wd_red_fetch(ctx, 1, red)) != WD_OK) return st;
        const double rr_new = red[0].x;
        if (!std::isfinite(rr_new)) {
            stats->iterations = iters;
            return wd_fail(ctx, WD_ERR_NAN, "CG residual is not finite");
        }
        const double beta = rr_new / rr;
        rr = rr_new;
        if ((st = wd_blas_axpby(ctx, make_double2(1.0, 0.0), r, make_double2(beta, 0.0), p, nh)) != WD_OK)
            return st;
        ++iters;
    }
    if (!converged) {
        if ((st = wd_hop(ctx, lat, x_e, x_o, b_o, 1, 0, 0.5 / a, 1.0 / a, WD_PREC_F64)) != WD_OK) return st;
    }
    (void)checks;
    stats->iterations = iters;
    stats->residual = std::sqrt(rr) / (norm_mb > 0 ? norm_mb : 1.0);
    stats->converged = converged;
    return WD_OK;
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
}

extern "C" wd_status wd_solve(wd_context *ctx, const wd_lattice *lat, const wd_field *src, wd_field *dest,
                              const wd_solver_params *params, wd_solver_stats *stats)
{
    if (!ctx || !lat || !src || !dest || !params) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (src == dest) return wd_fail(ctx, WD_ERR_BAD_ARG, "source and solution must be different fields");
    if (src->lat->volume != lat->volume || dest->lat->volume != lat->volume)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "field does not belong to this lattice size");
    if (params->max_iter < 1 || !(params->tol > 0)) return wd_fail(ctx, WD_ERR_BAD_ARG, "bad tolerance or max_iter");
    wd_solver_stats local;
    if (!stats) stats = &local;
    *stats = wd_solver_stats{};
    const auto t0 = std::chrono::steady_clock::now();
    wd_status st;
    switch (params->kind) {
    case WD_SOLVER_CGNR_REF: st = solve_cgnr_ref(ctx, lat, src->d, dest->d, params, stats); break;
    case WD_SOLVER_CG_EO:
        if (params->prec == WD_PREC_F32 || params->prec == WD_PREC_F16)
            st = wd_solve_cg_eo_mixed(ctx, lat, src->d, dest->d, params, stats);
        else
            st = solve_cg_eo(ctx, lat, src->d, dest->d, params, stats);
        break;
    default: return wd_fail(ctx, WD_ERR_BAD_ARG, "unknown solver kind");
    }
    if (st != WD_OK) return st;
    // the FP64 true residual |b - M x|/|b| of whatever the solver returned
    double2 *tmp = nullptr;
    WD_CUDA(ctx, cudaMalloc((void **)&tmp, (size_t)lat->volume * 12 * sizeof(double2)));
    st = wd_true_residual(ctx, lat, src->d, dest->d, tmp, params->mass, &stats->true_residual);
    cudaFree(tmp);
    if (st != WD_OK) return st;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return stats->converged ? WD_OK : WD_ERR_NOT_CONVERGED;
}

extern "C" wd_status wd_check(wd_context *ctx, const wd_lattice *lat, const wd_field *b, const wd_field *x,
                              double mass, double out[12])
{
    if (!ctx || !lat || !b || !x || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    const int64_t n = lat->volume * 12;
    std::vector<DevBuf> bufs(6);
    wd_status st = alloc_bufs(ctx, bufs, n);
    if (st != WD_OK) return st;
    double2 *Mb = bufs[0].p, *Mdb = bufs[1].p, *MMb = bufs[2].p, *Mx = bufs[3].p, *MMx = bufs[4].p,
            *tmp = bufs[5].p;
    // the sequence of src/check.cpp:37-60
    if ((st = wd_apply_M(ctx, lat, b->d, Mb, mass, 0, WD_PREC_F64)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, b->d, Mdb, mass, 1, WD_PREC_F64)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, Mb, MMb, mass, 1, WD_PREC_F64)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, x->d, Mx, mass, 0, WD_PREC_F64)) != WD_OK) return st;
    if ((st = wd_apply_M(ctx, lat, Mx, MMx, mass, 1, WD_PREC_F64)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, b->d, n, 0)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, x->d, n, 1)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, Mb, Mb, n, 2)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, b->d, MMb, n, 3)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, Mx, Mx, n, 4)) != WD_OK) return st;
    if ((st = wd_red_dot(ctx, x->d, MMx, n, 5)) != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, Mx, make_double2(-1.0, 0.0), b->d, tmp, n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, tmp, n, 6)) != WD_OK) return st;
    if ((st = wd_blas_xpayz(ctx, MMx, make_double2(-1.0, 0.0), Mdb, tmp, n)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx, tmp, n, 7)) != WD_OK) return st;
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
