// wd_kernels.h -- internal launchers shared between the library's translation
// units.  All run on ctx->stream; none allocates memory.
#pragma once
#include "wd_internal.cuh"

// Fixed reduction grid: results are bitwise reproducible for a given length.
#define WD_RED_BLOCKS 608
#define WD_RED_THREADS 256
// result slots after the partials in ctx->red_partial (double2 each)
#define WD_RED_SLOTS 16

// ---- hopping term: out_cb = alpha * D_{cb,1-cb} in_{1-cb} + beta * x_cb
wd_status wd_hop_f64(wd_context *ctx, const wd_lattice *lat, const double2 *in_block,
                     double2 *out_block, const double2 *x_block, int cb, int dag, double alpha,
                     double beta);

// ---- layout conversion (reference AoS <-> device SoA), on device buffers
// spinor: ref[(p*Vh + s)*12 + c]  <->  soa[(p*12 + c)*Vh + s]
wd_status wd_spinor_ref_to_soa(wd_context *ctx, const WdGeom &g, const double2 *ref, double2 *soa);
wd_status wd_spinor_soa_to_ref(wd_context *ctx, const WdGeom &g, const double2 *soa, double2 *ref);
// gauge, one direction: ref[(p*Vh + s)*9 + k]  ->  soa[((mu*2 + p)*9 + k)*Vh + s]
wd_status wd_gauge_ref_to_soa(wd_context *ctx, const WdGeom &g, int mu, const double2 *ref,
                              double2 *soa);

// ---- BLAS-1 on double2 arrays of n complex entries
// results of reductions are written to ctx->red_partial[WD_RED_BLOCKS + slot]
wd_status wd_red_norm2(wd_context *ctx, const double2 *a, int64_t n, int slot);
wd_status wd_red_dot(wd_context *ctx, const double2 *a, const double2 *b, int64_t n, int slot);
// copy result slots [0, nslots) to the host (synchronises the stream)
wd_status wd_red_fetch(wd_context *ctx, int nslots, double2 *host);
// y = a*x + b*y   (a, b complex)
wd_status wd_blas_axpby(wd_context *ctx, double2 a, const double2 *x, double2 b, double2 *y,
                        int64_t n);
// z = x + a*y     (a complex)
wd_status wd_blas_xpayz(wd_context *ctx, const double2 *x, double2 a, const double2 *y,
                        double2 *z, int64_t n);
// x += alpha p; r -= alpha q; slot <- |r|^2
wd_status wd_blas_cg_update(wd_context *ctx, double2 alpha, const double2 *p, const double2 *q,
                            double2 *x, double2 *r, int64_t n, int slot);
// y = a*x (real a)
wd_status wd_blas_scale(wd_context *ctx, double a, const double2 *x, double2 *y, int64_t n);
