// wd_short.cpp -- the short entry-point names of the drop-in boundary
// (context, gauge upload, fermion upload/download, D_eo, M, CG), each a
// forward to the full C ABI in wilson_gb300.h.
#include "wilson_gb300.h"

extern "C" wd_status wd_ctx_create(int device, wd_context **ctx) { return wd_context_create(device, ctx); }

extern "C" void wd_ctx_destroy(wd_context *ctx) { wd_context_destroy(ctx); }

extern "C" wd_status wd_gauge_upload(wd_context *ctx, const double *const ref_layout[4], const int dims[4],
                                     wd_lattice **lat)
{
    return wd_lattice_create(ctx, dims, ref_layout, lat);
}

extern "C" wd_status wd_fermion_upload(wd_context *ctx, wd_field *f, const double *ref_layout)
{
    return wd_field_upload(ctx, f, ref_layout);
}

extern "C" wd_status wd_fermion_download(wd_context *ctx, const wd_field *f, double *ref_layout)
{
    return wd_field_download(ctx, f, ref_layout);
}

extern "C" wd_status wd_M(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out, double mass,
                          int dag)
{
    return wd_dslash_full(ctx, lat, in, out, mass, dag, WD_PREC_F64);
}

extern "C" wd_status wd_cg(wd_context *ctx, const wd_lattice *lat, const wd_field *src, wd_field *dest, double mass,
                           double tol, int max_iter, int flags, wd_solver_stats *stats)
{
    wd_solver_params p;
    wd_solver_params_default(&p);
    p.kind = (flags & WD_CG_REFERENCE) ? WD_SOLVER_CGNR_REF : WD_SOLVER_CG_EO;
    p.mass = mass;
    p.tol = tol;
    p.max_iter = max_iter;
    p.prec = (wd_precision)((flags >> 1) & 3);
    p.prec_reliable = (flags & WD_CG_RELIABLE_DF64) ? WD_PREC_DF64 : WD_PREC_F64;
    p.use_initial_guess = (flags & WD_CG_INITIAL_GUESS) ? 1 : 0;
    return wd_solve(ctx, lat, src, dest, &p, stats);
}
