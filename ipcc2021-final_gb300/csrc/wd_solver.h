// wd_solver.h -- operator compositions shared by the solvers (internal).
#pragma once
#include "wd_internal.cuh"

// out_cb = alpha * D_{cb,1-cb} in_{1-cb} + beta * x_cb on FP64 blocks.
wd_status wd_hop(wd_context *ctx, const wd_lattice *lat, const double2 *in_block, double2 *out_block,
                 const double2 *x_block, int cb, int dag, double alpha, double beta, wd_precision prec);
wd_status wd_apply_M(wd_context *ctx, const wd_lattice *lat, const double2 *in, double2 *out, double mass,
                     int dag, wd_precision prec);
wd_status wd_apply_Mhat(wd_context *ctx, const wd_lattice *lat, const double2 *v, double2 *out,
                        double2 *tmp_o, double mass, int dag, wd_precision prec);
wd_status wd_true_residual(wd_context *ctx, const wd_lattice *lat, const double2 *b, const double2 *x,
                           double2 *tmp, double mass, double *rel);
// mixed-precision (FP32 / FP16 inner) even-odd CG with FP64 reliable updates
wd_status wd_solve_cg_eo_mixed(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x,
                               const wd_solver_params *prm, wd_solver_stats *stats);
