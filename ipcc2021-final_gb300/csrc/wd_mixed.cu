// wd_mixed.cu -- mixed-precision even-odd CG with FP64 reliable updates.
#include "wd_kernels.h"
#include "wd_solver.h"

wd_status wd_solve_cg_eo_mixed(wd_context *ctx, const wd_lattice *, const double2 *, double2 *,
                               const wd_solver_params *, wd_solver_stats *)
{
    return wd_fail(ctx, WD_ERR_BAD_ARG, "mixed-precision solver not built yet");
}
