// wd_contract.cu -- point-source quark propagator and the pion two-point
// function, the consumer of multi-RHS solves (the reference's NumPy prototype
// does the same with 12 sequential solves, refs/python/main.py:50-66,
// refs/python/contraction.py:26-45).
//
// Propagator: S(x; x0)_{.,(s,c)} = M^{-1} e_{(s,c)} delta(x - x0), the 12
// columns solved together by the batch engine (or one by one in FP64 /
// double-float).  Pion correlator, by gamma5-hermiticity
// (gamma5 M gamma5 = M^dag, gamma5 = diag(1,1,-1,-1) in this basis):
//   C(t) = sum_{x in slice t} sum_{s,c} sum_{s',c'} |S(x)_{(s',c'),(s,c)}|^2
// reduced per time slice in a fixed order (deterministic).
#include <vector>
#include "wd_reduce.cuh"
#include "wd_solver.h"

namespace {

constexpr int kSliceChunk = 4096;  // sites of one parity's slice per block

struct Props {
    const double2 *col[12];
};

// one block per (t, parity, chunk): sum over its sites of sum_k |psi_k|^2
__global__ void __launch_bounds__(WD_RED_THREADS) k_slice_density(Props P, WdGeom g, int chunks_per_slice,
                                                                  double2 *partial)
{
    const int b = blockIdx.x;
    const int t = b / (2 * chunks_per_slice);
    const int rem = b - t * 2 * chunks_per_slice;
    const int par = rem / chunks_per_slice, chunk = rem - par * chunks_per_slice;
    const int slice = g.Lxh * g.L[1] * g.L[2];  // sites of one parity in one time slice
    const int s0 = t * slice + chunk * kSliceChunk;
    const int s1 = min(s0 + kSliceChunk, (t + 1) * slice);
    const size_t blk = (size_t)12 * g.Vh;
    double acc = 0.0;
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
#pragma unroll 1
        for (int k = 0; k < 12; ++k) {
            const double2 *f = P.col[k] + par * blk + s;
#pragma unroll
            for (int c = 0; c < 12; ++c) {
                const double2 v = f[(size_t)c * g.Vh];
                acc = fma(v.x, v.x, acc);
                acc = fma(v.y, v.y, acc);
            }
        }
    }
    wd_block_partial(acc, 0.0, partial);
}

__global__ void k_slice_finish(const double2 *partial, int Lt, int per_slice, double *ct)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Lt) return;
    double s = 0.0;
    for (int i = 0; i < per_slice; ++i) s += partial[t * per_slice + i].x;
    ct[t] = s;
}

}  // namespace

extern "C" wd_status wd_pion_correlator(wd_context *ctx, const wd_lattice *lat, const wd_field *const props[12],
                                        double *ct)
{
    if (!ctx || !lat || !props || !ct) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    Props P;
    for (int k = 0; k < 12; ++k) {
        if (!props[k] || props[k]->storage != WD_PREC_F64 || props[k]->lat->volume != lat->volume)
            return wd_fail(ctx, WD_ERR_BAD_ARG, "propagator columns must be FP64 fields of this lattice");
        P.col[k] = props[k]->d;
    }
    const WdGeom &g = lat->g;
    const int slice = g.Lxh * g.L[1] * g.L[2];
    const int chunks = (slice + kSliceChunk - 1) / kSliceChunk;
    const int nblocks = g.L[3] * 2 * chunks;
    WdVecBuf part, out;
    wd_status st;
    if ((st = wd_vec_alloc(ctx, part, WD_PREC_F64, nblocks)) != WD_OK) return st;  // double2 partials
    if ((st = wd_vec_alloc(ctx, out, WD_PREC_F64, (g.L[3] + 1) / 2)) != WD_OK) return st;
    k_slice_density<<<nblocks, WD_RED_THREADS, 0, ctx->stream>>>(P, g, chunks, (double2 *)part.v.p);
    WD_LAUNCHED(ctx);
    k_slice_finish<<<(g.L[3] + 127) / 128, 128, 0, ctx->stream>>>((const double2 *)part.v.p, g.L[3], 2 * chunks,
                                                                 (double *)out.v.p);
    WD_LAUNCHED(ctx);
    WD_CUDA(ctx, cudaMemcpyAsync(ct, out.v.p, g.L[3] * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_point_source(wd_context *ctx, wd_field *f, const int x[4], int spin, int colour)
{
    if (!ctx || !f || !x || spin < 0 || spin > 3 || colour < 0 || colour > 2)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "bad point source");
    if (f->storage != WD_PREC_F64) return wd_fail(ctx, WD_ERR_BAD_ARG, "point sources are FP64 fields");
    const WdGeom &g = f->lat->g;
    for (int i = 0; i < 4; ++i)
        if (x[i] < 0 || x[i] >= g.L[i]) return wd_fail(ctx, WD_ERR_BAD_ARG, "source site outside the lattice");
    const int par = (x[0] + x[1] + x[2] + x[3]) & 1;
    const int s = x[0] / 2 + g.Lxh * (x[1] + g.L[1] * (x[2] + g.L[2] * x[3]));
    wd_status st = wd_field_zero(ctx, f);
    if (st != WD_OK) return st;
    static const double2 one = {1.0, 0.0};
    WD_CUDA(ctx, cudaMemcpyAsync(f->d + ((size_t)(par * 12 + spin * 3 + colour) * g.Vh + s), &one, sizeof(one),
                                 cudaMemcpyHostToDevice, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_propagator(wd_context *ctx, const wd_lattice *lat, const int x_src[4],
                                   const wd_solver_params *prm, wd_field *const props[12], wd_solver_stats stats[12])
{
    if (!ctx || !lat || !x_src || !prm || !props) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    std::vector<wd_field *> srcs(12, nullptr);
    wd_status st = WD_OK;
    for (int k = 0; k < 12 && st == WD_OK; ++k) {
        st = wd_field_create(ctx, lat, &srcs[k]);
        if (st == WD_OK) st = wd_point_source(ctx, srcs[k], x_src, k / 3, k % 3);
    }
    if (st == WD_OK) {
        if (prm->prec == WD_PREC_F32 || prm->prec == WD_PREC_F16) {
            const wd_lattice *lats[12];
            double masses[12];
            for (int k = 0; k < 12; ++k) lats[k] = lat, masses[k] = prm->mass;
            st = wd_solve_batch(ctx, 12, lats, srcs.data(), props, masses, prm, stats);
        } else {
            for (int k = 0; k < 12 && (st == WD_OK || st == WD_ERR_NOT_CONVERGED); ++k)
                st = wd_solve(ctx, lat, srcs[k], props[k], prm, stats ? &stats[k] : nullptr);
        }
    }
    for (wd_field *f : srcs) wd_field_destroy(f);
    return st;
}
