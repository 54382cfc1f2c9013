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
// spinor: ref[(p*Vh + s)*12 + c]  <->  soa[(p*12 + c)*Vh + s] in the vector's storage format
wd_status wd_spinor_ref_to_soa(wd_context *ctx, const WdGeom &g, const double2 *ref, WdVec soa);
wd_status wd_spinor_soa_to_ref(wd_context *ctx, const WdGeom &g, WdVec soa, double2 *ref);
// gauge, one direction: ref[(p*Vh + s)*9 + k]  ->  soa[((mu*2 + p)*9 + k)*Vh + s]
wd_status wd_gauge_ref_to_soa(wd_context *ctx, const WdGeom &g, int mu, const double2 *ref,
                              double2 *soa);

// ---- BLAS-1 on double2 arrays of n complex entries
// results of reductions are written to ctx->red_partial[WD_RED_BLOCKS + slot]
wd_status wd_red_norm2(wd_context *ctx, const double2 *a, int64_t n, int slot);
wd_status wd_red_dot(wd_context *ctx, const double2 *a, const double2 *b, int64_t n, int slot);
// fold the WD_RED_BLOCKS partials written by a reduction kernel into result slot `slot`
wd_status wd_red_finish(wd_context *ctx, int slot);
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

// ---- double-float (df64) storage: float4 {re.h, im.h, re.l, im.l} per complex
wd_status wd_hop_df(wd_context *ctx, const wd_lattice *lat, const float4 *in_block, float4 *out_block,
                    const float4 *x_block, int cb, int dag, double alpha, double beta);
wd_status wd_convert_f64_to_df(wd_context *ctx, const double2 *in, float4 *out, int64_t n);
wd_status wd_convert_df_to_f64(wd_context *ctx, const float4 *in, double2 *out, int64_t n);
wd_status wd_lattice_gauge_df(wd_context *ctx, const wd_lattice *lat);

// ---- BLAS-1 dispatched on the storage of the vectors (FP64 or double-float);
// n counts complex entries.  Reductions land in result slot `slot`.
wd_status wd_v_norm2(wd_context *ctx, WdVec a, int64_t n, int slot);
wd_status wd_v_dot(wd_context *ctx, WdVec a, WdVec b, int64_t n, int slot);
wd_status wd_v_axpby(wd_context *ctx, double2 a, WdVec x, double2 b, WdVec y, int64_t n);
wd_status wd_v_xpayz(wd_context *ctx, WdVec x, double2 a, WdVec y, WdVec z, int64_t n);
wd_status wd_v_cg_update(wd_context *ctx, double2 alpha, WdVec p, WdVec q, WdVec x, WdVec r, int64_t n, int slot);
// real-scalar forms (even-odd CG): y = x + b y; x += alpha p, r -= alpha q, |r|^2 -> slot
wd_status wd_v_xpby(wd_context *ctx, WdVec x, double b, WdVec y, int64_t n);
wd_status wd_v_cg_update_real(wd_context *ctx, double alpha, WdVec p, WdVec q, WdVec x, WdVec r, int64_t n, int slot);
wd_status wd_v_copy(wd_context *ctx, WdVec dst, WdVec src, int64_t n);
wd_status wd_v_zero(wd_context *ctx, WdVec v, int64_t n);

// ---- FP32 / FP16 storage (wd_lp.cuh) with 12-real links
wd_status wd_lattice_gauge_lp(wd_context *ctx, const wd_lattice *lat, wd_precision prec);
// stop (device, optional): the launch is a no-op while *stop != 0
wd_status wd_hop_f32(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                     double alpha, double beta, const int *stop = nullptr);
wd_status wd_hop_f16(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                     double alpha, double beta, const int *stop = nullptr);
struct WdMxDev;
// The two reducing operator steps of a mixed-precision CG iteration on even
// blocks (FP32 or FP16 storage, 12-real links), with the device scalars dev:
//  * norm:   t = -D_eo in / (4a) + a p  (in = D_oe p, odd), stored; |t|^2 is
//            reduced and dev->alpha = rr / |t|^2 set by the last block;
//  * update: q = -D_eo^dag in / (4a) + a t (in = D_oe^dag t), not stored:
//            rs -= alpha q, xs += alpha p, and |rs|^2 reduced; the last block
//            applies the reliable-update rule (wd_solver.h).
// partial: at least Vh/64 + 1 doubles.  Both are no-ops while dev->stop != 0.
wd_status wd_hop_lp_norm(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec t, WdVec p, double mass,
                         WdMxDev *dev, double *partial);
wd_status wd_hop_lp_update(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec t, WdVec p, WdVec rs, WdVec xs,
                           double mass, WdMxDev *dev, double *partial);
// The reliable update's reducing steps (even outputs, Schur operator second
// hops).  partial: at least Vh/16 + 1 doubles; counter: zero at launch (the
// last block resets it).
//  * FP32: out = a x - D_eo in / (4a) (D^dag with dag), stored; |out|^2 -> *result
wd_status wd_hop_f32_norm(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, WdVec x, double mass, int dag,
                          double *partial, unsigned *counter, double *result);
//  * high precision (FP64 or double-float storage of in, x, bhat): the true
//    residual s = bhat - (a x - D_eo in / (4a)) of the Schur system, rounded
//    to FP32 into s32 (FP32 storage), and |s32|^2 -> *result
wd_status wd_hop_hi_residual(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec x, WdVec bhat, WdVec s32,
                             double mass, double *partial, unsigned *counter, double *result);
// FP64 block [12][Vh] <-> low-precision block; accumulate != 0 adds into out
wd_status wd_lp_from_f64(wd_context *ctx, int Vh, const double2 *in, WdVec out);
wd_status wd_lp_to_f64(wd_context *ctx, int Vh, WdVec in, double2 *out, int accumulate);
wd_status wd_spinor_ref_to_h16(wd_context *ctx, const WdGeom &g, const double2 *ref, WdVec f);
wd_status wd_spinor_h16_to_ref(wd_context *ctx, const WdGeom &g, WdVec f, double2 *ref);
// out_cb = alpha * D_{cb,1-cb} in_{1-cb} + beta * x_cb, dispatched on the storage
wd_status wd_hop_v(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                   double alpha, double beta);

// ---- pipelined host-buffer path: one parity block, output sites [s_lo, s_hi), given stream
wd_status wd_hop_f64_range(wd_context *ctx, cudaStream_t stream, const wd_lattice *lat, const double2 *in_block,
                           double2 *out_block, int cb, int dag, double alpha, int s_lo, int s_hi);
// n 16-byte entries src -> dst by a kernel on `stream` (for host memory the
// device addresses directly)
wd_status wd_copy_kernel(wd_context *ctx, cudaStream_t stream, const double2 *src, double2 *dst, int64_t n);
// the same on AoS (reference-layout) input and output parity blocks; with
// x_aos (the output parity's AoS block) out = alpha * hop + beta * x
wd_status wd_hop_f64_aos_range(wd_context *ctx, cudaStream_t stream, const wd_lattice *lat, const double2 *in_aos,
                               double2 *out_aos, const double2 *x_aos, int cb, int dag, double alpha, double beta,
                               int s_lo, int s_hi);
// aos holds sites [s_lo, s_hi) of one parity block, 12 complex per site; soa_block is the block's planes
wd_status wd_range_aos_to_soa(wd_context *ctx, cudaStream_t stream, int Vh, const double2 *aos, double2 *soa_block,
                              int s_lo, int s_hi);
wd_status wd_range_soa_to_aos(wd_context *ctx, cudaStream_t stream, int Vh, const double2 *soa_block, double2 *aos,
                              int s_lo, int s_hi);
