// wd_solver.h -- operator compositions and work buffers shared by the solvers (internal).
#pragma once
#include "wd_internal.cuh"

// A device vector owned by a solver (freed on scope exit).
struct WdVecBuf {
    WdVec v;
    wd_context *ctx = nullptr;  // owner of the cached block
    WdVecBuf() = default;
    WdVecBuf(const WdVecBuf &) = delete;
    WdVecBuf &operator=(const WdVecBuf &) = delete;
    ~WdVecBuf() { release(); }
    void release();
};
wd_status wd_vec_alloc(wd_context *ctx, WdVecBuf &b, wd_precision prec, int64_t n_complex);

// M (dag=0) or M^dag on full-lattice vectors of one storage
wd_status wd_apply_M_v(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, double mass, int dag);
// Schur operator a - D_eo D_oe/(4a) (or its adjoint) on even blocks; tmp_o is an odd block
wd_status wd_apply_Mhat_v(wd_context *ctx, const wd_lattice *lat, WdVec v, WdVec out, WdVec tmp_o, double mass,
                          int dag);
// |b - M x| / |b| in FP64
wd_status wd_true_residual(wd_context *ctx, const wd_lattice *lat, const double2 *b, const double2 *x, double2 *tmp,
                           double mass, double *rel);
// mixed-precision (FP32 / FP16 inner) even-odd CG with reliable updates
wd_status wd_solve_cg_eo_mixed(wd_context *ctx, const wd_lattice *lat, const double2 *src, double2 *x,
                               const wd_solver_params *prm, wd_solver_stats *stats);
// reliable-update pieces shared by the mixed solvers (wd_mixed.cu):
// xh (FP64 or double-float) += xs (FP32), xs = 0
wd_status wd_mx_accum(wd_context *ctx, int Vh, wd_precision H, WdVec xs, WdVec xh);
// rs (FP32) <- h and p (storage L) <- h
wd_status wd_mx_from_h(wd_context *ctx, int Vh, wd_precision L, wd_precision H, WdVec h, WdVec rs, WdVec p);
// one system's buffers for a reliable update (even-parity half-lattice blocks)
struct WdMxReliable {
    WdVec xs;         // FP32 solution increment (zeroed)
    WdVec x_e;        // high-precision solution
    WdVec bhat;       // high-precision Schur source
    WdVec tmp_oh;     // high-precision odd-parity work
    WdVec scratch_h;  // high-precision work, used as two FP32 blocks
    WdVec rs;         // FP32 iterated residual, receives Mhat^dag s
};
// x_e += xs; s = bhat - Mhat x_e (high precision, kept only as FP32);
// rs = Mhat^dag s (FP32); rr = |rs|^2, ss = |s|^2; p_restart (storage L) <- rs
// when given
wd_status wd_mx_reliable(wd_context *ctx, const wd_lattice *lat, double mass, wd_precision L, wd_precision H,
                         const WdMxReliable &v, const WdVec *p_restart, double *rr, double *ss);
// the same with no host wait: |rs|^2 and |s|^2 land in the device doubles
// rr_dev and ss_dev, for the caller to fetch (several systems per fetch).
// Its kernels go to ctx->stream.  scratch (device, optional): the
// reductions' work space of wd_mx_reliable_scratch_doubles(Vh) doubles,
// owned by the caller -- needed when updates of several systems run on
// different streams at once; without it a block from the context's
// work-buffer cache (stream-ordered on ctx->stream) is used.
wd_status wd_mx_reliable_enqueue(wd_context *ctx, const wd_lattice *lat, double mass, wd_precision L, wd_precision H,
                                 const WdMxReliable &v, const WdVec *p_restart, double *rr_dev, double *ss_dev,
                                 double *scratch = nullptr);
size_t wd_mx_reliable_scratch_doubles(int Vh);
// p (storage L) = rs (FP32) + beta p
wd_status wd_mx_xpay(wd_context *ctx, int Vh, wd_precision L, WdVec rs, double beta, WdVec p);

// Device-side scalars of one mixed-precision solve.  The iteration kernels
// read and write them, so iterations run back to back with no host wait: the
// hop that forms t = Mhat p also reduces |t|^2 and sets alpha, the hop that
// forms q = Mhat^dag t applies the CG update and reduces |r_s|^2, and the
// last block of that reduction decides on the device whether a reliable
// update is due (stop = 1) -- after which every later iteration kernel in the
// queue returns at once until the host has run the update and cleared stop.
struct WdMxDev {
    double rr;        // |r_s|^2 of the current iterate
    double rr_max;    // |r_s|^2 right after the last reliable update
    double target2;   // an update is due once |r_s|^2 <= target2 (squared normal-residual target)
    double delta2;    // ... or once |r_s|^2 < delta2 * rr_max
    double tt;        // |t|^2 = |Mhat p|^2 of the running iteration
    double rr_new;    // |r_s|^2 after the running iteration's update
    float alpha, beta;
    int stop;         // 0 iterate; 1 reliable update due; 2 non-finite scalar
    int iters;        // iterations completed on the device
    unsigned count_t, count_r;  // last-block counters of the two reductions
};
