/*
 * wilson_gb300.h -- C ABI of the GB300 (sm_103a) Wilson-fermion Dslash and CG
 * library.
 *
 * Every entry point takes plain pointers and sizes and returns a wd_status.
 * The host-buffer entry points (wd_host_*) take and return fields in the
 * reference's layout, so they replace the reference's functions one for one:
 *
 *   fermion  psi[(eo*12 + spin*3 + colour)]   complex double, 16-byte entries
 *   gauge    U[mu][(eo*9 + row*3 + col)]      U_mu(x), link from x to x+mu
 *   eo       = lex/2 + ((x+y+z+t)&1) * V/2,   lex = x + Lx*(y + Ly*(z + Lz*t))
 *   dims     = {Lx, Ly, Lz, Lt}; Lx even; periodic boundaries in all directions
 *
 * (reference: include/operator.h:56-67, src/lattice_fermion.cpp:15-22,
 *  src/load_gauge.cpp:141-161).  The handle-based entry points keep gauge and
 * fermion fields resident in device memory in an even-odd split,
 * structure-of-arrays layout; layout conversion happens on the device.
 *
 * Threading: a context owns one CUDA stream; calls on one context must come
 * from one host thread at a time.  Different contexts are independent.
 */
#ifndef WILSON_GB300_H
#define WILSON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum wd_status {
    WD_OK = 0,
    WD_ERR_BAD_DIMS = 1,      /* lattice extents invalid (Lx odd, <= 0, too large) */
    WD_ERR_OOM = 2,           /* device allocation failed or HBM budget exceeded */
    WD_ERR_NOT_CONVERGED = 3, /* solver reached max iterations */
    WD_ERR_TIMEOUT = 4,       /* a bounded device wait ran out */
    WD_ERR_CUDA = 5,          /* CUDA runtime error (see wd_last_error) */
    WD_ERR_BAD_ARG = 6,       /* null pointer, mismatched lattice, bad enum */
    WD_ERR_NO_DEVICE = 7,     /* no CUDA device / wrong architecture */
    WD_ERR_NAN = 8            /* solver produced a non-finite residual */
} wd_status;

/* Arithmetic used by the hopping kernels. */
typedef enum wd_precision {
    WD_PREC_F64 = 0,  /* native FP64 */
    WD_PREC_DF64 = 1, /* double-float: FP32 hi/lo pairs, ~48-bit mantissa, FP64-class results */
    WD_PREC_F32 = 2,  /* FP32 storage and arithmetic */
    WD_PREC_F16 = 3   /* FP16 spinors with a per-site FP32 scale, 12-real links, FP32 arithmetic */
} wd_precision;

typedef struct wd_context wd_context; /* device, stream, scratch */
typedef struct wd_lattice wd_lattice; /* lattice extents + resident gauge field */
typedef struct wd_field wd_field;     /* resident full-lattice spinor field (FP64) */

/* ---- context ---------------------------------------------------------- */
wd_status wd_context_create(int device, wd_context **ctx);
void wd_context_destroy(wd_context *ctx);
const char *wd_status_string(wd_status s);
/* Text of the last error recorded on this context ("" if none). */
const char *wd_last_error(const wd_context *ctx);
/* Wait for all work queued on the context's stream. */
wd_status wd_context_sync(wd_context *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or overlap work. */
void *wd_context_stream(wd_context *ctx);
/* Device kernels launched on this context since creation (bookkeeping for benchmarks). */
uint64_t wd_context_launches(const wd_context *ctx);
/* Wait for the context's stream, then report (and clear) the device-side
 * error flag: WD_ERR_TIMEOUT if a kernel's bounded wait gave up since the
 * last check (the TMA-staged FP16 hopping kernel waits on its copies for at
 * most 0.5 s, after which the block writes nothing and sets the flag; its
 * output is then undefined), else WD_OK. */
wd_status wd_context_device_check(wd_context *ctx);
/* Testing aid, host-side failure injection: after n more successful field or
 * work-buffer allocations on this context, the next ones fail with
 * WD_ERR_OOM; n < 0 turns it off (the default).  Returns the previous
 * setting (the allocations left before failing, or -1). */
int wd_debug_fail_allocations_after(wd_context *ctx, int n);
/* Testing aid for the bounded device waits: one warp waits on a shared-memory
 * barrier that nothing completes; the wait gives up after its bound (0.5 s)
 * and sets the device error flag, as a kernel whose copies never landed
 * would, so the next wd_context_device_check returns WD_ERR_TIMEOUT.
 * *waited_seconds: how long the wait ran, as the device's timer measured it. */
wd_status wd_debug_expire_wait(wd_context *ctx, double *waited_seconds);

/* ---- gauge field (replaces lattice_gauge, include/lattice_gauge.h:11-26) ---- */
/* Upload four reference-layout link arrays (each V*9 complex doubles).
 * The library keeps its own device copy; the host arrays may be freed after. */
wd_status wd_lattice_create(wd_context *ctx, const int dims[4], const double *const gauge[4],
                            wd_lattice **lat);
/* Refresh the device copy of the links from host arrays of the same lattice. */
wd_status wd_lattice_update(wd_context *ctx, wd_lattice *lat, const double *const gauge[4]);
void wd_lattice_destroy(wd_lattice *lat);
/* Sites of the full lattice. */
int64_t wd_lattice_volume(const wd_lattice *lat);

/* ---- fermion fields (replaces lattice_fermion, include/lattice_fermion.h:12-32) ---- */
wd_status wd_field_create(wd_context *ctx, const wd_lattice *lat, wd_field **f);
/* A field stored in another format (WD_PREC_DF64 float pairs, WD_PREC_F32, or
 * WD_PREC_F16 with per-site scale); upload/download convert from/to FP64.
 * Operators on such fields run in the arithmetic of their storage. */
wd_status wd_field_create_prec(wd_context *ctx, const wd_lattice *lat, wd_precision prec, wd_field **f);
wd_precision wd_field_precision(const wd_field *f);
void wd_field_destroy(wd_field *f);
/* host: V*12 complex doubles in the reference layout */
wd_status wd_field_upload(wd_context *ctx, wd_field *f, const double *host);
wd_status wd_field_download(wd_context *ctx, const wd_field *f, double *host);
wd_status wd_field_zero(wd_context *ctx, wd_field *f);
wd_status wd_field_copy(wd_context *ctx, wd_field *dst, const wd_field *src);

/* ---- operators on resident fields ------------------------------------ */
/* DslashoffdNew (src/dslash_new.cpp:1341) / Dslashoffd (src/dslash.cpp:38):
 * out[cb] = -1/2 * D_{cb,1-cb} in[1-cb]; out[1-cb] = 0.  dag != 0 gives the
 * hermitian conjugate hopping term.  prec selects the kernel arithmetic. */
wd_status wd_dslash_offd(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                         int dag, int cb, wd_precision prec);
/* The even-odd hopping half-application alone (the unit "one even-odd Dslash"
 * of the benchmarks; the inner operator of DslashoffdNew, src/dslash_new.cpp:1831-2296):
 * out[cb] = -1/2 * D_{cb,1-cb} in[1-cb]; out[1-cb] is left untouched. */
wd_status wd_dslash_eo(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                       int dag, int cb, wd_precision prec);
/* DslashEEOONew (src/dslash_new.cpp:1301): out = (4+mass) in on all sites. */
wd_status wd_dslash_eeoo(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                         double mass);
/* DslashNew / Dslash (src/invert.cpp:123-156): out = M in (dag=0) or M^dag in. */
wd_status wd_dslash_full(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                         double mass, int dag, wd_precision prec);
/* norm_2 (include/operator_mpi.h:15): sum |a_i|^2, FP64, deterministic order. */
wd_status wd_norm2(wd_context *ctx, const wd_field *a, double *out);
/* vector_p (include/operator_mpi.h:48): sum conj(a_i) b_i -> out[0] + i out[1]. */
wd_status wd_dot(wd_context *ctx, const wd_field *a, const wd_field *b, double out[2]);

/* ---- solvers --------------------------------------------------------- */
typedef enum wd_solver_kind {
    WD_SOLVER_CGNR_REF = 0, /* the reference CGinvert: full-lattice CG on M^dag M x = M^dag b,
                               absolute stop |r_normal| < tol (src/invert.cpp:25-121) */
    WD_SOLVER_CG_EO = 1     /* even-odd (Schur) preconditioned CG on the normal equations of
                               Mhat = a - D_eo D_oe/(4a); relative stop on |b - Mx|/|b| */
} wd_solver_kind;

typedef struct wd_solver_params {
    wd_solver_kind kind;
    double mass;
    double tol;          /* CGNR_REF: absolute |r|; CG_EO: target relative true residual */
    int max_iter;
    wd_precision prec;   /* arithmetic of the inner hopping kernel; FP64/DF64 or mixed F32/F16 */
    double delta;        /* reliable-update threshold for mixed precision (0 -> 0.1) */
    int use_initial_guess; /* CG_EO: 1 = start from dest, 0 = start from zero */
    wd_precision prec_reliable; /* mixed precision: arithmetic of the reliable updates and of
                                   the solution accumulation, WD_PREC_F64 or WD_PREC_DF64 */
} wd_solver_params;

typedef struct wd_solver_stats {
    int iterations;        /* CG iterations (inner iterations for mixed precision) */
    int reliable_updates;  /* FP64 residual recomputations */
    double residual;       /* solver's final residual as defined by the solver kind */
    double true_residual;  /* |b - M x| / |b| recomputed in FP64 on the device */
    double seconds;        /* wall time of the solve on the device stream */
    int converged;
} wd_solver_stats;

void wd_solver_params_default(wd_solver_params *p);

/* CGinvert (src/invert.cpp:25-121) on resident fields; dest holds the initial
 * guess on entry (the reference's own random guess is generated by the C++
 * compatibility layer with rand(), as src/invert.cpp:42-44 does). */
wd_status wd_solve(wd_context *ctx, const wd_lattice *lat, const wd_field *src, wd_field *dest,
                   const wd_solver_params *params, wd_solver_stats *stats);

/* Many systems solved together (multi-RHS on one lattice, and lattices of
 * uneven volume, in any mix): system i solves M(lats[i], masses[i]) x = b on
 * srcs[i] -> dests[i] (FP64 fields).  Systems on the same lattice handle
 * share link loads.  Mixed-precision even-odd CG: params->prec = WD_PREC_F32
 * or WD_PREC_F16 inner operator, params->prec_reliable for the reliable
 * updates, params->tol the relative true residual of every system.  One
 * batched launch per operator application covers all systems; iterations
 * run as a captured CUDA graph with per-system convergence masking.
 * stats (nsys entries, may be NULL) receive each system's counts and FP64
 * true residual.  Systems need no relation to the reference; this entry
 * point has no counterpart there (it replaces a loop of CGinvert calls). */
wd_status wd_solve_batch(wd_context *ctx, int nsys, const wd_lattice *const *lats, const wd_field *const *srcs,
                         wd_field *const *dests, const double *masses, const wd_solver_params *params,
                         wd_solver_stats *stats);

/* ---- propagator and pion correlator (the reference prototype's refs/python/main.py:50-66,
 *      refs/python/contraction.py:26-45, in this library's gamma basis) ---- */
/* f = unit point source at site x (global coordinates), spin s, colour c (FP64 field). */
wd_status wd_point_source(wd_context *ctx, wd_field *f, const int x[4], int spin, int colour);
/* The 12 columns props[s*3+c] = M^-1 point_source(x_src, s, c), solved with params (a mixed
 * prec batches all 12 as right-hand sides of one lattice); stats may be NULL. */
wd_status wd_propagator(wd_context *ctx, const wd_lattice *lat, const int x_src[4], const wd_solver_params *params,
                        wd_field *const props[12], wd_solver_stats stats[12]);
/* Pion two-point function ct[t] = sum over the sites of time slice t (absolute t) of
 * sum_{columns} |psi|^2 (gamma5-hermiticity), t = 0..Lt-1, deterministic order. */
wd_status wd_pion_correlator(wd_context *ctx, const wd_lattice *lat, const wd_field *const props[12], double *ct);

/* ---- serving: continuous batching of solve requests (no counterpart in the reference) ---- */
typedef struct wd_server wd_server;
typedef struct wd_server_config {
    wd_precision prec;          /* WD_PREC_F32 / WD_PREC_F16: batched mixed precision;
                                   WD_PREC_F64: the plain FP64 solver, one system at a time */
    wd_precision prec_reliable; /* reliable updates of the mixed solver: WD_PREC_F64 or WD_PREC_DF64 */
    double hbm_budget_bytes;    /* admission limit: resident links + admitted requests */
    int max_systems;            /* right-hand sides iterating together */
    int max_iter;
    double delta;               /* reliable-update threshold (0 -> 0.1) */
} wd_server_config;
/* defaults: FP16 inner solver (the fastest), double-float reliable updates, 150 GB budget,
 * 256 systems, 5000 iterations, delta 0.1 */
void wd_server_config_default(wd_server_config *c);
wd_status wd_server_create(wd_context *ctx, const wd_server_config *cfg, wd_server **server);
void wd_server_destroy(wd_server *server);
/* make a gauge field resident (reference layout); its derived link copies count against the budget */
wd_status wd_server_add_lattice(wd_server *server, const int dims[4], const double *const gauge[4], int *lattice_id);
/* queue a request of nsrc right-hand sides: host sources (reference layout), or, when sources is
 * NULL, unit-norm Gaussian sources generated on the device from seeds[k]; WD_ERR_OOM if it could
 * never fit the budget. */
wd_status wd_server_submit(wd_server *server, int lattice_id, int nsrc, const double *const *sources,
                           const uint64_t *seeds, double mass, double tol, int64_t *request_id);
/* admit queued requests that fit, advance every admitted system by one quantum, retire finished ones.
 * A request whose admission fails (device allocation) leaves the queue with its unadmitted systems
 * completed as failed (converged = 0, iterations = 0) and the error is returned; the server stays
 * usable. */
wd_status wd_server_step(wd_server *server, int *completed);
/* done: 1 when finished; then solutions (nsrc host arrays, may be NULL), stats (nsrc) and the
 * submit-to-finish latency are returned and the request's device memory is released */
wd_status wd_server_poll(wd_server *server, int64_t request_id, int *done, double *const *solutions,
                         wd_solver_stats *stats, double *latency_s);
wd_status wd_server_status(const wd_server *server, int *queued, int *active_systems, double *bytes_in_use);

/* check (src/check.cpp:28-110): out[0]=|b| out[1]=|x| out[2..3]=(Mb,Mb) out[4..5]=(b,M^dag M b)
 * out[6..7]=(Mx,Mx) out[8..9]=(x,M^dag M x) out[10]=|Mx-b| out[11]=|M^dag M x - M^dag b| */
wd_status wd_check(wd_context *ctx, const wd_lattice *lat, const wd_field *b, const wd_field *x,
                   double mass, double out[12]);

/* ---- host-buffer entry points (reference layout in and out) ------------ */
/* Each uploads its inputs, runs on the device and downloads the result within
 * the call.  gauge is the reference's U.A[4].  After a return other than
 * WD_OK the contents of dest are undefined (it may be partly written); no
 * copy or kernel touches src or dest after the call returns. */
wd_status wd_host_dslash_offd(wd_context *ctx, const int dims[4], const double *const gauge[4],
                              const double *src, double *dest, int dag, int cb);
wd_status wd_host_dslash_full(wd_context *ctx, const int dims[4], const double *const gauge[4],
                              const double *src, double *dest, double mass, int dag);
/* CGinvert(complex<double>* ...) (src/invert.cpp:15-23).  dest holds the
 * initial guess on entry and the solution on return. */
wd_status wd_host_cg(wd_context *ctx, const int dims[4], const double *const gauge[4],
                     const double *src, double *dest, const wd_solver_params *params,
                     wd_solver_stats *stats);

/* ---- allocation-free dot product (no counterpart in the reference) ------- */
/* sum_i conj(a_i) b_i over n complex doubles, for callers that cannot
 * allocate device memory: codes that hand all of HBM to their own pool, and
 * latency-critical loops that must not call cudaMalloc/cudaFree (both
 * synchronise the device).  a and b are device pointers (16-byte aligned) to
 * n interleaved (re, im) pairs; out is a device pointer (8-byte aligned) that
 * receives re, im.  Work is queued on `stream` (a cudaStream_t, NULL = the
 * default stream); the call itself allocates nothing.
 * Limit: n <= 134217728 (32768 partial sums of 4096 entries in a fixed 512 KiB
 * device array that every GPU loading the library keeps until exit); larger n
 * returns WD_ERR_BAD_ARG.  The first call on a device looks up that array's
 * device address and should come before any stream capture.  All calls share
 * the array, so calls that overlap on the GPU race and give undefined results.
 * The looked-up address is kept for the life of the process: resetting a
 * device (cudaDeviceReset) after the first call on it is not supported. */
wd_status wd_dot_noalloc(const double *a, const double *b, int64_t n, double *out, void *stream);

/* ---- diagnostics (no counterpart in the reference) ---------------------- */
/* Measured FMA throughput of this device: FP64 and FP32, in TFLOP/s (an FMA
 * counts two flops).  Used as the compute roof of the hopping kernels. */
wd_status wd_diag_fma_peak(wd_context *ctx, double *fp64_tflops, double *fp32_tflops);

/* DslashEEOONew / DslashEE / DslashOO (src/dslash_new.cpp:1301, src/dslash.cpp:11-35) on
 * host arrays: dest = (4+mass) src on parity `parity` (0 even, 1 odd; the other
 * half of dest is zeroed) or on both halves (parity = -1). */
wd_status wd_host_dslash_eeoo(wd_context *ctx, const int dims[4], const double *src, double *dest, double mass,
                              int parity);
/* norm_2 / vector_p on host arrays of n complex doubles (any layout):
 * copied to the device and reduced there in FP64, deterministic order. */
wd_status wd_host_norm2(wd_context *ctx, int64_t n, const double *a, double *out);
wd_status wd_host_dot(wd_context *ctx, int64_t n, const double *a, const double *b, double out[2]);
/* check (src/check.cpp:28-110) on host arrays in the reference layout; out as wd_check. */
wd_status wd_host_check(wd_context *ctx, const int dims[4], const double *const gauge[4], const double *b,
                        const double *x, double mass, double out[12]);

/* Launch-shape autotuner: the first call of a hopping kernel for a lattice
 * half-volume times its launch variants and keeps the fastest.  The report
 * lists "device kernel Vh variant ms" lines; returns its length.  Tuning
 * can be switched off (variant 0 everywhere); WD_TUNE=0 does the same and
 * WD_TUNE_CACHE=<file> persists decisions. */
int wd_tune_report(char *buf, int len);
void wd_tune_enable(int on);
/* Pin the launch variant of one kernel ("hop_f64", "hop_df64", "hop_f32",
 * "hop_f16") for one device and half-volume, bypassing the timing (every
 * variant computes bit-identical results; only the launch shape differs).
 * variant < 0 removes the pin.  Returns 0, or -1 for a bad argument or a
 * variant beyond the kernel's count once that count is known. */
int wd_tune_pin(int device, const char *kernel, int half_volume, int variant);
/* Number of launch variants of a kernel, known after its first launch (else 0). */
int wd_tune_variants(const char *kernel);

/* ---- gauge-configuration files (host only) ------------------------------- */
/* The reference's load_gauge reads one format (src/load_gauge.cpp:58-161);
 * its refs/utils_nersc_lat.cpp reads NERSC and ILDG files.  All are read
 * here into the reference layout (4 arrays of V*9 complex, eo order):
 *   REF   big-endian doubles [site][mu][row][col][re,im], the payload the
 *         whole file or ending 280 bytes before its end (LIME framing);
 *   NERSC ASCII header, 3x3 or two-row (row 2 rebuilt) links, IEEE64/32,
 *         big or little endian, DIMENSION_i checked against dims;
 *   ILDG  the last V*72 big-endian values of the file (LIME binary record),
 *         double precision when the file holds them, else single.
 * AUTO takes NERSC when the file starts with BEGIN_HEADER, else REF when the
 * size fits it, else single-precision ILDG.  format_found (optional)
 * receives the format read.  BAD_DIMS when the file cannot hold the
 * lattice, BAD_ARG when it cannot be opened or read. */
typedef enum {
    WD_GAUGE_FILE_AUTO = 0,
    WD_GAUGE_FILE_REF = 1,
    WD_GAUGE_FILE_NERSC = 2,
    WD_GAUGE_FILE_ILDG = 3
} wd_gauge_file_format;
wd_status wd_read_gauge_file(const char *path, const int dims[4], int format, double *const gauge[4],
                             int *format_found);

/* ---- seeded synthetic inputs (host, deterministic) ---------------------- */
/* Gauge links U = exp(i eps H) re-unitarised to SU(3), H Gaussian traceless
 * hermitian; written in the reference layout (4 arrays of V*9 complex). */
wd_status wd_gen_gauge(const int dims[4], uint64_t seed, double eps, double *const gauge[4]);
/* Complex Gaussian source on V*12 entries, normalised to unit L2. */
wd_status wd_gen_source(const int dims[4], uint64_t seed, double *src);

/* ---- short names of the drop-in boundary -------------------------------- */
/* Forwards to the entry points above: context, gauge upload (the reference
 * layout of src/load_gauge.cpp:141-161 -> a resident lattice), fermion
 * upload/download (eo*12 + spin*3 + colour), the full operator M
 * (DslashNew, src/invert.cpp:138-156) in FP64, and CG. */
wd_status wd_ctx_create(int device, wd_context **ctx);
void wd_ctx_destroy(wd_context *ctx);
wd_status wd_gauge_upload(wd_context *ctx, const double *const ref_layout[4], const int dims[4], wd_lattice **lat);
wd_status wd_fermion_upload(wd_context *ctx, wd_field *f, const double *ref_layout);
wd_status wd_fermion_download(wd_context *ctx, const wd_field *f, double *ref_layout);
wd_status wd_M(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out, double mass, int dag);
/* CG on the field's lattice.  flags: WD_CG_REFERENCE selects the reference's
 * CG recurrences (CGinvert, src/invert.cpp:25-121) instead of the even-odd
 * CG; bits 1-2 the inner precision (wd_precision << 1); WD_CG_RELIABLE_DF64
 * double-float reliable updates; WD_CG_INITIAL_GUESS starts from dest. */
enum {
    WD_CG_REFERENCE = 1,
    WD_CG_RELIABLE_DF64 = 8,
    WD_CG_INITIAL_GUESS = 16
};
wd_status wd_cg(wd_context *ctx, const wd_lattice *lat, const wd_field *src, wd_field *dest, double mass, double tol,
                int max_iter, int flags, wd_solver_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* WILSON_GB300_H */
