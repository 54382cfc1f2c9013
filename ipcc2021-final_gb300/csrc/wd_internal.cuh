// wd_internal.cuh -- shared definitions of the GB300 Wilson-Dslash library.
//
// Device layout (all fields even-odd split, structure of arrays):
//   spinor, FP64:  double2 psi[parity][comp 0..11][Vh]         comp = spin*3 + colour
//   gauge,  FP64:  double2 U[mu 0..3][parity][k 0..8][Vh]      k = row*3 + col
// Site s of parity p has half-x index xh = s % Lxh and row index
// s / Lxh = y + Ly*(z + Lz*t); its full x is 2*xh + ((y+z+t+p)&1).
// This is the reference's eo ordering (include/operator.h:62-67) with the
// 12 (or 9) complex components of a site spread over planes of Vh entries,
// so a warp's 32 threads read 32 consecutive 16-byte entries per component.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <map>
#include <string>
#include <unordered_map>
#include "../../include/wilson_gb300.h"

#define WD_MAX_SITES (int64_t(1) << 30)

// pinned host bytes for reading back a solver's device-side scalars
constexpr size_t WD_STATE_HOST_BYTES = 4096;

// compute chunks and upload units of the pipelined host-buffer hopping term
constexpr int WD_MAX_CHUNKS = 16;
constexpr int WD_MAX_UPLOADS = 32;

struct WdGeom {
    int L[4];  // Lx, Ly, Lz, Lt
    int Lxh;   // Lx / 2
    int Vh;    // sites per parity
};

struct wd_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // device->host copies overlapped with compute
    cudaStream_t h2d_stream = nullptr;   // host->device copies overlapped with compute
    cudaStream_t aux_stream = nullptr;   // second compute stream of the pipelined host path
    int pageable_access = 0;             // the device reads and writes pageable host memory
    cudaEvent_t chunk_done[WD_MAX_CHUNKS] = {};  // compute -> copy hand-off of the pipelined host path
    cudaEvent_t chunk_in[WD_MAX_UPLOADS] = {};   // upload -> compute hand-off
    std::string last_error;
    uint64_t launches = 0;
    // scratch: reduction partials (double2 per block) and the staging area
    // used for layout conversion of host buffers.
    void *red_partial = nullptr;  // WD_RED_BLOCKS double2 (+ result slots)
    void *red_result = nullptr;   // pinned host mirror of the reduction results
    void *state_host = nullptr;   // pinned host mirror of a solver's device scalars (WD_STATE_HOST_BYTES)
    int *dev_err = nullptr;       // device flag: a kernel's bounded wait gave up (wd_context_device_check)
    void *staging = nullptr;      // device staging buffer for reference-layout copies
    size_t staging_bytes = 0;
    // cached host-buffer path state (wd_host_*): one lattice + fields
    wd_lattice *host_lat = nullptr;
    const double *host_gauge_ptr[4] = {nullptr, nullptr, nullptr, nullptr};
    uint64_t host_gauge_print = 0;  // sampled fingerprint of the cached links
    wd_field *host_f[3] = {nullptr, nullptr, nullptr};
    // caching allocator for solver work buffers: blocks freed by one call are
    // reused by the next in stream order (one stream per context)
    std::multimap<size_t, void *> pool_free;
    std::unordered_map<void *, size_t> pool_used;
    size_t pool_bytes = 0;
    // host-side failure injection for tests: after this many more successful
    // field / work-buffer allocations the next ones fail with WD_ERR_OOM
    // (-1: off)
    int fail_alloc_after = -1;
};

// true when the injected allocation failure applies to this allocation
inline bool wd_alloc_fails(wd_context *ctx)
{
    if (ctx->fail_alloc_after < 0) return false;
    if (ctx->fail_alloc_after == 0) return true;
    --ctx->fail_alloc_after;
    return false;
}

// Work-buffer allocation through the context's cache (stream-ordered reuse;
// on allocation failure the cached blocks are released and the call retried).
wd_status wd_dev_alloc(wd_context *ctx, void **p, size_t bytes);
void wd_dev_free(wd_context *ctx, void *p);
void wd_pool_release(wd_context *ctx);

struct wd_lattice {
    wd_context *ctx = nullptr;
    WdGeom g;
    int64_t volume = 0;
    double2 *gauge = nullptr;     // FP64 [mu][parity][9][Vh]
    float4 *gauge_df = nullptr;   // double-float copy, same shape (lazily built)
    void *gauge_f32 = nullptr;    // FP32 12-real links [mu][parity][3][Vh] float4 (lazily built)
    void *gauge_h12 = nullptr;    // FP16 12-real links: uint4 [8][Vh] then uint2 [8][Vh] (lazily built)
};

struct wd_field {
    const wd_lattice *lat = nullptr;
    wd_precision storage = WD_PREC_F64;
    void *data = nullptr;     // [parity][12][Vh] entries of the storage type
    float *scale = nullptr;   // FP16 storage: [parity][Vh] per-site scales (inside data)
    double2 *d = nullptr;     // == data for FP64 storage, else null
};

// A typed view of a spinor array (one parity block or a whole field).
struct WdVec {
    void *p = nullptr;
    float *scale = nullptr;  // FP16 only
    wd_precision prec = WD_PREC_F64;
};

// bytes of one complex entry in each storage format (FP16: half2 + scale per 12 entries)
inline size_t wd_entry_bytes(wd_precision p)
{
    switch (p) {
    case WD_PREC_F64: return 16;
    case WD_PREC_DF64: return 16;
    case WD_PREC_F32: return 8;
    default: return 4;
    }
}

// view of parity block `par` (0/1) of a field
inline WdVec wd_block(const wd_field *f, int par)
{
    WdVec v;
    v.prec = f->storage;
    const size_t blk = (size_t)12 * f->lat->g.Vh;
    v.p = (char *)f->data + par * blk * wd_entry_bytes(f->storage);
    if (f->scale) v.scale = f->scale + (size_t)par * f->lat->g.Vh;
    return v;
}
inline WdVec wd_whole(const wd_field *f)
{
    WdVec v;
    v.prec = f->storage;
    v.p = f->data;
    v.scale = f->scale;
    return v;
}
inline WdVec wd_offset(WdVec v, int64_t entries, int64_t sites)
{
    v.p = (char *)v.p + entries * (int64_t)wd_entry_bytes(v.prec);
    if (v.scale) v.scale += sites;
    return v;
}

// Error plumbing: record text on the context and return a status.
wd_status wd_fail(wd_context *ctx, wd_status s, const std::string &msg);
wd_status wd_cuda_check(wd_context *ctx, cudaError_t e, const char *what);
#define WD_CUDA(ctx, call)                                        \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return wd_cuda_check(ctx, _e, #call); \
    } while (0)
#define WD_LAUNCHED(ctx)                                                     \
    do {                                                                     \
        (ctx)->launches++;                                                   \
        cudaError_t _e = cudaGetLastError();                                 \
        if (_e != cudaSuccess) return wd_cuda_check(ctx, _e, "kernel launch"); \
    } while (0)

// ---------------------------------------------------------------- complex
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 ctimesi(double2 a) { return make_double2(-a.y, a.x); }

// --------------------------------------------------------------- geometry
// Coordinates of site s in parity p.
struct WdSite {
    int xh, y, z, t, xodd;
};

__device__ __forceinline__ WdSite wd_site(const WdGeom &g, int s, int p)
{
    WdSite c;
    c.xh = s % g.Lxh;
    int r = s / g.Lxh;
    c.y = r % g.L[1];
    r /= g.L[1];
    c.z = r % g.L[2];
    c.t = r / g.L[2];
    c.xodd = (c.y + c.z + c.t + p) & 1;
    return c;
}

// Index, within the opposite parity, of the neighbour of site s in direction
// mu (0..3), forward (fwd=true) or backward.  Periodic in every direction:
// this is where the reference's MPI halo exchange used to be.
__device__ __forceinline__ int wd_neighbour(const WdGeom &g, int s, const WdSite &c, int mu, bool fwd)
{
    switch (mu) {
    case 0: {
        // full x = 2 xh + xodd; x+1 has half index xh (xodd=0) or xh+1 (xodd=1)
        int xh;
        if (fwd) xh = c.xodd ? (c.xh + 1 == g.Lxh ? 0 : c.xh + 1) : c.xh;
        else xh = c.xodd ? c.xh : (c.xh == 0 ? g.Lxh - 1 : c.xh - 1);
        return s - c.xh + xh;
    }
    case 1: {
        int step = g.Lxh;
        if (fwd) return c.y + 1 == g.L[1] ? s - step * (g.L[1] - 1) : s + step;
        return c.y == 0 ? s + step * (g.L[1] - 1) : s - step;
    }
    case 2: {
        int step = g.Lxh * g.L[1];
        if (fwd) return c.z + 1 == g.L[2] ? s - step * (g.L[2] - 1) : s + step;
        return c.z == 0 ? s + step * (g.L[2] - 1) : s - step;
    }
    default: {
        int step = g.Lxh * g.L[1] * g.L[2];
        if (fwd) return c.t + 1 == g.L[3] ? s - step * (g.L[3] - 1) : s + step;
        return c.t == 0 ? s + step * (g.L[3] - 1) : s - step;
    }
    }
}

// ------------------------------------------------------------ spin algebra
// Projector and reconstruction of the reference's gamma basis
// (src/dslash.cpp:544-873).  For direction mu, forward (F) or backward, and
// dagger flag, let sg = (F ? -1 : +1) * (dag ? -1 : +1):
//   mu=0 (x): h0 = s0 + sg i s3, h1 = s1 + sg i s2;  d2 += -sg i t1, d3 += -sg i t0
//   mu=1 (y): h0 = s0 - sg s3,   h1 = s1 + sg s2;    d2 +=  sg t1,   d3 += -sg t0
//   mu=2 (z): h0 = s0 + sg i s2, h1 = s1 - sg i s3;  d2 += -sg i t0, d3 +=  sg i t1
//   mu=3 (t): h0 = s0 + sg s2,   h1 = s1 + sg s3;    d2 +=  sg t0,   d3 +=  sg t1
// with t = W h (W = U_mu(x) forward, U_mu(x-mu)^dag backward) and d0 += t0, d1 += t1.
// Written once as templates over the arithmetic type T (double2-like complex
// with +, -, *scalar and "times i").

template <int MU, int SG, typename C>
__device__ __forceinline__ void wd_project(const C &s0, const C &s1, const C &s2, const C &s3, C &h0, C &h1);

template <int MU, int SG, typename C>
__device__ __forceinline__ void wd_reconstruct(const C &t0, const C &t1, C &d0, C &d1, C &d2, C &d3);
