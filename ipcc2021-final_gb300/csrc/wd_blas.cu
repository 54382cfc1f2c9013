// wd_blas.cu -- layout conversion and BLAS-1 with deterministic reductions.
//
// Reductions (norm_2 / vector_p of include/operator_mpi.h:15-79) use a fixed
// grid of WD_RED_BLOCKS blocks: each block folds its grid-stride share with
// warp shuffles into one FP64 partial, and a single-block pass adds the
// partials in a fixed tree order.  The result is bitwise reproducible for a
// given length and lands in a device slot, so solvers can keep it on the
// device.  Double-float vectors accumulate per thread in double-float on the
// FP32 pipe and convert to FP64 once per thread.
#include "wd_kernels.h"
#include "wd_df.cuh"

namespace {

constexpr int kTile = 64;  // sites per transpose tile

// ------------------------------------------------ storage converters
struct StF64 {
    __device__ static void store(void *out, int c, int s, int Vh, double2 v) { ((double2 *)out)[(size_t)c * Vh + s] = v; }
    __device__ static double2 load(const void *in, int c, int s, int Vh) { return ((const double2 *)in)[(size_t)c * Vh + s]; }
};
struct StDF {
    __device__ static void store(void *out, int c, int s, int Vh, double2 v) { ((float4 *)out)[(size_t)c * Vh + s] = df_pack(v); }
    __device__ static double2 load(const void *in, int c, int s, int Vh) { return df_unpack(((const float4 *)in)[(size_t)c * Vh + s]); }
};
// FP32: components in pairs, plane j = comps (2j, 2j+1) as float4 {re0, im0, re1, im1}
struct StF32 {
    __device__ static void store(void *out, int c, int s, int Vh, double2 v)
    {
        ((float2 *)out)[((size_t)(c >> 1) * Vh + s) * 2 + (c & 1)] = make_float2((float)v.x, (float)v.y);
    }
    __device__ static double2 load(const void *in, int c, int s, int Vh)
    {
        const float2 f = ((const float2 *)in)[((size_t)(c >> 1) * Vh + s) * 2 + (c & 1)];
        return make_double2(f.x, f.y);
    }
};

template <int NC, class St>
__global__ void __launch_bounds__(256) k_aos_to_soa(const double2 *__restrict__ aos, void *__restrict__ soa,
                                                    int Vh, size_t block_bytes)
{
    __shared__ double2 tile[kTile * NC];
    const int b = blockIdx.y;
    const int s0 = blockIdx.x * kTile;
    const int ns = min(kTile, Vh - s0);
    const double2 *src = aos + ((size_t)b * Vh + s0) * NC;
    void *dst = (char *)soa + b * block_bytes;
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) tile[i] = src[i];
    __syncthreads();
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        St::store(dst, c, s0 + s, Vh, tile[s * NC + c]);
    }
}

template <int NC, class St>
__global__ void __launch_bounds__(256) k_soa_to_aos(const void *__restrict__ soa, double2 *__restrict__ aos,
                                                    int Vh, size_t block_bytes)
{
    __shared__ double2 tile[kTile * NC];
    const int b = blockIdx.y;
    const int s0 = blockIdx.x * kTile;
    const int ns = min(kTile, Vh - s0);
    const void *src = (const char *)soa + b * block_bytes;
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        tile[s * NC + c] = St::load(src, c, s0 + s, Vh);
    }
    __syncthreads();
    double2 *dst = aos + ((size_t)b * Vh + s0) * NC;
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) dst[i] = tile[i];
}

// one parity block, sites [s_lo, s_hi): AoS (12 per site, starting at site s_lo) <-> SoA planes
__global__ void __launch_bounds__(256) k_range_aos_to_soa(const double2 *__restrict__ aos, double2 *__restrict__ soa,
                                                          int Vh, int s_lo, int s_hi)
{
    __shared__ double2 tile[kTile * 12];
    const int s0 = s_lo + blockIdx.x * kTile;
    const int ns = min(kTile, s_hi - s0);
    const double2 *src = aos + (size_t)(s0 - s_lo) * 12;
    for (int i = threadIdx.x; i < ns * 12; i += blockDim.x) tile[i] = src[i];
    __syncthreads();
    for (int i = threadIdx.x; i < ns * 12; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        soa[(size_t)c * Vh + s0 + s] = tile[s * 12 + c];
    }
}

__global__ void __launch_bounds__(256) k_range_soa_to_aos(const double2 *__restrict__ soa, double2 *__restrict__ aos,
                                                          int Vh, int s_lo, int s_hi)
{
    __shared__ double2 tile[kTile * 12];
    const int s0 = s_lo + blockIdx.x * kTile;
    const int ns = min(kTile, s_hi - s0);
    for (int i = threadIdx.x; i < ns * 12; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        tile[s * 12 + c] = soa[(size_t)c * Vh + s0 + s];
    }
    __syncthreads();
    double2 *dst = aos + (size_t)(s0 - s_lo) * 12;
    for (int i = threadIdx.x; i < ns * 12; i += blockDim.x) dst[i] = tile[i];
}

// ------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-reduce (a, b) and write one partial per block.
__device__ __forceinline__ void block_partial(double a, double b, double2 *partial)
{
    __shared__ double sa[WD_RED_THREADS / 32], sb[WD_RED_THREADS / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = l < WD_RED_THREADS / 32 ? sa[l] : 0.0;
        b = l < WD_RED_THREADS / 32 ? sb[l] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        if (l == 0) partial[blockIdx.x] = make_double2(a, b);
    }
}

#define GRID_STRIDE(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void __launch_bounds__(WD_RED_THREADS) k_norm2(const double2 *__restrict__ a, int64_t n, double2 *partial)
{
    double s = 0.0;
    GRID_STRIDE(i, n)
    {
        const double2 v = a[i];
        s = fma(v.x, v.x, s);
        s = fma(v.y, v.y, s);
    }
    block_partial(s, 0.0, partial);
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_dot(const double2 *__restrict__ a, const double2 *__restrict__ b,
                                                        int64_t n, double2 *partial)
{
    double re = 0.0, im = 0.0;
    GRID_STRIDE(i, n)
    {
        const double2 u = a[i], v = b[i];
        re = fma(u.x, v.x, re);
        re = fma(u.y, v.y, re);
        im = fma(u.x, v.y, im);
        im = fma(-u.y, v.x, im);
    }
    block_partial(re, im, partial);
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_norm2_df(const float4 *__restrict__ a, int64_t n, double2 *partial)
{
    dfr s{0.f, 0.f};
    GRID_STRIDE(i, n)
    {
        const dfc v = df_from_f4(a[i]);
        s = df_madd(df_madd(s, v.re, v.re), v.im, v.im);
    }
    block_partial(df_value(s), 0.0, partial);
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_dot_df(const float4 *__restrict__ a, const float4 *__restrict__ b,
                                                           int64_t n, double2 *partial)
{
    dfc s = c_zero(dfc());
    GRID_STRIDE(i, n) { s = c_maddc(s, df_from_f4(a[i]), df_from_f4(b[i])); }
    block_partial(df_value(s.re), df_value(s.im), partial);
}

// One block of 1024 threads folds WD_RED_BLOCKS partials into *result.
__global__ void __launch_bounds__(1024) k_red_finish(const double2 *__restrict__ partial, int nparts, double2 *result)
{
    __shared__ double sa[32], sb[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        a += partial[i].x;
        b += partial[i].y;
    }
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = l < (int)(blockDim.x >> 5) ? sa[l] : 0.0;
        b = l < (int)(blockDim.x >> 5) ? sb[l] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        if (l == 0) *result = make_double2(a, b);
    }
}

// ------------------------------------------------------------ FP64 BLAS
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

__global__ void k_axpby(double2 a, const double2 *__restrict__ x, double2 b, double2 *__restrict__ y, int64_t n)
{
    GRID_STRIDE(i, n)
    {
        const double2 u = cmul(a, x[i]), v = cmul(b, y[i]);
        y[i] = make_double2(u.x + v.x, u.y + v.y);
    }
}

// z may alias y (element-wise read before write)
__global__ void k_xpayz(const double2 *__restrict__ x, double2 a, const double2 *y, double2 *z, int64_t n)
{
    GRID_STRIDE(i, n)
    {
        const double2 u = x[i], v = y[i];
        z[i] = make_double2(u.x + fma(a.x, v.x, -a.y * v.y), u.y + fma(a.x, v.y, a.y * v.x));
    }
}

__global__ void k_scale(double a, const double2 *__restrict__ x, double2 *__restrict__ y, int64_t n)
{
    GRID_STRIDE(i, n)
    {
        const double2 u = x[i];
        y[i] = make_double2(a * u.x, a * u.y);
    }
}

// x += alpha p; r -= alpha q; partial |r|^2  (src/invert.cpp:89-107 fused)
__global__ void __launch_bounds__(WD_RED_THREADS) k_cg_update(double2 alpha, const double2 *__restrict__ p,
                                                              const double2 *__restrict__ q, double2 *__restrict__ x,
                                                              double2 *__restrict__ r, int64_t n, double2 *partial)
{
    double s = 0.0;
    GRID_STRIDE(i, n)
    {
        const double2 pv = p[i], qv = q[i];
        double2 xv = x[i], rv = r[i];
        const double2 ap = cmul(alpha, pv), aq = cmul(alpha, qv);
        xv.x += ap.x;
        xv.y += ap.y;
        rv.x -= aq.x;
        rv.y -= aq.y;
        x[i] = xv;
        r[i] = rv;
        s = fma(rv.x, rv.x, s);
        s = fma(rv.y, rv.y, s);
    }
    block_partial(s, 0.0, partial);
}

// Real-scalar forms for the even-odd CG, whose alpha and beta are real
// (ratios of norms): one FMA per real instead of a complex product.
// y = x + b y
__global__ void k_xpby_real(const double2 *__restrict__ x, double b, double2 *__restrict__ y, int64_t n)
{
    GRID_STRIDE(i, n)
    {
        const double2 u = x[i], v = y[i];
        y[i] = make_double2(fma(b, v.x, u.x), fma(b, v.y, u.y));
    }
}

// x += alpha p; r -= alpha q; partial |r|^2
__global__ void __launch_bounds__(WD_RED_THREADS) k_cg_update_real(double alpha, const double2 *__restrict__ p,
                                                                   const double2 *__restrict__ q,
                                                                   double2 *__restrict__ x, double2 *__restrict__ r,
                                                                   int64_t n, double2 *partial)
{
    double s = 0.0;
    GRID_STRIDE(i, n)
    {
        const double2 pv = p[i], qv = q[i];
        double2 xv = x[i], rv = r[i];
        xv = make_double2(fma(alpha, pv.x, xv.x), fma(alpha, pv.y, xv.y));
        rv = make_double2(fma(-alpha, qv.x, rv.x), fma(-alpha, qv.y, rv.y));
        x[i] = xv;
        r[i] = rv;
        s = fma(rv.x, rv.x, s);
        s = fma(rv.y, rv.y, s);
    }
    block_partial(s, 0.0, partial);
}

// ----------------------------------------------------- double-float BLAS
__host__ __device__ __forceinline__ dfc dfc_split(double2 a) { return dfc{df_split(a.x), df_split(a.y)}; }

__global__ void k_axpby_df(dfc a, const float4 *__restrict__ x, dfc b, float4 *__restrict__ y, int64_t n)
{
    GRID_STRIDE(i, n) { y[i] = df_to_f4(c_madd(c_mul(a, df_from_f4(x[i])), b, df_from_f4(y[i]))); }
}

__global__ void k_xpayz_df(const float4 *__restrict__ x, dfc a, const float4 *y, float4 *z, int64_t n)
{
    GRID_STRIDE(i, n) { z[i] = df_to_f4(c_madd(df_from_f4(x[i]), a, df_from_f4(y[i]))); }
}

__global__ void k_xpby_real_df(const float4 *__restrict__ x, dfr b, float4 *__restrict__ y, int64_t n)
{
    GRID_STRIDE(i, n)
    {
        const dfc u = df_from_f4(x[i]), v = df_from_f4(y[i]);
        y[i] = df_to_f4(dfc{df_madd(u.re, b, v.re), df_madd(u.im, b, v.im)});
    }
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_cg_update_real_df(dfr alpha, dfr malpha,
                                                                      const float4 *__restrict__ p,
                                                                      const float4 *__restrict__ q,
                                                                      float4 *__restrict__ x, float4 *__restrict__ r,
                                                                      int64_t n, double2 *partial)
{
    dfr s{0.f, 0.f};
    GRID_STRIDE(i, n)
    {
        const dfc pv = df_from_f4(p[i]), qv = df_from_f4(q[i]);
        dfc xv = df_from_f4(x[i]), rv = df_from_f4(r[i]);
        xv = dfc{df_madd(xv.re, alpha, pv.re), df_madd(xv.im, alpha, pv.im)};
        rv = dfc{df_madd(rv.re, malpha, qv.re), df_madd(rv.im, malpha, qv.im)};
        x[i] = df_to_f4(xv);
        r[i] = df_to_f4(rv);
        s = df_madd(df_madd(s, rv.re, rv.re), rv.im, rv.im);
    }
    block_partial(df_value(s), 0.0, partial);
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_cg_update_df(dfc alpha, dfc malpha, const float4 *__restrict__ p,
                                                                 const float4 *__restrict__ q, float4 *__restrict__ x,
                                                                 float4 *__restrict__ r, int64_t n, double2 *partial)
{
    dfr s{0.f, 0.f};
    GRID_STRIDE(i, n)
    {
        const dfc xv = c_madd(df_from_f4(x[i]), alpha, df_from_f4(p[i]));
        const dfc rv = c_madd(df_from_f4(r[i]), malpha, df_from_f4(q[i]));
        x[i] = df_to_f4(xv);
        r[i] = df_to_f4(rv);
        s = df_madd(df_madd(s, rv.re, rv.re), rv.im, rv.im);
    }
    block_partial(df_value(s), 0.0, partial);
}

inline int blas_blocks(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

// ------------------------------------------------------------- layout
template <int NC>
static wd_status to_soa(wd_context *ctx, const WdGeom &g, const double2 *ref, void *soa, wd_precision prec)
{
    dim3 grid((g.Vh + kTile - 1) / kTile, 2);
    const size_t bb = (size_t)NC * g.Vh * wd_entry_bytes(prec);
    switch (prec) {
    case WD_PREC_F64: k_aos_to_soa<NC, StF64><<<grid, 256, 0, ctx->stream>>>(ref, soa, g.Vh, bb); break;
    case WD_PREC_DF64: k_aos_to_soa<NC, StDF><<<grid, 256, 0, ctx->stream>>>(ref, soa, g.Vh, bb); break;
    case WD_PREC_F32: k_aos_to_soa<NC, StF32><<<grid, 256, 0, ctx->stream>>>(ref, soa, g.Vh, bb); break;
    default: return wd_fail(ctx, WD_ERR_BAD_ARG, "no direct layout conversion for this storage");
    }
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_spinor_ref_to_soa(wd_context *ctx, const WdGeom &g, const double2 *ref, WdVec soa)
{
    return to_soa<12>(ctx, g, ref, soa.p, soa.prec);
}

wd_status wd_spinor_soa_to_ref(wd_context *ctx, const WdGeom &g, WdVec soa, double2 *ref)
{
    dim3 grid((g.Vh + kTile - 1) / kTile, 2);
    const size_t bb = (size_t)12 * g.Vh * wd_entry_bytes(soa.prec);
    switch (soa.prec) {
    case WD_PREC_F64: k_soa_to_aos<12, StF64><<<grid, 256, 0, ctx->stream>>>(soa.p, ref, g.Vh, bb); break;
    case WD_PREC_DF64: k_soa_to_aos<12, StDF><<<grid, 256, 0, ctx->stream>>>(soa.p, ref, g.Vh, bb); break;
    case WD_PREC_F32: k_soa_to_aos<12, StF32><<<grid, 256, 0, ctx->stream>>>(soa.p, ref, g.Vh, bb); break;
    default: return wd_fail(ctx, WD_ERR_BAD_ARG, "no direct layout conversion for this storage");
    }
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_gauge_ref_to_soa(wd_context *ctx, const WdGeom &g, int mu, const double2 *ref, double2 *soa)
{
    return to_soa<9>(ctx, g, ref, soa + (size_t)mu * 2 * 9 * g.Vh, WD_PREC_F64);
}

wd_status wd_range_aos_to_soa(wd_context *ctx, cudaStream_t stream, int Vh, const double2 *aos, double2 *soa_block,
                              int s_lo, int s_hi)
{
    if (s_hi <= s_lo) return WD_OK;
    k_range_aos_to_soa<<<(s_hi - s_lo + kTile - 1) / kTile, 256, 0, stream>>>(aos, soa_block, Vh, s_lo, s_hi);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_range_soa_to_aos(wd_context *ctx, cudaStream_t stream, int Vh, const double2 *soa_block, double2 *aos,
                              int s_lo, int s_hi)
{
    if (s_hi <= s_lo) return WD_OK;
    k_range_soa_to_aos<<<(s_hi - s_lo + kTile - 1) / kTile, 256, 0, stream>>>(soa_block, aos, Vh, s_lo, s_hi);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// n 16-byte entries from src to dst on `stream`, either side possibly host
// memory the device addresses directly.  76 blocks (half the SMs) keep the
// CPU-GPU link busy and leave the SMs to the concurrent arithmetic: the
// pageable host-buffer DslashoffdNew at 32^3x64 ran 2.72-2.80 ms per call
// with 19-114 blocks and 3.1-3.2 ms with 304-1216.
__global__ void k_copy16(const double2 *__restrict__ src, double2 *__restrict__ dst, int64_t n)
{
    GRID_STRIDE(i, n) { dst[i] = src[i]; }
}

wd_status wd_copy_kernel(wd_context *ctx, cudaStream_t stream, const double2 *src, double2 *dst, int64_t n)
{
    if (n <= 0) return WD_OK;
    const int64_t b = (n + 255) / 256;
    k_copy16<<<(int)(b < 76 ? b : 76), 256, 0, stream>>>(src, dst, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// ---------------------------------------------------------- reductions
wd_status wd_red_finish(wd_context *ctx, int slot)
{
    double2 *part = (double2 *)ctx->red_partial;
    k_red_finish<<<1, 1024, 0, ctx->stream>>>(part, WD_RED_BLOCKS, part + WD_RED_BLOCKS + slot);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_red_norm2(wd_context *ctx, const double2 *a, int64_t n, int slot)
{
    k_norm2<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(a, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_red_dot(wd_context *ctx, const double2 *a, const double2 *b, int64_t n, int slot)
{
    k_dot<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(a, b, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_red_fetch(wd_context *ctx, int nslots, double2 *host)
{
    double2 *part = (double2 *)ctx->red_partial;
    WD_CUDA(ctx, cudaMemcpyAsync(ctx->red_result, part + WD_RED_BLOCKS, sizeof(double2) * nslots,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    memcpy(host, ctx->red_result, sizeof(double2) * nslots);
    return WD_OK;
}

wd_status wd_blas_axpby(wd_context *ctx, double2 a, const double2 *x, double2 b, double2 *y, int64_t n)
{
    k_axpby<<<blas_blocks(n), 256, 0, ctx->stream>>>(a, x, b, y, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_blas_xpayz(wd_context *ctx, const double2 *x, double2 a, const double2 *y, double2 *z, int64_t n)
{
    k_xpayz<<<blas_blocks(n), 256, 0, ctx->stream>>>(x, a, y, z, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_blas_scale(wd_context *ctx, double a, const double2 *x, double2 *y, int64_t n)
{
    k_scale<<<blas_blocks(n), 256, 0, ctx->stream>>>(a, x, y, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_blas_cg_update(wd_context *ctx, double2 alpha, const double2 *p, const double2 *q, double2 *x,
                            double2 *r, int64_t n, int slot)
{
    k_cg_update<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(alpha, p, q, x, r, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

// ------------------------------------------- precision-dispatched BLAS
static wd_status same_prec(wd_context *ctx, std::initializer_list<WdVec> v)
{
    const wd_precision p = v.begin()->prec;
    for (const WdVec &x : v)
        if (x.prec != p) return wd_fail(ctx, WD_ERR_BAD_ARG, "mixed storage precisions in one BLAS call");
    if (p != WD_PREC_F64 && p != WD_PREC_DF64)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "BLAS-1 on this storage is not available");
    return WD_OK;
}

wd_status wd_v_norm2(wd_context *ctx, WdVec a, int64_t n, int slot)
{
    wd_status st = same_prec(ctx, {a});
    if (st != WD_OK) return st;
    if (a.prec == WD_PREC_F64) return wd_red_norm2(ctx, (const double2 *)a.p, n, slot);
    k_norm2_df<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>((const float4 *)a.p, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_v_dot(wd_context *ctx, WdVec a, WdVec b, int64_t n, int slot)
{
    wd_status st = same_prec(ctx, {a, b});
    if (st != WD_OK) return st;
    if (a.prec == WD_PREC_F64) return wd_red_dot(ctx, (const double2 *)a.p, (const double2 *)b.p, n, slot);
    k_dot_df<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>((const float4 *)a.p, (const float4 *)b.p, n,
                                                                (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_v_axpby(wd_context *ctx, double2 a, WdVec x, double2 b, WdVec y, int64_t n)
{
    wd_status st = same_prec(ctx, {x, y});
    if (st != WD_OK) return st;
    if (x.prec == WD_PREC_F64) return wd_blas_axpby(ctx, a, (const double2 *)x.p, b, (double2 *)y.p, n);
    k_axpby_df<<<blas_blocks(n), 256, 0, ctx->stream>>>(dfc_split(a), (const float4 *)x.p, dfc_split(b),
                                                        (float4 *)y.p, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_v_xpayz(wd_context *ctx, WdVec x, double2 a, WdVec y, WdVec z, int64_t n)
{
    wd_status st = same_prec(ctx, {x, y, z});
    if (st != WD_OK) return st;
    if (x.prec == WD_PREC_F64) return wd_blas_xpayz(ctx, (const double2 *)x.p, a, (const double2 *)y.p, (double2 *)z.p, n);
    k_xpayz_df<<<blas_blocks(n), 256, 0, ctx->stream>>>((const float4 *)x.p, dfc_split(a), (const float4 *)y.p,
                                                        (float4 *)z.p, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_v_cg_update(wd_context *ctx, double2 alpha, WdVec p, WdVec q, WdVec x, WdVec r, int64_t n, int slot)
{
    wd_status st = same_prec(ctx, {p, q, x, r});
    if (st != WD_OK) return st;
    if (p.prec == WD_PREC_F64)
        return wd_blas_cg_update(ctx, alpha, (const double2 *)p.p, (const double2 *)q.p, (double2 *)x.p,
                                 (double2 *)r.p, n, slot);
    k_cg_update_df<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(
        dfc_split(alpha), dfc_split(make_double2(-alpha.x, -alpha.y)), (const float4 *)p.p, (const float4 *)q.p,
        (float4 *)x.p, (float4 *)r.p, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_v_xpby(wd_context *ctx, WdVec x, double b, WdVec y, int64_t n)
{
    wd_status st = same_prec(ctx, {x, y});
    if (st != WD_OK) return st;
    if (x.prec == WD_PREC_F64)
        k_xpby_real<<<blas_blocks(n), 256, 0, ctx->stream>>>((const double2 *)x.p, b, (double2 *)y.p, n);
    else
        k_xpby_real_df<<<blas_blocks(n), 256, 0, ctx->stream>>>((const float4 *)x.p, df_split(b), (float4 *)y.p, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_v_cg_update_real(wd_context *ctx, double alpha, WdVec p, WdVec q, WdVec x, WdVec r, int64_t n, int slot)
{
    wd_status st = same_prec(ctx, {p, q, x, r});
    if (st != WD_OK) return st;
    double2 *part = (double2 *)ctx->red_partial;
    if (p.prec == WD_PREC_F64)
        k_cg_update_real<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(
            alpha, (const double2 *)p.p, (const double2 *)q.p, (double2 *)x.p, (double2 *)r.p, n, part);
    else
        k_cg_update_real_df<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(
            df_split(alpha), df_split(-alpha), (const float4 *)p.p, (const float4 *)q.p, (float4 *)x.p,
            (float4 *)r.p, n, part);
    WD_LAUNCHED(ctx);
    return wd_red_finish(ctx, slot);
}

wd_status wd_v_copy(wd_context *ctx, WdVec dst, WdVec src, int64_t n)
{
    if (dst.prec != src.prec) return wd_fail(ctx, WD_ERR_BAD_ARG, "copy between different storages");
    WD_CUDA(ctx, cudaMemcpyAsync(dst.p, src.p, n * wd_entry_bytes(src.prec), cudaMemcpyDeviceToDevice, ctx->stream));
    if (src.scale && dst.scale)
        WD_CUDA(ctx, cudaMemcpyAsync(dst.scale, src.scale, n / 12 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    return WD_OK;
}

wd_status wd_v_zero(wd_context *ctx, WdVec v, int64_t n)
{
    WD_CUDA(ctx, cudaMemsetAsync(v.p, 0, n * wd_entry_bytes(v.prec), ctx->stream));
    if (v.scale) WD_CUDA(ctx, cudaMemsetAsync(v.scale, 0, n / 12 * sizeof(float), ctx->stream));
    return WD_OK;
}
