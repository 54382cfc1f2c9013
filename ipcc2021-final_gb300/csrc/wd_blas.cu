// wd_blas.cu -- layout conversion and FP64 BLAS-1 with deterministic reductions.
//
// Reductions (norm_2 / vector_p of include/operator_mpi.h:15-79) use a fixed
// grid of WD_RED_BLOCKS blocks: each block folds its grid-stride share with
// warp shuffles into one partial, and a single-block pass adds the partials
// in a fixed tree order.  The result is bitwise reproducible for a given
// length and lands in a device slot, so solvers can keep it on the device.
#include "wd_kernels.h"

namespace {

constexpr int kTile = 64;  // sites per transpose tile

template <int NC>
__global__ void __launch_bounds__(256) k_aos_to_soa(const double2 *__restrict__ aos,
                                                    double2 *__restrict__ soa, int Vh)
{
    __shared__ double2 tile[kTile * NC];
    const int b = blockIdx.y;
    const int s0 = blockIdx.x * kTile;
    const int ns = min(kTile, Vh - s0);
    const double2 *src = aos + ((size_t)b * Vh + s0) * NC;
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) tile[i] = src[i];
    __syncthreads();
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        soa[((size_t)b * NC + c) * Vh + s0 + s] = tile[s * NC + c];
    }
}

template <int NC>
__global__ void __launch_bounds__(256) k_soa_to_aos(const double2 *__restrict__ soa,
                                                    double2 *__restrict__ aos, int Vh)
{
    __shared__ double2 tile[kTile * NC];
    const int b = blockIdx.y;
    const int s0 = blockIdx.x * kTile;
    const int ns = min(kTile, Vh - s0);
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) {
        const int c = i / ns, s = i - c * ns;
        tile[s * NC + c] = soa[((size_t)b * NC + c) * Vh + s0 + s];
    }
    __syncthreads();
    double2 *dst = aos + ((size_t)b * Vh + s0) * NC;
    for (int i = threadIdx.x; i < ns * NC; i += blockDim.x) dst[i] = tile[i];
}

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

__global__ void __launch_bounds__(WD_RED_THREADS) k_norm2(const double2 *__restrict__ a, int64_t n,
                                                          double2 *partial)
{
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = a[i];
        s = fma(v.x, v.x, s);
        s = fma(v.y, v.y, s);
    }
    block_partial(s, 0.0, partial);
}

__global__ void __launch_bounds__(WD_RED_THREADS) k_dot(const double2 *__restrict__ a,
                                                        const double2 *__restrict__ b, int64_t n,
                                                        double2 *partial)
{
    double re = 0.0, im = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 u = a[i], v = b[i];
        re = fma(u.x, v.x, re);
        re = fma(u.y, v.y, re);
        im = fma(u.x, v.y, im);
        im = fma(-u.y, v.x, im);
    }
    block_partial(re, im, partial);
}

// One block of 1024 threads folds WD_RED_BLOCKS partials into result[0].
__global__ void __launch_bounds__(1024) k_red_finish(const double2 *__restrict__ partial, int nparts,
                                                     double2 *result)
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

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

__global__ void k_axpby(double2 a, const double2 *__restrict__ x, double2 b, double2 *__restrict__ y,
                        int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 u = cmul(a, x[i]), v = cmul(b, y[i]);
        y[i] = make_double2(u.x + v.x, u.y + v.y);
    }
}

__global__ void k_xpayz(const double2 *__restrict__ x, double2 a, const double2 *__restrict__ y,
                        double2 *__restrict__ z, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 u = x[i], v = y[i];
        z[i] = make_double2(u.x + fma(a.x, v.x, -a.y * v.y), u.y + fma(a.x, v.y, a.y * v.x));
    }
}

__global__ void k_scale(double a, const double2 *__restrict__ x, double2 *__restrict__ y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double2 u = x[i];
        y[i] = make_double2(a * u.x, a * u.y);
    }
}

// x += alpha p; r -= alpha q; partial |r|^2  (src/invert.cpp:89-107 fused)
__global__ void __launch_bounds__(WD_RED_THREADS) k_cg_update(double2 alpha,
                                                              const double2 *__restrict__ p,
                                                              const double2 *__restrict__ q,
                                                              double2 *__restrict__ x,
                                                              double2 *__restrict__ r, int64_t n,
                                                              double2 *partial)
{
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
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

inline int blas_blocks(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

wd_status wd_spinor_ref_to_soa(wd_context *ctx, const WdGeom &g, const double2 *ref, double2 *soa)
{
    dim3 grid((g.Vh + kTile - 1) / kTile, 2);
    k_aos_to_soa<12><<<grid, 256, 0, ctx->stream>>>(ref, soa, g.Vh);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_spinor_soa_to_ref(wd_context *ctx, const WdGeom &g, const double2 *soa, double2 *ref)
{
    dim3 grid((g.Vh + kTile - 1) / kTile, 2);
    k_soa_to_aos<12><<<grid, 256, 0, ctx->stream>>>(soa, ref, g.Vh);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_gauge_ref_to_soa(wd_context *ctx, const WdGeom &g, int mu, const double2 *ref,
                              double2 *soa)
{
    dim3 grid((g.Vh + kTile - 1) / kTile, 2);
    k_aos_to_soa<9><<<grid, 256, 0, ctx->stream>>>(ref, soa + (size_t)mu * 2 * 9 * g.Vh, g.Vh);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

static wd_status red_finish(wd_context *ctx, int slot)
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
    return red_finish(ctx, slot);
}

wd_status wd_red_dot(wd_context *ctx, const double2 *a, const double2 *b, int64_t n, int slot)
{
    k_dot<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(a, b, n, (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return red_finish(ctx, slot);
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

wd_status wd_blas_axpby(wd_context *ctx, double2 a, const double2 *x, double2 b, double2 *y,
                        int64_t n)
{
    k_axpby<<<blas_blocks(n), 256, 0, ctx->stream>>>(a, x, b, y, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_blas_xpayz(wd_context *ctx, const double2 *x, double2 a, const double2 *y,
                        double2 *z, int64_t n)
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

wd_status wd_blas_cg_update(wd_context *ctx, double2 alpha, const double2 *p, const double2 *q,
                            double2 *x, double2 *r, int64_t n, int slot)
{
    k_cg_update<<<WD_RED_BLOCKS, WD_RED_THREADS, 0, ctx->stream>>>(alpha, p, q, x, r, n,
                                                                   (double2 *)ctx->red_partial);
    WD_LAUNCHED(ctx);
    return red_finish(ctx, slot);
}
