// wd_dslash_df.cu -- double-float (df64) hopping kernel.
//
// Same algorithm and memory traffic as the FP64 kernel (1536 B per output
// site: every complex number is a 16-byte float4 {re.h, re.l, im.h, im.l}),
// with the arithmetic moved from the FP64 pipe to the FP32 pipe
// (wd_df.cuh): ~8.5k FP32 operations per site instead of ~890 FP64 ones.
// Results agree with FP64 to ~1e-14 relative L2 (storage rounding 2^-49,
// arithmetic ~2^-48 per operation).
#include "wd_hop.cuh"
#include "wd_df.cuh"
#include "wd_kernels.h"

namespace {

struct HopDF {
    using C = dfc;
    static constexpr int kThreads = 128;
    WdGeom g;
    int cb;
    const float4 *__restrict__ in;     // parity 1-cb block [12][Vh]
    const float4 *__restrict__ gauge;  // [4][2][9][Vh]
    const float4 *__restrict__ x;      // parity cb block or null
    float4 *__restrict__ out;          // parity cb block
    dfr alpha, beta;

    __device__ __forceinline__ void load_in(int s, C *v) const
    {
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = df_from_f4(in[(size_t)c * g.Vh + s]);
    }
    __device__ __forceinline__ void load_link(int mu, int par, int s, C *U) const
    {
        const float4 *b = gauge + (size_t)((mu * 2 + par) * 9) * g.Vh + s;
#pragma unroll
        for (int k = 0; k < 9; ++k) U[k] = df_from_f4(b[(size_t)k * g.Vh]);
    }
    __device__ __forceinline__ void epilogue(int s, const C *acc) const
    {
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            dfc r{df_mul(alpha, acc[c].re), df_mul(alpha, acc[c].im)};
            if (x) {
                const dfc v = df_from_f4(x[(size_t)c * g.Vh + s]);
                r.re = df_madd(r.re, beta, v.re);
                r.im = df_madd(r.im, beta, v.im);
            }
            out[(size_t)c * g.Vh + s] = df_to_f4(r);
        }
    }
};

__global__ void k_f64_to_df(const double2 *__restrict__ in, float4 *__restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = df_pack(in[i]);
}

__global__ void k_df_to_f64(const float4 *__restrict__ in, double2 *__restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = df_unpack(in[i]);
}

int conv_blocks(int64_t n)
{
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

}  // namespace

wd_status wd_hop_df(wd_context *ctx, const wd_lattice *lat, const float4 *in_block, float4 *out_block,
                    const float4 *x_block, int cb, int dag, double alpha, double beta)
{
    wd_status st = wd_lattice_gauge_df(ctx, lat);
    if (st != WD_OK) return st;
    HopDF p;
    p.g = lat->g;
    p.cb = cb;
    p.in = in_block;
    p.gauge = lat->gauge_df;
    p.x = x_block;
    p.out = out_block;
    p.alpha = df_split(alpha);
    p.beta = df_split(beta);
    const int threads = HopDF::kThreads;
    const int blocks = (lat->g.Vh + threads - 1) / threads;
    if (dag) wd_hop_kernel<true><<<blocks, threads, 0, ctx->stream>>>(p);
    else wd_hop_kernel<false><<<blocks, threads, 0, ctx->stream>>>(p);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_convert_f64_to_df(wd_context *ctx, const double2 *in, float4 *out, int64_t n)
{
    k_f64_to_df<<<conv_blocks(n), 256, 0, ctx->stream>>>(in, out, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_convert_df_to_f64(wd_context *ctx, const float4 *in, double2 *out, int64_t n)
{
    k_df_to_f64<<<conv_blocks(n), 256, 0, ctx->stream>>>(in, out, n);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// df copy of the resident links, built on first use (wd_lattice_invalidate_derived drops it).
wd_status wd_lattice_gauge_df(wd_context *ctx, const wd_lattice *lat_c)
{
    wd_lattice *lat = const_cast<wd_lattice *>(lat_c);
    if (lat->gauge_df) return WD_OK;
    const int64_t n = lat->volume * 4 * 9;
    WD_CUDA(ctx, cudaMalloc(&lat->gauge_df, n * sizeof(float4)));
    return wd_convert_f64_to_df(ctx, lat->gauge, lat->gauge_df, n);
}
