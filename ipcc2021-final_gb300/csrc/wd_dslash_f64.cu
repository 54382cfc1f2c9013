// wd_dslash_f64.cu -- native FP64 hopping kernel (the plain drop-in arithmetic).
//
// Storage: double2 planes, spinor [12][Vh] per parity, links [mu][parity][9][Vh].
// Algorithmic traffic per output site: 8 links x 144 B + 1 spinor in x 192 B
// + 1 spinor out x 192 B = 1536 B (+192 B when the epilogue reads x).
// Arithmetic: 1320 flop per site.  On GB300 the FP64 pipe (~1.2 TFLOP/s
// measured) rather than HBM bounds this kernel; wd_dslash_df.cu holds the
// double-float variant that moves the arithmetic onto the FP32 pipe.
#include "wd_hop.cuh"
#include "wd_kernels.h"
#include <type_traits>
#include "wd_tune.h"

namespace {

template <int THREADS>
struct HopF64 {
    using C = double2;
    static constexpr int kThreads = THREADS;
    WdGeom g;
    int cb;
    const double2 *__restrict__ in;     // parity 1-cb block [12][Vh]
    const double2 *__restrict__ gauge;  // [4][2][9][Vh]
    const double2 *__restrict__ x;      // parity cb block or null
    double2 *__restrict__ out;          // parity cb block
    double alpha, beta;

    __device__ __forceinline__ void load_in(int s, C *v) const
    {
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = in[(size_t)c * g.Vh + s];
    }
    __device__ __forceinline__ void load_link(int mu, int par, int s, C *U) const
    {
        const double2 *b = gauge + (size_t)((mu * 2 + par) * 9) * g.Vh + s;
#pragma unroll
        for (int k = 0; k < 9; ++k) U[k] = b[(size_t)k * g.Vh];
    }
    __device__ __forceinline__ void epilogue(int s, const C *acc) const
    {
        if (x) {
#pragma unroll
            for (int c = 0; c < 12; ++c)
                out[(size_t)c * g.Vh + s] = c_axpby(alpha, acc[c], beta, x[(size_t)c * g.Vh + s]);
        } else {
#pragma unroll
            for (int c = 0; c < 12; ++c) out[(size_t)c * g.Vh + s] = c_scale(acc[c], alpha);
        }
    }
};

// The same kernel on the reference's own site-major layout (AoS: the 12
// complex components of a site contiguous, [site][spin*3+colour]) for the
// input and output parity blocks; the links stay in the SoA planes.  A warp's
// 32 neighbour sites are 6 KB of consecutive bytes, so every fetched line is
// used, and the FP64 pipe (not the access pattern) still bounds the kernel.
// The host-buffer path runs it on the staging buffers directly, with no
// layout conversion between the copies and the arithmetic.
template <int THREADS>
struct HopF64AoS : HopF64<THREADS> {
    __device__ __forceinline__ void load_in(int s, double2 *v) const
    {
        const double2 *b = this->in + (size_t)s * 12;
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = b[c];
    }
    __device__ __forceinline__ void epilogue(int s, const double2 *acc) const
    {
        double2 *o = this->out + (size_t)s * 12;
#pragma unroll
        for (int c = 0; c < 12; ++c) o[c] = c_scale(acc[c], this->alpha);
    }
};

}  // namespace

wd_status wd_hop_f64_aos_range(wd_context *ctx, cudaStream_t stream, const wd_lattice *lat, const double2 *in_aos,
                               double2 *out_aos, int cb, int dag, double alpha, int s_lo, int s_hi)
{
    using P = HopF64AoS<64>;
    P p;
    p.g = lat->g;
    p.cb = cb;
    p.in = in_aos;
    p.gauge = lat->gauge;
    p.x = nullptr;
    p.out = out_aos;
    p.alpha = alpha;
    p.beta = 0.0;
    const int n = s_hi - s_lo;
    if (n <= 0) return WD_OK;
    const int blocks = (n + P::kThreads - 1) / P::kThreads;
    if (dag) wd_hop_kernel_range<true><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    else wd_hop_kernel_range<false><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_hop_f64(wd_context *ctx, const wd_lattice *lat, const double2 *in_block,
                     double2 *out_block, const double2 *x_block, int cb, int dag, double alpha,
                     double beta)
{
    auto run = [&](auto tag) -> wd_status {
        using P = HopF64<decltype(tag)::value>;
        P p;
        p.g = lat->g;
        p.cb = cb;
        p.in = in_block;
        p.gauge = lat->gauge;
        p.x = x_block;
        p.out = out_block;
        p.alpha = alpha;
        p.beta = beta;
        const int blocks = (lat->g.Vh + P::kThreads - 1) / P::kThreads;
        if (dag) wd_hop_kernel<true><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
        else wd_hop_kernel<false><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    // variants: 128, 64, 256 threads per block
    return wd_tune_launch(ctx, "hop_f64", lat->g.Vh, 3, [&](int v) -> wd_status {
        if (v == 1) return run(std::integral_constant<int, 64>());
        if (v == 2) return run(std::integral_constant<int, 256>());
        return run(std::integral_constant<int, 128>());
    });
}

wd_status wd_hop_f64_range(wd_context *ctx, cudaStream_t stream, const wd_lattice *lat, const double2 *in_block,
                           double2 *out_block, int cb, int dag, double alpha, int s_lo, int s_hi)
{
    using P = HopF64<64>;
    P p;
    p.g = lat->g;
    p.cb = cb;
    p.in = in_block;
    p.gauge = lat->gauge;
    p.x = nullptr;
    p.out = out_block;
    p.alpha = alpha;
    p.beta = 0.0;
    const int n = s_hi - s_lo;
    if (n <= 0) return WD_OK;
    const int blocks = (n + P::kThreads - 1) / P::kThreads;
    if (dag) wd_hop_kernel_range<true><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    else wd_hop_kernel_range<false><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    WD_LAUNCHED(ctx);
    return WD_OK;
}
