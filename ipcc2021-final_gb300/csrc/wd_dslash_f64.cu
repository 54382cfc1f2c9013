// wd_dslash_f64.cu -- native FP64 hopping kernel (the plain drop-in arithmetic).
//
// Storage: double2 planes, spinor [12][Vh] per parity, links [mu][parity][9][Vh].
// Algorithmic traffic per output site: 8 links x 144 B + 1 spinor in x 192 B
// + 1 spinor out x 192 B = 1536 B (+192 B when the epilogue reads x).
// Arithmetic: 1320 flop per site.  On GB300 the FP64 pipe (~1.2 TFLOP/s
// measured) rather than HBM bounds this kernel, so it is written for the
// fewest FP64 operations (~790 per site): direction pairs combined
// (wd_hop_mu), the first direction assigned, and a power-of-two output scale
// applied on the exponent bits (F64Scale).  wd_dslash_df.cu holds the
// double-float variant that moves the arithmetic onto the FP32 pipe.
#include <cmath>
#include <cstdint>
#include "wd_hop.cuh"
#include "wd_kernels.h"
#include "wd_reduce.cuh"
#include <type_traits>
#include "wd_tune.h"

namespace {

// Output scaling without the FP64 pipe when alpha is 1 or a power of two
// (DslashoffdNew's -1/2, the Schur operator's first hop's 1): a power-of-two
// factor only moves the exponent, so integer arithmetic on the bits gives
// the FP64 product exactly; zeros, subnormal results and non-finite values
// take the FP64 multiply.  24 fewer FP64 operations per site (of ~890).
struct F64Scale {
    double alpha;
    int mode;       // 0: multiply, 1: identity, 2: exponent shift
    int shift;      // mode 2: alpha = sign * 2^shift
    uint64_t sign;  // mode 2: sign bit of alpha

    static F64Scale make(double a)
    {
        F64Scale f{a, 0, 0, 0};
        int e = 0;
        const double m = std::frexp(a, &e);  // a = m * 2^e, |m| in [0.5, 1)
        if (a == 1.0) f.mode = 1;
        else if (std::fabs(m) == 0.5 && e - 1 > -1000 && e - 1 < 1000) {
            f.mode = 2;
            f.shift = e - 1;
            f.sign = a < 0 ? 0x8000000000000000ull : 0ull;
        }
        return f;
    }
    __device__ __forceinline__ double apply(double v) const
    {
        if (mode == 1) return v;
        if (mode == 2) {
            const uint64_t b = (uint64_t)__double_as_longlong(v);
            const int ex = (int)((b >> 52) & 0x7ff);
            if (ex > 0 && ex < 0x7ff && ex + shift > 0 && ex + shift < 0x7ff)
                return __longlong_as_double((long long)((b + ((uint64_t)(int64_t)shift << 52)) ^ sign));
        }
        return v * alpha;
    }
    __device__ __forceinline__ double2 apply(double2 v) const { return make_double2(apply(v.x), apply(v.y)); }
};

template <int THREADS>
struct HopF64 {
    using C = double2;
    static constexpr int kThreads = THREADS;
    static constexpr bool kPairDirs = true;  // FP64-pipe bound: fewest operations wins
    WdGeom g;
    int cb;
    const double2 *__restrict__ in;     // parity 1-cb block [12][Vh]
    const double2 *__restrict__ gauge;  // [4][2][9][Vh]
    const double2 *__restrict__ x;      // parity cb block or null
    double2 *__restrict__ out;          // parity cb block
    double alpha, beta;
    F64Scale scale;                     // alpha, applied when there is no x

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
            for (int c = 0; c < 12; ++c) out[(size_t)c * g.Vh + s] = scale.apply(acc[c]);
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
        if (this->x) {  // site-major x block of the output parity
            const double2 *xv = this->x + (size_t)s * 12;
#pragma unroll
            for (int c = 0; c < 12; ++c) o[c] = c_axpby(this->alpha, acc[c], this->beta, xv[c]);
        } else {
#pragma unroll
            for (int c = 0; c < 12; ++c) o[c] = this->scale.apply(acc[c]);
        }
    }
};

// The reliable update's second Schur hop fused with the true residual:
// s = bhat - (alpha acc + beta x), rounded to FP32 into s32 (FP32 site
// layout: plane j holds components 2j, 2j+1), |s32|^2 reduced over the grid.
struct ResSink {
    const double2 *bhat;
    float4 *s32;
    double *partial;
    unsigned *counter;
    double *result;
};

template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads) k_hop_f64_res(const P p, const ResSink r)
{
    const int s = blockIdx.x * P::kThreads + threadIdx.x;
    float n = 0.f;
    if (s < p.g.Vh) {
        double2 acc[12];
        wd_hop_site<DAG>(p, s, acc);
        const size_t Vh = p.g.Vh;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            float v[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const size_t i = (size_t)(2 * j + h) * Vh + s;
                const double2 o = c_axpby(p.alpha, acc[2 * j + h], p.beta, p.x[i]);
                const double2 b = r.bhat[i];
                v[2 * h] = (float)(b.x - o.x);
                v[2 * h + 1] = (float)(b.y - o.y);
                n = fmaf(v[2 * h], v[2 * h], fmaf(v[2 * h + 1], v[2 * h + 1], n));
            }
            r.s32[(size_t)j * Vh + s] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
    double tot;
    if (wd_grid_sum<P::kThreads>((double)n, r.partial, r.counter, &tot)) *r.result = tot;
}

}  // namespace

wd_status wd_hop_df_residual(wd_context *ctx, const wd_lattice *lat, const float4 *in_block, const float4 *x_block,
                             const float4 *bhat, float4 *s32, double mass, double *partial, unsigned *counter,
                             double *result);

wd_status wd_hop_hi_residual(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec x, WdVec bhat, WdVec s32,
                             double mass, double *partial, unsigned *counter, double *result)
{
    if (in.prec != x.prec || in.prec != bhat.prec || s32.prec != WD_PREC_F32)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "residual hop: in, x, bhat of one storage, s32 FP32");
    const double a = 4.0 + mass;
    if (in.prec == WD_PREC_DF64)
        return wd_hop_df_residual(ctx, lat, (const float4 *)in.p, (const float4 *)x.p, (const float4 *)bhat.p,
                                  (float4 *)s32.p, mass, partial, counter, result);
    if (in.prec != WD_PREC_F64) return wd_fail(ctx, WD_ERR_BAD_ARG, "residual hop: FP64 or double-float storage");
    const ResSink r{(const double2 *)bhat.p, (float4 *)s32.p, partial, counter, result};
    auto run = [&](auto tag) -> wd_status {
        using P = HopF64<decltype(tag)::value>;
        P p;
        p.g = lat->g;
        p.cb = 0;
        p.in = (const double2 *)in.p;
        p.gauge = lat->gauge;
        p.x = (const double2 *)x.p;
        p.out = nullptr;
        p.alpha = -0.25 / a;
        p.beta = a;
        p.scale = F64Scale::make(p.alpha);
        const int blocks = (lat->g.Vh + P::kThreads - 1) / P::kThreads;
        k_hop_f64_res<false><<<blocks, P::kThreads, 0, ctx->stream>>>(p, r);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    // the plain FP64 hop's tuned shape: 128, 64 or 256 threads per block
    const int v = wd_tune_choice(ctx, "hop_f64", lat->g.Vh);
    if (v == 1) return run(std::integral_constant<int, 64>());
    if (v == 2) return run(std::integral_constant<int, 256>());
    return run(std::integral_constant<int, 128>());
}

wd_status wd_hop_f64_aos_range(wd_context *ctx, cudaStream_t stream, const wd_lattice *lat, const double2 *in_aos,
                               double2 *out_aos, const double2 *x_aos, int cb, int dag, double alpha, double beta,
                               int s_lo, int s_hi)
{
    using P = HopF64AoS<64>;
    P p;
    p.g = lat->g;
    p.cb = cb;
    p.in = in_aos;
    p.gauge = lat->gauge;
    p.x = x_aos;
    p.out = out_aos;
    p.alpha = alpha;
    p.beta = beta;
    p.scale = F64Scale::make(alpha);
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
        p.scale = F64Scale::make(alpha);
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
    p.scale = F64Scale::make(alpha);
    const int n = s_hi - s_lo;
    if (n <= 0) return WD_OK;
    const int blocks = (n + P::kThreads - 1) / P::kThreads;
    if (dag) wd_hop_kernel_range<true><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    else wd_hop_kernel_range<false><<<blocks, P::kThreads, 0, stream>>>(p, s_lo, s_hi);
    WD_LAUNCHED(ctx);
    return WD_OK;
}
