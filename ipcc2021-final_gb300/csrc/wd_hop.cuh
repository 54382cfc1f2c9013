// wd_hop.cuh -- the Wilson hopping term, written once for every arithmetic
// type.  One thread computes one output site of parity cb:
//
//   acc = sum_mu [ (1 - s g_mu) U_mu(x) psi(x+mu) + (1 + s g_mu) U_mu(x-mu)^dag psi(x-mu) ]
//   out = alpha * acc + beta * x            (x: same-parity field, optional)
//
// s = +1 for D, -1 for D^dag.  The reference's -1/2 (src/dslash.cpp:544-873)
// is alpha = -0.5; the diagonal (4+m) term of DslashNew is beta.  Neighbours
// wrap periodically inside the kernel, replacing the reference's halo
// exchange (src/dslash_new.cpp:1416-1826, 2304-2654).
//
// A policy class P supplies the storage format: the complex arithmetic type
// P::C, loads of a neighbour spinor and of a link matrix, and the epilogue.
//
// A storage with a per-site scale (FP16) may instead expose
// `static constexpr bool kSiteScale = true` and `float load_in_raw(int, C*)`,
// returning the unscaled components and the site's scale: the scale then
// rides on the accumulation (one FMA per real) instead of multiplying the 24
// loaded reals.
#pragma once
#include <type_traits>
#include "wd_internal.cuh"
#include "wd_complex.cuh"

template <class P, class = void>
struct wd_site_scaled : std::false_type {};
template <class P>
struct wd_site_scaled<P, std::void_t<decltype(P::kSiteScale)>> : std::bool_constant<P::kSiteScale> {};

template <int SG, class C>
__device__ __forceinline__ C wd_addsg(const C &a, const C &b)
{
    if constexpr (SG > 0) return c_add(a, b);
    else return c_sub(a, b);
}

// Spin projection of one colour: (s0, s1, s2, s3) -> (h0, h1) for direction
// MU and sign SG (the table in wd_internal.cuh).
template <int MU, int SG, class C>
__device__ __forceinline__ void wd_proj1(const C &s0, const C &s1, const C &s2, const C &s3, C &h0, C &h1)
{
    if constexpr (MU == 0) {
        h0 = wd_addsg<SG>(s0, c_i(s3));
        h1 = wd_addsg<SG>(s1, c_i(s2));
    } else if constexpr (MU == 1) {
        h0 = wd_addsg<-SG>(s0, s3);
        h1 = wd_addsg<SG>(s1, s2);
    } else if constexpr (MU == 2) {
        h0 = wd_addsg<SG>(s0, c_i(s2));
        h1 = wd_addsg<-SG>(s1, c_i(s3));
    } else {
        h0 = wd_addsg<SG>(s0, s2);
        h1 = wd_addsg<SG>(s1, s3);
    }
}

// Accumulate (t0, t1) = W (h0, h1) of one colour into its four spin components d[0..3].
template <int MU, int SG, class C>
__device__ __forceinline__ void wd_recon1(const C &t0, const C &t1, C &d0, C &d1, C &d2, C &d3)
{
    d0 = c_add(d0, t0);
    d1 = c_add(d1, t1);
    if constexpr (MU == 0) {
        d2 = wd_addsg<-SG>(d2, c_i(t1));
        d3 = wd_addsg<-SG>(d3, c_i(t0));
    } else if constexpr (MU == 1) {
        d2 = wd_addsg<SG>(d2, t1);
        d3 = wd_addsg<-SG>(d3, t0);
    } else if constexpr (MU == 2) {
        d2 = wd_addsg<-SG>(d2, c_i(t0));
        d3 = wd_addsg<SG>(d3, c_i(t1));
    } else {
        d2 = wd_addsg<SG>(d2, t0);
        d3 = wd_addsg<SG>(d3, t1);
    }
}

// wd_recon1 for the first direction, into zero accumulators: assignments
// instead of additions to zero (24 fewer adds per site; a result can differ
// only in the sign of a zero)
template <int X, class C>
__device__ __forceinline__ C wd_sgv(const C &v)
{
    if constexpr (X > 0) return v;
    else return c_neg(v);
}
template <int MU, int SG, class C>
__device__ __forceinline__ void wd_recon1_first(const C &t0, const C &t1, C &d0, C &d1, C &d2, C &d3)
{
    d0 = t0;
    d1 = t1;
    if constexpr (MU == 0) {
        d2 = wd_sgv<-SG>(c_i(t1));
        d3 = wd_sgv<-SG>(c_i(t0));
    } else if constexpr (MU == 1) {
        d2 = wd_sgv<SG>(t1);
        d3 = wd_sgv<-SG>(t0);
    } else if constexpr (MU == 2) {
        d2 = wd_sgv<-SG>(c_i(t0));
        d3 = wd_sgv<SG>(c_i(t1));
    } else {
        d2 = wd_sgv<SG>(t0);
        d3 = wd_sgv<SG>(t1);
    }
}

// d + k t and d + k (i t), k real (FP32 complex only)
__device__ __forceinline__ float2 wd_cfma(float k, float2 t, float2 d)
{
    return make_float2(fmaf(k, t.x, d.x), fmaf(k, t.y, d.y));
}
__device__ __forceinline__ float2 wd_cfma_i(float k, float2 t, float2 d)
{
    return make_float2(fmaf(-k, t.y, d.x), fmaf(k, t.x, d.y));
}

// wd_recon1 with the neighbour's scale k folded in: d += k * (the same terms)
template <int MU, int SG>
__device__ __forceinline__ void wd_recon1_scaled(float2 t0, float2 t1, float k, float2 &d0, float2 &d1, float2 &d2,
                                                 float2 &d3)
{
    d0 = wd_cfma(k, t0, d0);
    d1 = wd_cfma(k, t1, d1);
    if constexpr (MU == 0) {
        d2 = wd_cfma_i(-SG * k, t1, d2);
        d3 = wd_cfma_i(-SG * k, t0, d3);
    } else if constexpr (MU == 1) {
        d2 = wd_cfma(SG * k, t1, d2);
        d3 = wd_cfma(-SG * k, t0, d3);
    } else if constexpr (MU == 2) {
        d2 = wd_cfma_i(-SG * k, t0, d2);
        d3 = wd_cfma_i(SG * k, t1, d3);
    } else {
        d2 = wd_cfma(SG * k, t0, d2);
        d3 = wd_cfma(SG * k, t1, d3);
    }
}

// Whole-site forms: sp/acc hold 12 components, index spin*3 + colour.
template <int MU, int SG, class C>
__device__ __forceinline__ void wd_proj(const C *sp, C *h0, C *h1)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) wd_proj1<MU, SG>(sp[k], sp[3 + k], sp[6 + k], sp[9 + k], h0[k], h1[k]);
}

template <int MU, int SG, class C>
__device__ __forceinline__ void wd_recon(const C *t0, const C *t1, C *acc)
{
#pragma unroll
    for (int a = 0; a < 3; ++a) wd_recon1<MU, SG>(t0[a], t1[a], acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
}

// One of the eight neighbour terms (FIRST: the accumulators hold zeros).
template <int MU, bool FWD, bool DAG, class P, bool FIRST = false>
__device__ __forceinline__ void wd_hop_dir(const P &p, int s, const WdSite &c, typename P::C *acc)
{
    using C = typename P::C;
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    constexpr bool kScaled = wd_site_scaled<P>::value;
    const int nb = wd_neighbour(p.g, s, c, MU, FWD);
    C sp[12];
    float sc = 1.f;
    if constexpr (kScaled) sc = p.load_in_raw(nb, sp);
    else p.load_in(nb, sp);
    C h0[3], h1[3];
    wd_proj<MU, SG>(sp, h0, h1);
    C U[9];
    // forward: U_mu(x) stored at this site (parity cb);
    // backward: U_mu(x - mu) stored at the neighbour (parity 1-cb)
    if constexpr (FWD) p.load_link(MU, p.cb, s, U);
    else p.load_link(MU, 1 - p.cb, nb, U);
    C t0[3], t1[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if constexpr (FWD) {
            t0[a] = c_mul(U[a * 3 + 0], h0[0]);
            t1[a] = c_mul(U[a * 3 + 0], h1[0]);
#pragma unroll
            for (int b = 1; b < 3; ++b) {
                t0[a] = c_madd(t0[a], U[a * 3 + b], h0[b]);
                t1[a] = c_madd(t1[a], U[a * 3 + b], h1[b]);
            }
        } else {
            t0[a] = c_mulc(U[a], h0[0]);
            t1[a] = c_mulc(U[a], h1[0]);
#pragma unroll
            for (int b = 1; b < 3; ++b) {
                t0[a] = c_maddc(t0[a], U[b * 3 + a], h0[b]);
                t1[a] = c_maddc(t1[a], U[b * 3 + a], h1[b]);
            }
        }
    }
    if constexpr (kScaled) {
#pragma unroll
        for (int a = 0; a < 3; ++a) wd_recon1_scaled<MU, SG>(t0[a], t1[a], sc, acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
    } else if constexpr (FIRST) {
#pragma unroll
        for (int a = 0; a < 3; ++a) wd_recon1_first<MU, SG>(t0[a], t1[a], acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
    } else {
        wd_recon<MU, SG>(t0, t1, acc);
    }
}

template <bool DAG, class P>
__device__ __forceinline__ void wd_hop_site(const P &p, int s, typename P::C *acc)
{
    using C = typename P::C;
    const WdSite c = wd_site(p.g, s, p.cb);
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = c_zero(C());
    wd_hop_dir<0, true, DAG, P, true>(p, s, c, acc);
    wd_hop_dir<0, false, DAG>(p, s, c, acc);
    wd_hop_dir<1, true, DAG>(p, s, c, acc);
    wd_hop_dir<1, false, DAG>(p, s, c, acc);
    wd_hop_dir<2, true, DAG>(p, s, c, acc);
    wd_hop_dir<2, false, DAG>(p, s, c, acc);
    wd_hop_dir<3, true, DAG>(p, s, c, acc);
    wd_hop_dir<3, false, DAG>(p, s, c, acc);
}

template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads) wd_hop_kernel(const P p)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.g.Vh) return;
    typename P::C acc[12];
    wd_hop_site<DAG>(p, s, acc);
    p.epilogue(s, acc);
}

// The same over output sites [s_lo, s_hi) only (pipelined host-buffer path).
template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads) wd_hop_kernel_range(const P p, int s_lo, int s_hi)
{
    const int s = s_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s_hi) return;
    typename P::C acc[12];
    wd_hop_site<DAG>(p, s, acc);
    p.epilogue(s, acc);
}
