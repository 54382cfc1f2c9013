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

// A policy whose arithmetic, not its memory traffic, bounds the kernel (FP64)
// sets `static constexpr bool kPairDirs = true` to take the direction-pair
// form below (fewer operations, more registers live across the loads).
template <class P, class = void>
struct wd_pair_dirs : std::false_type {};
template <class P>
struct wd_pair_dirs<P, std::void_t<decltype(P::kPairDirs)>> : std::bool_constant<P::kPairDirs> {};

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

// The terms of one of the eight neighbours from its spinor sp (site scale sc
// when SCALED) and link matrix U (FIRST: the accumulators hold zeros).
template <int MU, bool FWD, bool DAG, bool FIRST, bool SCALED, class C>
__device__ __forceinline__ void wd_dir_terms(const C *sp, float sc, const C *U, C *acc)
{
    constexpr int SG = (FWD ? -1 : 1) * (DAG ? -1 : 1);
    C h0[3], h1[3];
    wd_proj<MU, SG>(sp, h0, h1);
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
    if constexpr (SCALED) {
#pragma unroll
        for (int a = 0; a < 3; ++a) wd_recon1_scaled<MU, SG>(t0[a], t1[a], sc, acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
    } else if constexpr (FIRST) {
#pragma unroll
        for (int a = 0; a < 3; ++a) wd_recon1_first<MU, SG>(t0[a], t1[a], acc[a], acc[3 + a], acc[6 + a], acc[9 + a]);
    } else {
        wd_recon<MU, SG>(t0, t1, acc);
    }
}

// One of the eight neighbour terms (FIRST: the accumulators hold zeros).
template <int MU, bool FWD, bool DAG, class P, bool FIRST = false>
__device__ __forceinline__ void wd_hop_dir(const P &p, int s, const WdSite &c, typename P::C *acc)
{
    using C = typename P::C;
    constexpr bool kScaled = wd_site_scaled<P>::value;
    const int nb = wd_neighbour(p.g, s, c, MU, FWD);
    C sp[12];
    float sc = 1.f;
    if constexpr (kScaled) sc = p.load_in_raw(nb, sp);
    else p.load_in(nb, sp);
    C U[9];
    // forward: U_mu(x) stored at this site (parity cb);
    // backward: U_mu(x - mu) stored at the neighbour (parity 1-cb)
    if constexpr (FWD) p.load_link(MU, p.cb, s, U);
    else p.load_link(MU, 1 - p.cb, nb, U);
    wd_dir_terms<MU, FWD, DAG, FIRST, kScaled>(sp, sc, U, acc);
}

// 2 t - u, one rounding per real
__device__ __forceinline__ double2 wd_twice_minus(double2 t, double2 u)
{
    return make_double2(fma(2.0, t.x, -u.x), fma(2.0, t.y, -u.y));
}
__device__ __forceinline__ float2 wd_twice_minus(float2 t, float2 u)
{
    return make_float2(fmaf(2.f, t.x, -u.x), fmaf(2.f, t.y, -u.y));
}

// Both terms of direction MU at once (storages without a site scale).  In
// this basis the backward term's lower spin components are the negatives of
// the forward mapping applied to its (t0, t1), so with tf the forward and tb
// the backward colour vectors:
//   upper += tf + tb,   lower += R_fwd(tf - tb).
// u = tf + tb comes out of the backward SU(3) chain started at tf (no extra
// add) and tf - tb = 2 tf - u (one FMA): 12 fewer operations per direction
// pair than adding the two terms separately.
template <int MU, bool DAG, class P, bool FIRST>
__device__ __forceinline__ void wd_hop_mu(const P &p, int s, const WdSite &c, typename P::C *acc)
{
    using C = typename P::C;
    constexpr int SGF = DAG ? 1 : -1;  // forward sign, (FWD ? -1 : 1) * (DAG ? -1 : 1)
    constexpr int SGB = -SGF;
    C tf0[3], tf1[3];
    {
        const int nb = wd_neighbour(p.g, s, c, MU, true);
        C sp[12];
        p.load_in(nb, sp);
        C h0[3], h1[3];
        wd_proj<MU, SGF>(sp, h0, h1);
        C U[9];
        p.load_link(MU, p.cb, s, U);  // U_mu(x), stored at this site
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            tf0[a] = c_madd(c_madd(c_mul(U[a * 3], h0[0]), U[a * 3 + 1], h0[1]), U[a * 3 + 2], h0[2]);
            tf1[a] = c_madd(c_madd(c_mul(U[a * 3], h1[0]), U[a * 3 + 1], h1[1]), U[a * 3 + 2], h1[2]);
        }
    }
    C u0[3], u1[3];
    {
        const int nb = wd_neighbour(p.g, s, c, MU, false);
        C sp[12];
        p.load_in(nb, sp);
        C h0[3], h1[3];
        wd_proj<MU, SGB>(sp, h0, h1);
        C U[9];
        p.load_link(MU, 1 - p.cb, nb, U);  // U_mu(x - mu), stored at the neighbour
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            u0[a] = c_maddc(c_maddc(c_maddc(tf0[a], U[a], h0[0]), U[3 + a], h0[1]), U[6 + a], h0[2]);
            u1[a] = c_maddc(c_maddc(c_maddc(tf1[a], U[a], h1[0]), U[3 + a], h1[1]), U[6 + a], h1[2]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const C w0 = wd_twice_minus(tf0[a], u0[a]), w1 = wd_twice_minus(tf1[a], u1[a]);
        C &d0 = acc[a], &d1 = acc[3 + a], &d2 = acc[6 + a], &d3 = acc[9 + a];
        if constexpr (FIRST) {
            C z0, z1;
            wd_recon1_first<MU, SGF>(w0, w1, z0, z1, d2, d3);
            d0 = u0[a];
            d1 = u1[a];
        } else {
            C z0 = c_zero(C()), z1 = c_zero(C());
            wd_recon1<MU, SGF>(w0, w1, z0, z1, d2, d3);  // z0, z1 unused: only the lower part
            d0 = c_add(d0, u0[a]);
            d1 = c_add(d1, u1[a]);
        }
    }
}

template <bool DAG, class P>
__device__ __forceinline__ void wd_hop_site(const P &p, int s, typename P::C *acc)
{
    using C = typename P::C;
    const WdSite c = wd_site(p.g, s, p.cb);
    if constexpr (!wd_pair_dirs<P>::value || wd_site_scaled<P>::value) {
        // per-direction form (a site scale, if any, rides on each neighbour's own terms)
#pragma unroll
        for (int k = 0; k < 12; ++k) acc[k] = c_zero(C());
        wd_hop_dir<0, true, DAG, P, !wd_site_scaled<P>::value>(p, s, c, acc);
        wd_hop_dir<0, false, DAG>(p, s, c, acc);
        wd_hop_dir<1, true, DAG>(p, s, c, acc);
        wd_hop_dir<1, false, DAG>(p, s, c, acc);
        wd_hop_dir<2, true, DAG>(p, s, c, acc);
        wd_hop_dir<2, false, DAG>(p, s, c, acc);
        wd_hop_dir<3, true, DAG>(p, s, c, acc);
        wd_hop_dir<3, false, DAG>(p, s, c, acc);
    } else {
        wd_hop_mu<0, DAG, P, true>(p, s, c, acc);
        wd_hop_mu<1, DAG, P, false>(p, s, c, acc);
        wd_hop_mu<2, DAG, P, false>(p, s, c, acc);
        wd_hop_mu<3, DAG, P, false>(p, s, c, acc);
    }
}

// Optional occupancy hint: `static constexpr int kMinBlocks` (blocks per SM
// the register allocation must allow; 0 = no hint).
template <class P, class = void>
struct wd_min_blocks : std::integral_constant<int, 0> {};
template <class P>
struct wd_min_blocks<P, std::void_t<decltype(P::kMinBlocks)>> : std::integral_constant<int, P::kMinBlocks> {};

// Optional gate: a policy with a member `const int *stop` (non-null) makes the
// launch a no-op while *stop != 0 (device-driven solver loops queue
// iterations ahead and close the gate from the device).
template <class P, class = void>
struct wd_has_gate : std::false_type {};
template <class P>
struct wd_has_gate<P, std::void_t<decltype(P::stop)>> : std::true_type {};
template <class P>
__device__ __forceinline__ bool wd_gate_closed(const P &p)
{
    if constexpr (wd_has_gate<P>::value) return p.stop && *p.stop;
    return false;
}

template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads, wd_min_blocks<P>::value) wd_hop_kernel(const P p)
{
    if (wd_gate_closed(p)) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.g.Vh) return;
    typename P::C acc[12];
    wd_hop_site<DAG>(p, s, acc);
    p.epilogue(s, acc);
}

// The same over output sites [s_lo, s_hi) only (pipelined host-buffer path).
template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads, wd_min_blocks<P>::value) wd_hop_kernel_range(const P p, int s_lo,
                                                                                               int s_hi)
{
    const int s = s_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s_hi) return;
    typename P::C acc[12];
    wd_hop_site<DAG>(p, s, acc);
    p.epilogue(s, acc);
}
