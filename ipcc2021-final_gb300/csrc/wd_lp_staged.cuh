// wd_lp_staged.cuh -- the FP16 (per-site scale, 12-real links) hopping
// site with each thread's operands of the next direction staged in
// shared memory by cp.async while it computes the current direction from the
// other slot, so the prefetch holds no registers.  The decoding
// (Slot::unstage, as the storages' load functions decode) and the arithmetic
// (wd_dir_terms) are those of the register-loading kernels, so results are
// bit-identical to them.  A thread reads back only the slots it filled
// itself: no block barrier.  Every address copied is one the register-loading
// kernels read.
#pragma once
#include "wd_hop.cuh"
#include "wd_lp.cuh"

// two slots per thread of a block of T threads
template <class Sp, class Lk, int T>
struct LpStage {
    typename Sp::template Slot<T> sp[2];
    typename Lk::template Slot<T> lk[2];
};

// copy the operands of direction D = 2 mu + (0 forward, 1 backward) into a slot
template <int D, class P, class S>
__device__ __forceinline__ void lp_stage_dir(const P &p, int s, const WdSite &c, S &st, int slot)
{
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    const int t = threadIdx.x;
    const int nb = wd_neighbour(p.g, s, c, MU, FWD);
    p.in.stage(nb, st.sp[slot], t);
    // forward: U_mu(x) stored at this site (parity cb); backward: U_mu(x - mu) at the neighbour
    p.link.stage(MU, FWD ? p.cb : 1 - p.cb, FWD ? s : nb, st.lk[slot], t);
}

template <int D, bool DAG, class P, class S>
__device__ __forceinline__ void lp_compute_dir(const P &p, const S &st, int slot, float2 *acc)
{
    constexpr bool kScaled = wd_site_scaled<P>::value;
    const int t = threadIdx.x;
    float2 sp[12], U[9];
    const float sc = p.in.unstage(st.sp[slot], t, sp);
    p.link.unstage(st.lk[slot], t, U);
    // the first direction's terms are assigned, as in wd_hop_site
    wd_dir_terms<D / 2, (D % 2) == 0, DAG, D == 0 && !kScaled, kScaled>(sp, sc, U, acc);
}

template <int D, bool DAG, class P, class S>
__device__ __forceinline__ void lp_step(const P &p, int s, const WdSite &c, S &st, float2 *acc)
{
    if constexpr (D + 1 < 8) lp_stage_dir<D + 1>(p, s, c, st, (D + 1) & 1);
    wd_cp_async_commit();  // possibly empty: one group per step keeps the count
    wd_cp_async_wait<1>();
    lp_compute_dir<D, DAG>(p, st, D & 1, acc);
}

// acc = sum over the eight neighbours of output site s (the policy P has the
// members g, cb, in, link of the register-loading policies)
template <bool DAG, class P, class S>
__device__ __forceinline__ void lp_hop_site_staged(const P &p, int s, float2 *acc, S &st)
{
    const WdSite c = wd_site(p.g, s, p.cb);
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = c_zero(float2());
    lp_stage_dir<0>(p, s, c, st, 0);
    wd_cp_async_commit();
    lp_step<0, DAG>(p, s, c, st, acc);
    lp_step<1, DAG>(p, s, c, st, acc);
    lp_step<2, DAG>(p, s, c, st, acc);
    lp_step<3, DAG>(p, s, c, st, acc);
    lp_step<4, DAG>(p, s, c, st, acc);
    lp_step<5, DAG>(p, s, c, st, acc);
    lp_step<6, DAG>(p, s, c, st, acc);
    lp_step<7, DAG>(p, s, c, st, acc);
}
