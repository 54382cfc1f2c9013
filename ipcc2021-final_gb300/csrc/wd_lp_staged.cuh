// wd_lp_staged.cuh -- staging of the FP16 (per-site scale, 12-real links)
// hopping operands: each thread copies its operands of the next direction
// into shared memory by cp.async while it computes the current direction
// from the other slot (wd_h16m.cuh), so the prefetch holds no registers.  A
// thread reads back only the slots it filled itself: no block barrier.  Every
// address copied is one a register-loading kernel would read.
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
