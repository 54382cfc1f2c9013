// wd_batch.cu -- many systems in one launch: multi-RHS on one gauge field
// and lattices of uneven volume, solved together by a mixed-precision
// even-odd CG whose iterations are captured in a CUDA graph.
//
// Layout of a batch: systems are grouped by lattice (a group = one gauge
// field + the right-hand sides that use it).  A batched operator launch
// covers every group: blockIdx.x walks the groups' sites (a block table maps
// blocks to groups), blockIdx.y selects up to kSysPerBlock systems of the
// group.  Inside a block a warp holds 32 consecutive sites of one system,
// so spinor loads stay coalesced, and the kSysPerBlock warps that share a
// site range read the same links, which DRAM delivers once and L1 serves to
// the rest: link traffic is divided by the number of right-hand sides.
//
// Per-system scalars (rr, |t|^2, alpha, beta, active) live in device memory.
// One CG iteration (4 batched hops, per-system reductions, scalar update,
// vector updates) reads them there, so the iteration is captured once into a
// CUDA graph and replayed; systems that converge are masked off (active = 0)
// and their kernels return at once.  Between replays the host reads the
// per-system residuals and runs reliable updates (double-float or FP64) for
// the systems that need one -- the same recurrence as wd_mixed.cu.
#include <chrono>
#include <cmath>
#include <vector>
#include "wd_df.cuh"
#include "wd_hop.cuh"
#include "wd_lp.cuh"
#include "wd_reduce.cuh"
#include "wd_solver.h"

namespace {

constexpr int kSites = 32;       // sites per warp (one system per warp)
constexpr int kSysPerBlock = 8;  // warps (systems) per block
constexpr int kChunk = 8192;     // sites per reduction chunk (one block each)

struct BGroup {
    WdGeom g;
    const void *gauge;  // 12-real links of the group's lattice in the kernel storage
    int first_sys, nsys;
    int block_start;    // first blockIdx.x of this group
};

// one operand set per system for one batched hop launch
struct BSys {
    void *in, *out, *x;
    float *in_scale, *out_scale, *x_scale;
    int group;
};

struct BTable {
    const BGroup *groups;
    int ngroups;
    const BSys *sys;
    const float *alpha;  // per system
    const float *beta;
    const int *active;
    int cb;
};

template <class Sp, class Lk>
struct BatchHop {
    using C = float2;
    WdGeom g;
    int cb;
    Sp in, out, x;
    Lk link;
    bool has_x;
    float alpha, beta;
    __device__ __forceinline__ void load_in(int s, C *v) const { in.load(s, v); }
    __device__ __forceinline__ void load_link(int mu, int par, int s, C *U) const { link.load(mu, par, s, U); }
};

__device__ __forceinline__ int find_group(const BGroup *groups, int ngroups, int block)
{
    int lo = 0, hi = ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (groups[mid].block_start <= block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <bool DAG, bool F16>
__global__ void __launch_bounds__(kSites * kSysPerBlock) k_batch_hop(const BTable t)
{
    const int gi = find_group(t.groups, t.ngroups, blockIdx.x);
    const BGroup &G = t.groups[gi];
    const int r = blockIdx.y * kSysPerBlock + (threadIdx.x / kSites);
    const int s = (blockIdx.x - G.block_start) * kSites + (threadIdx.x % kSites);
    if (r >= G.nsys || s >= G.g.Vh) return;
    const int sys = G.first_sys + r;
    if (!t.active[sys]) return;
    const BSys &S = t.sys[sys];
    const int Vh = G.g.Vh;
    float2 acc[12];
    if constexpr (F16) {
        BatchHop<SpF16, LinkF16> p;
        p.g = G.g;
        p.cb = t.cb;
        p.in = SpF16{(uint4 *)S.in, S.in_scale, Vh};
        const uint4 *a = (const uint4 *)G.gauge;
        p.link = LinkF16{a, (const uint2 *)(a + (size_t)8 * Vh), Vh};
        wd_hop_site<DAG>(p, s, acc);
    } else {
        BatchHop<SpF32, LinkF32> p;
        p.g = G.g;
        p.cb = t.cb;
        p.in = SpF32{(float4 *)S.in, Vh};
        p.link = LinkF32{(const float4 *)G.gauge, Vh};
        wd_hop_site<DAG>(p, s, acc);
    }
    const float al = t.alpha[sys], be = t.beta[sys];
    float2 r12[12];
    if (S.x) {
        float2 xv[12];
        if constexpr (F16) SpF16{(uint4 *)S.x, S.x_scale, Vh}.load(s, xv);
        else SpF32{(float4 *)S.x, Vh}.load(s, xv);
#pragma unroll
        for (int c = 0; c < 12; ++c) r12[c] = c_axpby(al, acc[c], be, xv[c]);
    } else {
#pragma unroll
        for (int c = 0; c < 12; ++c) r12[c] = c_scale(acc[c], al);
    }
    if constexpr (F16) SpF16{(uint4 *)S.out, S.out_scale, Vh}.store(s, r12);
    else SpF32{(float4 *)S.out, Vh}.store(s, r12);
}

// ---------------------------------------------------------- batched BLAS
// per-system vectors: p, t, q (kernel storage), r_s, x_s (FP32), all even blocks
struct BVec {
    void *p, *t, *q;
    float *p_scale, *t_scale, *q_scale;
    float4 *rs, *xs;
    int Vh;
    int chunk0;  // first reduction chunk of this system
};

struct BState {
    double *rr;      // |r_s|^2 (sloppy) per system
    double *tt;      // |t|^2
    float *alpha, *beta;
    int *active;
    double *partial; // per reduction chunk
    int *chunk_sys;  // system of each reduction chunk
    int nchunks;
};

__device__ __forceinline__ dfr sq_acc(dfr acc, float2 v)
{
    return df_madd(df_madd(acc, dfr{v.x, 0.f}, dfr{v.x, 0.f}), dfr{v.y, 0.f}, dfr{v.y, 0.f});
}

// one block per chunk of kChunk... sites of one system
template <bool F16>
__global__ void __launch_bounds__(WD_RED_THREADS) k_batch_norm_t(const BVec *v, BState st)
{
    const int c = blockIdx.x;
    const int sys = st.chunk_sys[c];
    dfr acc{0.f, 0.f};
    if (st.active[sys]) {
        const BVec &B = v[sys];
        const int s0 = (c - B.chunk0) * kChunk;
        const int s1 = min(s0 + kChunk, B.Vh);
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            float2 tv[12];
            if constexpr (F16) SpF16{(uint4 *)B.t, B.t_scale, B.Vh}.load(s, tv);
            else SpF32{(float4 *)B.t, B.Vh}.load(s, tv);
#pragma unroll
            for (int k = 0; k < 12; ++k) acc = sq_acc(acc, tv[k]);
        }
    }
    double2 *part = reinterpret_cast<double2 *>(st.partial);
    wd_block_partial(df_value(acc), 0.0, part);
}

// x_s += alpha p; r_s -= alpha q; chunk partial of |r_s|^2
template <bool F16>
__global__ void __launch_bounds__(WD_RED_THREADS) k_batch_update(const BVec *v, BState st)
{
    const int c = blockIdx.x;
    const int sys = st.chunk_sys[c];
    dfr acc{0.f, 0.f};
    if (st.active[sys]) {
        const BVec &B = v[sys];
        const float a = st.alpha[sys];
        const int s0 = (c - B.chunk0) * kChunk;
        const int s1 = min(s0 + kChunk, B.Vh);
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            float2 pv[12], qv[12], xv[12], rv[12];
            if constexpr (F16) {
                SpF16{(uint4 *)B.p, B.p_scale, B.Vh}.load(s, pv);
                SpF16{(uint4 *)B.q, B.q_scale, B.Vh}.load(s, qv);
            } else {
                SpF32{(float4 *)B.p, B.Vh}.load(s, pv);
                SpF32{(float4 *)B.q, B.Vh}.load(s, qv);
            }
            const SpF32 xs{B.xs, B.Vh}, rs{B.rs, B.Vh};
            xs.load(s, xv);
            rs.load(s, rv);
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                xv[k] = make_float2(fmaf(a, pv[k].x, xv[k].x), fmaf(a, pv[k].y, xv[k].y));
                rv[k] = make_float2(fmaf(-a, qv[k].x, rv[k].x), fmaf(-a, qv[k].y, rv[k].y));
                acc = sq_acc(acc, rv[k]);
            }
            xs.store(s, xv);
            rs.store(s, rv);
        }
    }
    double2 *part = reinterpret_cast<double2 *>(st.partial);
    wd_block_partial(df_value(acc), 0.0, part);
}

// p = r_s + beta p
template <bool F16>
__global__ void __launch_bounds__(WD_RED_THREADS) k_batch_xpay(const BVec *v, BState st)
{
    const int c = blockIdx.x;
    const int sys = st.chunk_sys[c];
    if (!st.active[sys]) return;
    const BVec &B = v[sys];
    const float be = st.beta[sys];
    const int s0 = (c - B.chunk0) * kChunk;
    const int s1 = min(s0 + kChunk, B.Vh);
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        float2 pv[12], rv[12];
        SpF32{B.rs, B.Vh}.load(s, rv);
        if constexpr (F16) SpF16{(uint4 *)B.p, B.p_scale, B.Vh}.load(s, pv);
        else SpF32{(float4 *)B.p, B.Vh}.load(s, pv);
#pragma unroll
        for (int k = 0; k < 12; ++k) pv[k] = make_float2(fmaf(be, pv[k].x, rv[k].x), fmaf(be, pv[k].y, rv[k].y));
        if constexpr (F16) SpF16{(uint4 *)B.p, B.p_scale, B.Vh}.store(s, pv);
        else SpF32{(float4 *)B.p, B.Vh}.store(s, pv);
    }
}

// per-system sums of chunk partials (fixed order) -> out[sys]; then scalars
// mode 0: tt = sum; alpha = rr / tt
// mode 1: rr_new = sum; beta = rr_new / rr; rr = rr_new
__global__ void k_batch_scalars(const BVec *v, BState st, int nsys, int mode)
{
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= nsys || !st.active[sys]) return;
    const BVec &B = v[sys];
    const int nch = (B.Vh + kChunk - 1) / kChunk;
    const double2 *part = reinterpret_cast<const double2 *>(st.partial);
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += part[B.chunk0 + c].x;
    if (mode == 0) {
        st.tt[sys] = s;
        st.alpha[sys] = s > 0 ? (float)(st.rr[sys] / s) : 0.f;
    } else {
        st.beta[sys] = st.rr[sys] > 0 ? (float)(s / st.rr[sys]) : 0.f;
        st.rr[sys] = s;
    }
}

}  // namespace

// ====================================================== host-side solver

namespace {

struct SysBufs {
    WdVecBuf p, t, q, tmp_o, rs, xs;                       // low precision / FP32
    WdVecBuf hs, hx, bhat, s_e, r_h, t_h, tmp_oh;          // high precision
    double norm_b = 1, rr_max = 0, target = 0, ratio = 1, true_res = 1;
    int updates = 0, iters = 0;
    bool converged = false;
};

template <class T>
struct DevArray {
    T *p = nullptr;
    size_t n = 0;
    wd_context *ctx = nullptr;
    ~DevArray()
    {
        if (ctx) wd_dev_free(ctx, p);
    }
    wd_status alloc(wd_context *c, size_t count)
    {
        n = count;
        ctx = c;
        return wd_dev_alloc(c, (void **)&p, count * sizeof(T));
    }
    wd_status put(wd_context *ctx, const std::vector<T> &h)
    {
        WD_CUDA(ctx, cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
        return WD_OK;
    }
};

}  // namespace

extern "C" wd_status wd_solve_batch(wd_context *ctx, int nsys, const wd_lattice *const *lats,
                                    const wd_field *const *srcs, wd_field *const *dests, const double *masses,
                                    const wd_solver_params *prm, wd_solver_stats *stats)
{
    if (!ctx || nsys <= 0 || !lats || !srcs || !dests || !masses || !prm)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (prm->prec != WD_PREC_F32 && prm->prec != WD_PREC_F16)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "batched solves run a mixed FP32 or FP16 inner solver");
    const wd_precision L = prm->prec;
    const wd_precision H = prm->prec_reliable == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
    const bool f16 = L == WD_PREC_F16;
    const double delta = prm->delta > 0 && prm->delta < 1 ? prm->delta : 0.1;
    const auto t0 = std::chrono::steady_clock::now();
    wd_status st;

    // ---- groups: consecutive systems on the same lattice share links
    std::vector<int> order(nsys);
    for (int i = 0; i < nsys; ++i) {
        if (!lats[i] || !srcs[i] || !dests[i]) return wd_fail(ctx, WD_ERR_BAD_ARG, "null system");
        if (srcs[i]->storage != WD_PREC_F64 || dests[i]->storage != WD_PREC_F64 || srcs[i]->lat->volume != lats[i]->volume ||
            dests[i]->lat->volume != lats[i]->volume)
            return wd_fail(ctx, WD_ERR_BAD_ARG, "batch fields must be FP64 fields of their system's lattice");
        order[i] = i;
    }
    std::vector<BGroup> groups;
    std::vector<int> sys_of_slot;  // slot -> system index (grouped order)
    {
        std::vector<bool> done(nsys, false);
        int blocks = 0;
        for (int i = 0; i < nsys; ++i) {
            if (done[i]) continue;
            BGroup G{};
            G.g = lats[i]->g;
            G.first_sys = (int)sys_of_slot.size();
            G.block_start = blocks;
            for (int j = i; j < nsys; ++j)
                if (!done[j] && lats[j] == lats[i]) {
                    done[j] = true;
                    sys_of_slot.push_back(j);
                }
            G.nsys = (int)sys_of_slot.size() - G.first_sys;
            if ((st = wd_lattice_gauge_lp(ctx, lats[i], L)) != WD_OK) return st;
            G.gauge = f16 ? lats[i]->gauge_h12 : lats[i]->gauge_f32;
            blocks += (G.g.Vh + kSites - 1) / kSites;
            groups.push_back(G);
        }
    }
    int grid_y = 1;
    for (const BGroup &G : groups) grid_y = std::max(grid_y, (G.nsys + kSysPerBlock - 1) / kSysPerBlock);
    const int grid_x = groups.back().block_start + (groups.back().g.Vh + kSites - 1) / kSites;

    // ---- per-system buffers (slot order)
    std::vector<SysBufs> sb(nsys);
    std::vector<BVec> bvec(nsys);
    std::vector<int> chunk_sys;
    for (int k = 0; k < nsys; ++k) {
        const int i = sys_of_slot[k];
        const wd_lattice *lat = lats[i];
        const int64_t nh = (int64_t)12 * lat->g.Vh;
        SysBufs &B = sb[k];
        for (WdVecBuf *b : {&B.p, &B.t, &B.q, &B.tmp_o})
            if ((st = wd_vec_alloc(ctx, *b, L, nh)) != WD_OK) return st;
        for (WdVecBuf *b : {&B.rs, &B.xs})
            if ((st = wd_vec_alloc(ctx, *b, WD_PREC_F32, nh)) != WD_OK) return st;
        for (WdVecBuf *b : {&B.bhat, &B.s_e, &B.r_h, &B.t_h, &B.tmp_oh})
            if ((st = wd_vec_alloc(ctx, *b, H, nh)) != WD_OK) return st;
        if ((st = wd_vec_alloc(ctx, B.hs, H, 2 * nh)) != WD_OK) return st;
        if ((st = wd_vec_alloc(ctx, B.hx, H, 2 * nh)) != WD_OK) return st;
        BVec &v = bvec[k];
        v.p = B.p.v.p, v.t = B.t.v.p, v.q = B.q.v.p;
        v.p_scale = B.p.v.scale, v.t_scale = B.t.v.scale, v.q_scale = B.q.v.scale;
        v.rs = (float4 *)B.rs.v.p, v.xs = (float4 *)B.xs.v.p;
        v.Vh = lat->g.Vh;
        v.chunk0 = (int)chunk_sys.size();
        for (int c = 0; c < (v.Vh + kChunk - 1) / kChunk; ++c) chunk_sys.push_back(k);
    }
    const int nchunks = (int)chunk_sys.size();

    // ---- device tables: 4 hop tables (Mhat: p->tmp_o->t, Mhat^dag: t->tmp_o->q)
    DevArray<BGroup> d_groups;
    DevArray<BSys> d_sys[4];
    DevArray<float> d_alpha[4], d_beta[4];
    DevArray<BVec> d_vec;
    DevArray<double> d_rr, d_tt, d_partial;
    DevArray<float> d_a, d_b;
    DevArray<int> d_active, d_chunk_sys;
    if ((st = d_groups.alloc(ctx, groups.size())) != WD_OK || (st = d_groups.put(ctx, groups)) != WD_OK) return st;
    for (int h = 0; h < 4; ++h) {
        std::vector<BSys> tab(nsys);
        std::vector<float> al(nsys), be(nsys);
        for (int k = 0; k < nsys; ++k) {
            const double a = 4.0 + masses[sys_of_slot[k]];
            const SysBufs &B = sb[k];
            const WdVec *in, *out, *x = nullptr;
            // h = 0: p -> tmp_o (cb 1); 1: tmp_o -> t with x = p (cb 0); 2: t -> tmp_o; 3: tmp_o -> q with x = t
            const WdVec *vin[4] = {&B.p.v, &B.tmp_o.v, &B.t.v, &B.tmp_o.v};
            const WdVec *vout[4] = {&B.tmp_o.v, &B.t.v, &B.tmp_o.v, &B.q.v};
            const WdVec *vx[4] = {nullptr, &B.p.v, nullptr, &B.t.v};
            in = vin[h], out = vout[h], x = vx[h];
            tab[k] = BSys{in->p, out->p, x ? x->p : nullptr, in->scale, out->scale, x ? x->scale : nullptr, 0};
            al[k] = (h % 2 == 0) ? 1.0f : (float)(-0.25 / a);
            be[k] = (h % 2 == 0) ? 0.0f : (float)a;
        }
        if ((st = d_sys[h].alloc(ctx, nsys)) != WD_OK || (st = d_sys[h].put(ctx, tab)) != WD_OK) return st;
        if ((st = d_alpha[h].alloc(ctx, nsys)) != WD_OK || (st = d_alpha[h].put(ctx, al)) != WD_OK) return st;
        if ((st = d_beta[h].alloc(ctx, nsys)) != WD_OK || (st = d_beta[h].put(ctx, be)) != WD_OK) return st;
    }
    if ((st = d_vec.alloc(ctx, nsys)) != WD_OK || (st = d_vec.put(ctx, bvec)) != WD_OK) return st;
    if ((st = d_rr.alloc(ctx, nsys)) != WD_OK || (st = d_tt.alloc(ctx, nsys)) != WD_OK) return st;
    if ((st = d_a.alloc(ctx, nsys)) != WD_OK || (st = d_b.alloc(ctx, nsys)) != WD_OK) return st;
    if ((st = d_active.alloc(ctx, nsys)) != WD_OK) return st;
    if ((st = d_partial.alloc(ctx, 2 * (size_t)nchunks)) != WD_OK) return st;
    if ((st = d_chunk_sys.alloc(ctx, nchunks)) != WD_OK || (st = d_chunk_sys.put(ctx, chunk_sys)) != WD_OK) return st;
    const BState bst{d_rr.p, d_tt.p, d_a.p, d_b.p, d_active.p, d_partial.p, d_chunk_sys.p, nchunks};

    // ---- per-system set-up and the first (restart) reliable update
    auto sys_slices = [&](int k, WdVec &b_e, WdVec &b_o, WdVec &x_e, WdVec &x_o) {
        const int Vh = lats[sys_of_slot[k]]->g.Vh;
        b_e = sb[k].hs.v;
        b_o = wd_offset(sb[k].hs.v, (int64_t)12 * Vh, Vh);
        x_e = sb[k].hx.v;
        x_o = wd_offset(sb[k].hx.v, (int64_t)12 * Vh, Vh);
    };
    std::vector<double> h_rr(nsys), h_rr_last(nsys);
    std::vector<int> h_active(nsys, 1);
    // reliable update of system k: x_e += x_s; s = bhat - Mhat x_e; r = Mhat^dag s; r_s, (p) <- r
    auto reliable = [&](int k, bool reset_p, double *rr, double *ss) -> wd_status {
        const int i = sys_of_slot[k];
        const wd_lattice *lat = lats[i];
        const int Vh = lat->g.Vh;
        const int64_t nh = (int64_t)12 * Vh;
        const double m = masses[i];
        SysBufs &B = sb[k];
        WdVec b_e, b_o, x_e, x_o;
        sys_slices(k, b_e, b_o, x_e, x_o);
        wd_status e;
        // x_H += x_s; x_s = 0
        if ((e = wd_mx_accum(ctx, Vh, H, B.xs.v, x_e)) != WD_OK) return e;
        if ((e = wd_apply_Mhat_v(ctx, lat, x_e, B.t_h.v, B.tmp_oh.v, m, 0)) != WD_OK) return e;
        if ((e = wd_v_xpayz(ctx, B.bhat.v, make_double2(-1.0, 0.0), B.t_h.v, B.s_e.v, nh)) != WD_OK) return e;
        if ((e = wd_apply_Mhat_v(ctx, lat, B.s_e.v, B.r_h.v, B.tmp_oh.v, m, 1)) != WD_OK) return e;
        if ((e = wd_v_norm2(ctx, B.r_h.v, nh, 0)) != WD_OK) return e;
        if ((e = wd_v_norm2(ctx, B.s_e.v, nh, 1)) != WD_OK) return e;
        double2 v[2];
        if ((e = wd_red_fetch(ctx, 2, v)) != WD_OK) return e;
        *rr = v[0].x;
        *ss = v[1].x;
        // r_s <- r (FP32); p <- r on a restart (otherwise t, rewritten next iteration, takes the copy)
        return wd_mx_from_h(ctx, Vh, L, H, B.r_h.v, B.rs.v, reset_p ? B.p.v : B.t.v);
    };

    for (int k = 0; k < nsys; ++k) {
        const int i = sys_of_slot[k];
        const wd_lattice *lat = lats[i];
        const int Vh = lat->g.Vh;
        const int64_t nh = (int64_t)12 * Vh;
        const double a = 4.0 + masses[i];
        SysBufs &B = sb[k];
        if (H == WD_PREC_DF64) {
            if ((st = wd_convert_f64_to_df(ctx, srcs[i]->d, (float4 *)B.hs.v.p, 2 * nh)) != WD_OK) return st;
        } else {
            WD_CUDA(ctx, cudaMemcpyAsync(B.hs.v.p, srcs[i]->d, 2 * nh * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
        }
        WdVec b_e, b_o, x_e, x_o;
        sys_slices(k, b_e, b_o, x_e, x_o);
        if ((st = wd_hop_v(ctx, lat, b_o, B.bhat.v, &b_e, 0, 0, 0.5 / a, 1.0)) != WD_OK) return st;
        if ((st = wd_v_zero(ctx, B.hx.v, 2 * nh)) != WD_OK) return st;
        if ((st = wd_v_zero(ctx, B.xs.v, nh)) != WD_OK) return st;
        if ((st = wd_red_norm2(ctx, srcs[i]->d, 2 * nh, 0)) != WD_OK) return st;
        double2 v;
        if ((st = wd_red_fetch(ctx, 1, &v)) != WD_OK) return st;
        B.norm_b = v.x > 0 ? std::sqrt(v.x) : 1.0;
        double rr, ss;
        if ((st = reliable(k, true, &rr, &ss)) != WD_OK) return st;
        B.true_res = std::sqrt(ss) / B.norm_b;
        B.ratio = ss > 0 ? std::sqrt(rr / ss) : 1.0;
        B.target = prm->tol * B.norm_b * B.ratio * 0.5;
        B.rr_max = rr;
        h_rr[k] = rr;
        B.converged = B.true_res <= prm->tol;
        h_active[k] = B.converged ? 0 : 1;
    }
    if ((st = d_rr.put(ctx, h_rr)) != WD_OK) return st;
    if ((st = d_active.put(ctx, h_active)) != WD_OK) return st;

    // ---- capture one iteration into a CUDA graph
    auto hop = [&](int h, int cb, int dag) -> wd_status {
        const BTable t{d_groups.p, (int)groups.size(), d_sys[h].p, d_alpha[h].p, d_beta[h].p, d_active.p, cb};
        dim3 grid(grid_x, grid_y);
        const int threads = kSites * kSysPerBlock;
        if (f16) {
            if (dag) k_batch_hop<true, true><<<grid, threads, 0, ctx->stream>>>(t);
            else k_batch_hop<false, true><<<grid, threads, 0, ctx->stream>>>(t);
        } else {
            if (dag) k_batch_hop<true, false><<<grid, threads, 0, ctx->stream>>>(t);
            else k_batch_hop<false, false><<<grid, threads, 0, ctx->stream>>>(t);
        }
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    auto iteration = [&]() -> wd_status {
        wd_status e;
        if ((e = hop(0, 1, 0)) != WD_OK || (e = hop(1, 0, 0)) != WD_OK) return e;  // t = Mhat p
        if ((e = hop(2, 1, 1)) != WD_OK || (e = hop(3, 0, 1)) != WD_OK) return e;  // q = Mhat^dag t
        if (f16) k_batch_norm_t<true><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        else k_batch_norm_t<false><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        WD_LAUNCHED(ctx);
        k_batch_scalars<<<(nsys + 127) / 128, 128, 0, ctx->stream>>>(d_vec.p, bst, nsys, 0);
        WD_LAUNCHED(ctx);
        if (f16) k_batch_update<true><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        else k_batch_update<false><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        WD_LAUNCHED(ctx);
        k_batch_scalars<<<(nsys + 127) / 128, 128, 0, ctx->stream>>>(d_vec.p, bst, nsys, 1);
        WD_LAUNCHED(ctx);
        if (f16) k_batch_xpay<true><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        else k_batch_xpay<false><<<nchunks, WD_RED_THREADS, 0, ctx->stream>>>(d_vec.p, bst);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    const int per_graph = 4;  // iterations per graph launch between host checks
    const uint64_t launches_before_capture = ctx->launches;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    WD_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    wd_status cap = WD_OK;
    for (int k = 0; k < per_graph && cap == WD_OK; ++k) cap = iteration();
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (cap != WD_OK) {
        if (graph) cudaGraphDestroy(graph);
        return cap;
    }
    if (ce != cudaSuccess) return wd_cuda_check(ctx, ce, "cudaStreamEndCapture");
    const uint64_t kernels_per_graph = ctx->launches - launches_before_capture;
    ctx->launches = launches_before_capture;  // counted per replay below
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return wd_cuda_check(ctx, ie, "cudaGraphInstantiate");
    struct GraphGuard {
        cudaGraphExec_t e;
        ~GraphGuard() { cudaGraphExecDestroy(e); }
    } guard{exec};

    // ---- iterate: graph replays, host checks, reliable updates, masking
    int iters = 0, graph_launches = 0;
    std::vector<double> rr_dev(nsys);
    bool any = false;
    for (int v : h_active) any = any || v;
    while (any && iters < prm->max_iter) {
        h_rr_last.assign(h_rr.begin(), h_rr.end());
        WD_CUDA(ctx, cudaGraphLaunch(exec, ctx->stream));
        ctx->launches += kernels_per_graph;
        ++graph_launches;
        iters += per_graph;
        WD_CUDA(ctx, cudaMemcpyAsync(rr_dev.data(), d_rr.p, nsys * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        bool changed = false;
        any = false;
        for (int k = 0; k < nsys; ++k) {
            if (!h_active[k]) continue;
            SysBufs &B = sb[k];
            B.iters += per_graph;
            const double rr_new = rr_dev[k];
            if (!std::isfinite(rr_new)) return wd_fail(ctx, WD_ERR_NAN, "batched CG residual is not finite");
            if (rr_new < delta * delta * B.rr_max || std::sqrt(rr_new) <= B.target) {
                double rr, ss;
                if ((st = reliable(k, false, &rr, &ss)) != WD_OK) return st;
                B.updates++;
                B.true_res = std::sqrt(ss) / B.norm_b;
                if (B.true_res <= prm->tol) {
                    B.converged = true;
                    h_active[k] = 0;
                    changed = true;
                    continue;
                }
                if (std::sqrt(rr_new) <= B.target) {
                    B.ratio = ss > 0 ? std::sqrt(rr / ss) : B.ratio;
                    B.target = std::fmin(B.target * 0.5, prm->tol * B.norm_b * B.ratio * 0.5);
                }
                // continue the recurrence from the recomputed residual: beta of
                // the next iteration uses rr_new over this rr
                B.rr_max = rr;
                rr_dev[k] = rr;
                changed = true;
            }
            any = true;
        }
        if (changed) {
            std::vector<double> rr_put(rr_dev.begin(), rr_dev.end());
            WD_CUDA(ctx, cudaMemcpyAsync(d_rr.p, rr_put.data(), nsys * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
            WD_CUDA(ctx, cudaMemcpyAsync(d_active.p, h_active.data(), nsys * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
            WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
        h_rr.assign(rr_dev.begin(), rr_dev.end());
    }

    // ---- finish: fold x_s, reconstruct x_o, write the FP64 solutions
    for (int k = 0; k < nsys; ++k) {
        const int i = sys_of_slot[k];
        const wd_lattice *lat = lats[i];
        const int Vh = lat->g.Vh;
        const int64_t nh = (int64_t)12 * Vh;
        const double a = 4.0 + masses[i];
        SysBufs &B = sb[k];
        WdVec b_e, b_o, x_e, x_o;
        sys_slices(k, b_e, b_o, x_e, x_o);
        if (!B.converged) {
            double rr, ss;
            if ((st = reliable(k, false, &rr, &ss)) != WD_OK) return st;
            B.true_res = std::sqrt(ss) / B.norm_b;
        }
        if ((st = wd_hop_v(ctx, lat, x_e, x_o, &b_o, 1, 0, 0.5 / a, 1.0 / a)) != WD_OK) return st;
        if (H == WD_PREC_DF64) {
            if ((st = wd_convert_df_to_f64(ctx, (const float4 *)B.hx.v.p, dests[i]->d, 2 * nh)) != WD_OK) return st;
        } else {
            WD_CUDA(ctx, cudaMemcpyAsync(dests[i]->d, B.hx.v.p, 2 * nh * sizeof(double2), cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    bool all = true;
    for (int k = 0; k < nsys; ++k) {
        const int i = sys_of_slot[k];
        wd_solver_stats s{};
        s.iterations = sb[k].iters;
        s.reliable_updates = sb[k].updates;
        s.residual = sb[k].true_res;
        s.converged = sb[k].converged;
        s.seconds = secs;
        if (stats) {
            // FP64 true residual of each returned solution (a check, after the timed solve)
            WdVecBuf tmp;
            if ((st = wd_vec_alloc(ctx, tmp, WD_PREC_F64, lats[i]->volume * 12)) != WD_OK) return st;
            st = wd_true_residual(ctx, lats[i], srcs[i]->d, dests[i]->d, (double2 *)tmp.v.p, masses[i],
                                  &s.true_residual);
            if (st != WD_OK) return st;
            stats[i] = s;
        }
        all = all && sb[k].converged;
    }
    (void)graph_launches;
    return all ? WD_OK : WD_ERR_NOT_CONVERGED;
}
