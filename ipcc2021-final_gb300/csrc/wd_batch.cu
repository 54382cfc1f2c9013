// wd_batch.cu -- many systems in one launch: multi-RHS on one gauge field
// and lattices of uneven volume, solved together by a mixed-precision
// even-odd CG whose iterations are captured in a CUDA graph.
//
// Layout of a batch: systems are grouped by lattice (a group = one gauge
// field + the right-hand sides that use it).  A batched operator launch
// covers every group: blockIdx.x walks the groups' sites (a block table maps
// blocks to groups), blockIdx.y selects up to SYS systems of the group (SYS
// and the occupancy bound are tuned launch variants).  Inside a block a warp
// holds 32 consecutive sites of one system, so spinor loads stay coalesced,
// and the SYS warps that share a site range read the same links, which DRAM
// delivers once and L1 serves to the rest: link traffic is divided by the
// number of right-hand sides.
//
// Per-system scalars (rr, |t|^2, alpha, beta, active, the reliable-update
// trigger) live in device memory.  One CG iteration (4 batched hops, two of
// them with reducing epilogues, two per-system scalar kernels, the p update)
// reads them there, so iterations are captured into a CUDA graph and
// replayed; a system whose residual calls for a reliable update is masked by
// the device at that iteration and its kernels return at once.  Between
// replays the host reads the scalars and runs the reliable updates (double-
// float or FP64) the device asked for -- the recurrence of wd_mixed.cu.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <memory>
#include <type_traits>
#include <vector>
#include "wd_df.cuh"
#include "wd_hop.cuh"
#include "wd_lp.cuh"
#include "wd_h16m.cuh"
#include "wd_reduce.cuh"
#include "wd_solver.h"
#include "wd_tune.h"

namespace {

constexpr int kSites = 32;  // sites per warp (one system per warp)
constexpr int kChunk = 8192;     // sites per xpay chunk (one block each)
constexpr int kBatchHopVariants = 7;
constexpr int kMaxPerGraph = 8;  // iterations queued per graph launch at most

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
    void *p;              // update epilogue: p (kernel storage) and its scales
    float *p_scale;
    float4 *rs, *xs;      // update epilogue: FP32 r_s and x_s
    int part0, nparts;    // this system's warp partials: [part0, part0 + nparts)
};

// Per-system scalars of the batched CG, in device memory.  The iteration
// kernels read and write them; after a graph launch the host reads the
// whole array once.  A system whose |r_s|^2 has fallen by delta^2 since its
// last reliable update (or reached its target) is masked (active = 0,
// wait = 1) by the device at once; later iterations skip it until the host
// has run its reliable update.
struct BScal {
    double rr, rr_max, target2, tt, rr_new;
    float alpha, beta;
    int active;  // 1: iterating
    int wait;    // 1: reliable update due; 2: non-finite scalar
    int iters;
    int pad;
};

// epilogue of a batched hop: plain (h0, h2), |t|^2 (h1), CG update (h3)
enum { kBEpiPlain = 0, kBEpiNorm = 1, kBEpiUpdate = 2 };

struct BTable {
    const BGroup *groups;
    int ngroups;
    const BSys *sys;
    const float *alpha;  // per system: the hop's output scale and x coefficient
    const float *beta;
    BScal *sc;
    double *partial;     // warp partials of the reducing epilogues
    int cb;
};

template <class Sp, class Lk>
struct BatchHop {
    using C = float2;
    static constexpr bool kSiteScale = Sp::kScaled;
    WdGeom g;
    int cb;
    Sp in, out, x;
    Lk link;
    bool has_x;
    float alpha, beta;
    __device__ __forceinline__ void load_in(int s, C *v) const { in.load(s, v); }
    __device__ __forceinline__ float load_in_raw(int s, C *v) const
    {
        if constexpr (Sp::kScaled) return in.load_raw(s, v);
        in.load(s, v);
        return 1.f;
    }
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

template <bool F16>
struct BSp {
    using T = std::conditional_t<F16, SpF16, SpF32>;
    static __device__ __forceinline__ T make(void *p, float *scale, int Vh)
    {
        if constexpr (F16) return SpF16{(uint4 *)p, scale, Vh};
        else return SpF32{(float4 *)p, Vh};
    }
};

// r = alpha acc (+ beta x) of system sys at site s, then the epilogue EPI;
// returns the site's contribution to the reduction (0 for plain)
template <bool F16, int EPI>
__device__ __forceinline__ float batch_epilogue(const BTable &t, const BSys &S, int sys, int s, int Vh,
                                                const float2 *acc)
{
    const float al = t.alpha[sys], be = t.beta[sys];
    float2 r[12];
    if (S.x) {
        float2 xv[12];
        float bx = be;  // beta times the x site's scale
        if constexpr (F16) bx *= SpF16{(uint4 *)S.x, S.x_scale, Vh}.load_raw(s, xv);
        else SpF32{(float4 *)S.x, Vh}.load(s, xv);
#pragma unroll
        for (int c = 0; c < 12; ++c) r[c] = c_axpby(al, acc[c], bx, xv[c]);
    } else {
#pragma unroll
        for (int c = 0; c < 12; ++c) r[c] = c_scale(acc[c], al);
    }
    float n = 0.f;
    if constexpr (EPI != kBEpiUpdate) {
        if constexpr (EPI == kBEpiNorm) {
#pragma unroll
            for (int c = 0; c < 12; ++c) n = fmaf(r[c].x, r[c].x, fmaf(r[c].y, r[c].y, n));
        }
        BSp<F16>::make(S.out, S.out_scale, Vh).store(s, r);
    } else {
        // q = r is not stored: r_s -= alpha q, x_s += alpha p
        const float a = t.sc[sys].alpha;
        const SpF32 rs{S.rs, Vh}, xs{S.xs, Vh};
        float2 v[12];
        rs.load(s, v);
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            v[c] = make_float2(fmaf(-a, r[c].x, v[c].x), fmaf(-a, r[c].y, v[c].y));
            n = fmaf(v[c].x, v[c].x, fmaf(v[c].y, v[c].y, n));
        }
        rs.store(s, v);
        BSp<F16>::make(S.p, S.p_scale, Vh).load(s, r);
        xs.load(s, v);
#pragma unroll
        for (int c = 0; c < 12; ++c) v[c] = make_float2(fmaf(a, r[c].x, v[c].x), fmaf(a, r[c].y, v[c].y));
        xs.store(s, v);
    }
    return n;
}

// the operands of one system: its input spinor and the group's links
template <bool F16>
__device__ __forceinline__ auto batch_policy(const BTable &t, const BGroup &G, const BSys &S)
{
    const int Vh = G.g.Vh;
    if constexpr (F16) {
        BatchHop<SpF16, LinkF16> p;
        p.g = G.g;
        p.cb = t.cb;
        p.in = SpF16{(uint4 *)S.in, S.in_scale, Vh};
        const uint4 *a = (const uint4 *)G.gauge;
        p.link = LinkF16{a, (const uint2 *)(a + (size_t)8 * Vh), Vh};
        return p;
    } else {
        BatchHop<SpF32, LinkF32> p;
        p.g = G.g;
        p.cb = t.cb;
        p.in = SpF32{(float4 *)S.in, Vh};
        p.link = LinkF32{(const float4 *)G.gauge, Vh};
        return p;
    }
}

// SYS systems (warps) per block sharing the block's 32 sites; MINB blocks per
// SM (0: no bound) bound the registers.  A warp is one system's 32
// consecutive sites, so a reducing epilogue writes one partial per warp.
// R2 (FP16 storage): row 2 of the block's links is rebuilt once per site and
// direction into shared memory by all the block's warps together, and every
// system reads it there instead of rebuilding it (the same values).
template <bool DAG, bool F16, int SYS, int MINB, int EPI, bool R2 = false>
__global__ void __launch_bounds__(kSites * SYS, MINB) k_batch_hop(const BTable t)
{
    const int gi = find_group(t.groups, t.ngroups, blockIdx.x);
    const BGroup &G = t.groups[gi];
    const int r = blockIdx.y * SYS + (threadIdx.x / kSites);
    const int blk = blockIdx.x - G.block_start;
    const int lane = threadIdx.x % kSites;
    const int s = blk * kSites + lane;
    static_assert(!R2 || F16, "the shared row-2 table is for 12-real FP16 links");
    __shared__ unsigned r2[R2 ? 8 : 1][3][kSites];
    if constexpr (R2) {
        // every warp takes part, whether or not its system iterates
        if (s < G.g.Vh) {
            const uint4 *a = (const uint4 *)G.gauge;
            const LinkF16 lk{a, (const uint2 *)(a + (size_t)8 * G.g.Vh), G.g.Vh};
            h16_fill_row2<SYS>(G.g, t.cb, lk, s, r2, threadIdx.x / kSites, lane);
        }
        __syncthreads();
    }
    if (r >= G.nsys) return;  // whole warps
    const int sys = G.first_sys + r;
    if (!t.sc[sys].active) return;
    const BSys &S = t.sys[sys];
    float v = 0.f;
    if (s < G.g.Vh) {
        float2 acc[12];
        // FP16 storage: the FP16-operand arithmetic of the solo FP16 kernel
        if constexpr (R2) h16_hop_site_r2<DAG>(batch_policy<F16>(t, G, S), s, r2, lane, acc);
        else if constexpr (F16) h16_hop_site<DAG>(batch_policy<F16>(t, G, S), s, acc);
        else wd_hop_site<DAG>(batch_policy<F16>(t, G, S), s, acc);
        v = batch_epilogue<F16, EPI>(t, S, sys, s, G.g.Vh, acc);
    }
    if constexpr (EPI != kBEpiPlain) {
        const double d = wd_warp_sum((double)v);
        if ((threadIdx.x & 31) == 0) t.partial[S.part0 + blk] = d;
    }
}

// per-system vectors for the xpay pass (even blocks)
struct BVec {
    void *p;
    float *p_scale;
    float4 *rs;
    int Vh;
    int chunk0;  // first xpay chunk of this system
};

// p = r_s + beta p for the iterating systems
template <bool F16>
__global__ void __launch_bounds__(WD_RED_THREADS) k_batch_xpay(const BVec *v, const int *chunk_sys, const BScal *sc)
{
    const int c = blockIdx.x;
    const int sys = chunk_sys[c];
    if (!sc[sys].active) return;
    const BVec &B = v[sys];
    const float be = sc[sys].beta;
    const int s0 = (c - B.chunk0) * kChunk;
    const int s1 = min(s0 + kChunk, B.Vh);
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        float2 pv[12], rv[12];
        SpF32{B.rs, B.Vh}.load(s, rv);
        BSp<F16>::make(B.p, B.p_scale, B.Vh).load(s, pv);
#pragma unroll
        for (int k = 0; k < 12; ++k) pv[k] = make_float2(fmaf(be, pv[k].x, rv[k].x), fmaf(be, pv[k].y, rv[k].y));
        BSp<F16>::make(B.p, B.p_scale, B.Vh).store(s, pv);
    }
}

// One block per system folds its warp partials in a fixed order.
// mode 0 (|t|^2): alpha = rr / tt.
// mode 1 (|r_s|^2 after the update): the reliable-update rule -- mask the
// system and flag it when |r_s|^2 < delta2 rr_max or <= target2, else
// beta = rr_new / rr, rr = rr_new.
constexpr int kScalThreads = 128;
__global__ void __launch_bounds__(kScalThreads) k_batch_scalars(const BSys *sys_tab, BScal *sc, const double *partial,
                                                                int mode, double delta2)
{
    const int sys = blockIdx.x;
    if (!sc[sys].active) return;  // the whole block
    const BSys &S = sys_tab[sys];
    double v = 0.0;
    for (int i = threadIdx.x; i < S.nparts; i += kScalThreads) v += partial[S.part0 + i];
    v = wd_warp_sum(v);
    __shared__ double sw[kScalThreads / 32];
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x != 0) return;
    v = 0.0;
#pragma unroll
    for (int w = 0; w < kScalThreads / 32; ++w) v += sw[w];
    BScal &c = sc[sys];
    if (mode == 0) {
        c.tt = v;
        if (!(v > 0.0) || !isfinite(v)) {
            c.wait = 2;
            c.active = 0;
            return;
        }
        c.alpha = (float)(c.rr / v);
        return;
    }
    c.rr_new = v;
    c.iters += 1;
    if (!isfinite(v)) {
        c.wait = 2;
        c.active = 0;
    } else if (v < delta2 * c.rr_max || v <= c.target2) {
        c.wait = 1;
        c.active = 0;
    } else {
        c.beta = (float)(v / c.rr);
        c.rr = v;
    }
}

}  // namespace

// ====================================================== the batch engine
//
// BatchEngine keeps a changing set of systems iterating together.  Systems
// are added with add() (set-up and the first reliable update run at once)
// and step() advances every active system by one captured graph of K
// iterations.  The iterations run entirely on per-system device scalars
// (BScal): the hop forming t = Mhat p reduces |t|^2, the hop forming
// q = Mhat^dag t applies the CG update in place of storing q, and the
// scalar kernels set alpha and beta and mask a system the moment its
// residual calls for a reliable update, so K need not match any system's
// cycle.  After the graph the host reads the scalars once, runs the due
// reliable updates (their results land in a device array read with one more
// wait), retires converged systems (writes the FP64 solution and frees their
// buffers) and re-arms the rest.  K is the shortest expected remaining cycle
// (the previous cycle's length) of the iterating systems, at most
// kMaxPerGraph.  Retired systems are masked; the tables and graphs are
// rebuilt (compacted) when systems join or when masked systems make up half
// of the tables.

namespace {

struct SysBufs {
    WdVecBuf p, t, tmp_o, rs, xs;       // kernel storage / FP32
    WdVecBuf hs, hx, bhat, r_h, tmp_oh;  // high precision
    WdVecBuf rel;                        // reliable-update reduction scratch (doubles)
    void release()
    {
        for (WdVecBuf *b : {&p, &t, &tmp_o, &rs, &xs, &hs, &hx, &bhat, &r_h, &tmp_oh, &rel}) b->release();
    }
};

template <class T>
struct DevArray {
    T *p = nullptr;
    size_t n = 0;
    wd_context *ctx = nullptr;
    DevArray() = default;
    DevArray(const DevArray &) = delete;
    DevArray &operator=(const DevArray &) = delete;
    ~DevArray() { release(); }
    void release()
    {
        if (ctx) wd_dev_free(ctx, p);
        p = nullptr;
        n = 0;
        ctx = nullptr;
    }
    wd_status reserve(wd_context *c, size_t count)
    {
        if (count > n) {
            release();
            ctx = c;
            n = count;
            return wd_dev_alloc(c, (void **)&p, n * sizeof(T));
        }
        return WD_OK;
    }
    wd_status put(wd_context *c, const std::vector<T> &h)
    {
        wd_status st = reserve(c, h.size());
        if (st != WD_OK) return st;
        if (!h.empty())
            WD_CUDA(c, cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
        return WD_OK;
    }
};

struct EngineSys {
    int tag;
    const wd_lattice *lat;
    double mass, tol;
    const double2 *src;  // FP64 source (device, caller-owned)
    double2 *dest;       // FP64 solution (device, caller-owned)
    SysBufs B;
    double norm_b = 1, rr = 0, rr_max = 0, target = 0, ratio = 1, true_res = 1;
    int updates = 0, iters = 0;
    int since = 0, cycle = 4;  // iterations since the last reliable update; length of the previous cycle
    bool active = true;
};

// device bytes of one system's work buffers
size_t system_bytes(const wd_lattice *lat, wd_precision L, wd_precision H)
{
    const size_t nh = (size_t)12 * lat->g.Vh;
    size_t lbytes = nh * wd_entry_bytes(L) + (L == WD_PREC_F16 ? (size_t)lat->g.Vh * 4 : 0);
    return 3 * lbytes + 2 * nh * 8 + 3 * nh * wd_entry_bytes(H) + 2 * 2 * nh * wd_entry_bytes(H);
}

class BatchEngine {
  public:
    BatchEngine(wd_context *ctx, wd_precision L, wd_precision H, double delta, int max_iter)
        : ctx_(ctx), L_(L), H_(H), delta_(delta), max_iter_(max_iter)
    {
    }
    ~BatchEngine()
    {
        drop_graphs();
        for (auto &e : rel_ev_)
            if (e) cudaEventDestroy(e);
        for (auto &q : rel_stream_)
            if (q) cudaStreamDestroy(q);
    }

    size_t active() const
    {
        size_t n = 0;
        for (auto &s : sys_) n += s->active;
        return n;
    }
    bool idle() const { return active() == 0; }
    std::map<int, wd_solver_stats> results;  // tag -> stats of retired systems
    double solve_seconds = 0;                // time spent in step() and add()

    wd_status add(int tag, const wd_lattice *lat, const double2 *src, double2 *dest, double mass, double tol);
    // finished (optional) receives the tags retired since the previous call
    wd_status step(std::vector<int> *finished);
    void take_retired(std::vector<int> *out)
    {
        out->insert(out->end(), retired_.begin(), retired_.end());
        retired_.clear();
    }

  private:
    wd_context *ctx_;
    wd_precision L_, H_;
    double delta_;
    int max_iter_;
    std::vector<std::unique_ptr<EngineSys>> sys_;
    std::vector<int> retired_;
    bool rebuild_ = true, scalars_dirty_ = false;
    // device tables
    DevArray<BGroup> d_groups_;
    DevArray<BSys> d_sys_[4];
    DevArray<float> d_alpha_[4], d_beta_[4];
    DevArray<BVec> d_vec_;
    DevArray<BScal> d_sc_;
    DevArray<double> d_partial_, d_rel_;
    DevArray<int> d_chunk_sys_;
    std::vector<BScal> h_sc_;
    int grid_x_ = 0, nchunks_ = 0, ngroups_ = 0, max_group_sys_ = 1;
    int hop_variant_ = 0;  // launch shape of the batched hop (tuned in rebuild)
    std::map<int, cudaGraphExec_t> graphs_;  // K -> K captured iterations
    uint64_t kernels_per_iter_ = 0;
    // reliable updates due at the same step run on up to kRelStreams streams
    // at once (small lattices alone cannot fill the GPU)
    static constexpr int kRelStreams = 8;
    cudaStream_t rel_stream_[kRelStreams] = {};
    cudaEvent_t rel_ev_[kRelStreams + 1] = {};
    wd_status rel_streams();
    wd_status reliable_round(const std::vector<int> &upd);

    void drop_graphs()
    {
        for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
        graphs_.clear();
    }
    wd_status reliable(EngineSys &s, bool reset_p, double *rr, double *ss);
    wd_status reliable_enqueue(EngineSys &s, bool reset_p, double *rr_dev, double *ss_dev);
    wd_status finish(EngineSys &s);
    wd_status rebuild();
    wd_status graph(int k, cudaGraphExec_t *exec);
    wd_status iteration();
    wd_status hop(int h, int cb, int dag, int variant, int epi);
    wd_status upload_scalars();
};

static inline void slices(EngineSys &s, WdVec &b_e, WdVec &b_o, WdVec &x_e, WdVec &x_o)
{
    const int Vh = s.lat->g.Vh;
    b_e = s.B.hs.v;
    b_o = wd_offset(s.B.hs.v, (int64_t)12 * Vh, Vh);
    x_e = s.B.hx.v;
    x_o = wd_offset(s.B.hx.v, (int64_t)12 * Vh, Vh);
}

// reliable update: x_e += x_s; s = bhat - Mhat x_e; r_s = Mhat^dag s (FP32); p <- r_s on a restart
wd_status BatchEngine::reliable(EngineSys &s, bool reset_p, double *rr, double *ss)
{
    double2 *res = (double2 *)ctx_->red_partial + WD_RED_BLOCKS;
    wd_status e = reliable_enqueue(s, reset_p, &res[0].x, &res[1].x);
    if (e != WD_OK) return e;
    double2 red[2];
    if ((e = wd_red_fetch(ctx_, 2, red)) != WD_OK) return e;
    *rr = red[0].x;
    *ss = red[1].x;
    return WD_OK;
}

wd_status BatchEngine::reliable_enqueue(EngineSys &s, bool reset_p, double *rr_dev, double *ss_dev)
{
    SysBufs &B = s.B;
    WdVec b_e, b_o, x_e, x_o;
    slices(s, b_e, b_o, x_e, x_o);
    const WdMxReliable rv{B.xs.v, x_e, B.bhat.v, B.tmp_oh.v, B.r_h.v, B.rs.v};
    return wd_mx_reliable_enqueue(ctx_, s.lat, s.mass, L_, H_, rv, reset_p ? &B.p.v : nullptr, rr_dev, ss_dev,
                                  (double *)B.rel.v.p);
}

wd_status BatchEngine::add(int tag, const wd_lattice *lat, const double2 *src, double2 *dest, double mass,
                           double tol)
{
    const auto t0 = std::chrono::steady_clock::now();
    auto sp = std::make_unique<EngineSys>();
    EngineSys &s = *sp;
    s.tag = tag, s.lat = lat, s.mass = mass, s.tol = tol, s.src = src, s.dest = dest;
    const int Vh = lat->g.Vh;
    const int64_t nh = (int64_t)12 * Vh;
    const double a = 4.0 + mass;
    SysBufs &B = s.B;
    wd_status st;
    for (WdVecBuf *b : {&B.p, &B.t, &B.tmp_o})
        if ((st = wd_vec_alloc(ctx_, *b, L_, nh)) != WD_OK) return st;
    for (WdVecBuf *b : {&B.rs, &B.xs})
        if ((st = wd_vec_alloc(ctx_, *b, WD_PREC_F32, nh)) != WD_OK) return st;
    for (WdVecBuf *b : {&B.bhat, &B.r_h, &B.tmp_oh})
        if ((st = wd_vec_alloc(ctx_, *b, H_, nh)) != WD_OK) return st;
    for (WdVecBuf *b : {&B.hs, &B.hx})
        if ((st = wd_vec_alloc(ctx_, *b, H_, 2 * nh)) != WD_OK) return st;
    if ((st = wd_vec_alloc(ctx_, B.rel, WD_PREC_F64, (int64_t)(wd_mx_reliable_scratch_doubles(Vh) + 1) / 2)) != WD_OK)
        return st;
    if ((st = wd_lattice_gauge_lp(ctx_, lat, L_)) != WD_OK) return st;
    if (H_ == WD_PREC_DF64) {
        if ((st = wd_convert_f64_to_df(ctx_, src, (float4 *)B.hs.v.p, 2 * nh)) != WD_OK) return st;
    } else {
        WD_CUDA(ctx_, cudaMemcpyAsync(B.hs.v.p, src, 2 * nh * sizeof(double2), cudaMemcpyDeviceToDevice, ctx_->stream));
    }
    WdVec b_e, b_o, x_e, x_o;
    slices(s, b_e, b_o, x_e, x_o);
    if ((st = wd_hop_v(ctx_, lat, b_o, B.bhat.v, &b_e, 0, 0, 0.5 / a, 1.0)) != WD_OK) return st;
    if ((st = wd_v_zero(ctx_, B.hx.v, 2 * nh)) != WD_OK) return st;
    if ((st = wd_v_zero(ctx_, B.xs.v, nh)) != WD_OK) return st;
    if ((st = wd_red_norm2(ctx_, src, 2 * nh, 0)) != WD_OK) return st;
    double2 v;
    if ((st = wd_red_fetch(ctx_, 1, &v)) != WD_OK) return st;
    s.norm_b = v.x > 0 ? std::sqrt(v.x) : 1.0;
    double rr, ss;
    if ((st = reliable(s, true, &rr, &ss)) != WD_OK) return st;
    s.true_res = std::sqrt(ss) / s.norm_b;
    s.ratio = ss > 0 ? std::sqrt(rr / ss) : 1.0;
    s.target = tol * s.norm_b * s.ratio * 0.5;
    s.rr = s.rr_max = rr;
    sys_.push_back(std::move(sp));
    rebuild_ = true;
    solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (s.true_res <= tol) return finish(s);  // already solved (e.g. zero source)
    return WD_OK;
}

// fold x_s, reconstruct x_o, write the FP64 solution, record stats, free buffers
wd_status BatchEngine::finish(EngineSys &s)
{
    const int Vh = s.lat->g.Vh;
    const int64_t nh = (int64_t)12 * Vh;
    const double a = 4.0 + s.mass;
    WdVec b_e, b_o, x_e, x_o;
    slices(s, b_e, b_o, x_e, x_o);
    wd_status st;
    const bool converged = s.true_res <= s.tol;
    if ((st = wd_mx_accum(ctx_, Vh, H_, s.B.xs.v, x_e)) != WD_OK) return st;
    if ((st = wd_hop_v(ctx_, s.lat, x_e, x_o, &b_o, 1, 0, 0.5 / a, 1.0 / a)) != WD_OK) return st;
    if (H_ == WD_PREC_DF64) {
        if ((st = wd_convert_df_to_f64(ctx_, (const float4 *)s.B.hx.v.p, s.dest, 2 * nh)) != WD_OK) return st;
    } else {
        WD_CUDA(ctx_, cudaMemcpyAsync(s.dest, s.B.hx.v.p, 2 * nh * sizeof(double2), cudaMemcpyDeviceToDevice,
                                      ctx_->stream));
    }
    wd_solver_stats r{};
    r.iterations = s.iters;
    r.reliable_updates = s.updates;
    r.residual = s.true_res;
    r.converged = converged;
    results[s.tag] = r;
    retired_.push_back(s.tag);
    s.active = false;
    s.B.release();  // buffers back to the pool
    scalars_dirty_ = true;
    return WD_OK;
}

wd_status BatchEngine::rebuild()
{
    drop_graphs();
    // drop retired systems, group by lattice (stable)
    std::vector<std::unique_ptr<EngineSys>> keep;
    for (auto &s : sys_)
        if (s->active) keep.push_back(std::move(s));
    std::stable_sort(keep.begin(), keep.end(),
                     [](const std::unique_ptr<EngineSys> &x, const std::unique_ptr<EngineSys> &y) {
                         return x->lat < y->lat;
                     });
    sys_ = std::move(keep);
    const int nsys = (int)sys_.size();
    rebuild_ = false;
    scalars_dirty_ = false;
    if (nsys == 0) return WD_OK;
    const bool f16 = L_ == WD_PREC_F16;
    std::vector<BGroup> groups;
    std::vector<int> sys_group(nsys);
    int blocks = 0;
    for (int k = 0; k < nsys; ++k) {
        if (k == 0 || sys_[k]->lat != sys_[k - 1]->lat) {
            BGroup G{};
            G.g = sys_[k]->lat->g;
            G.gauge = f16 ? sys_[k]->lat->gauge_h12 : sys_[k]->lat->gauge_f32;
            G.first_sys = k;
            G.nsys = 0;
            G.block_start = blocks;
            blocks += (G.g.Vh + kSites - 1) / kSites;
            groups.push_back(G);
        }
        groups.back().nsys++;
        sys_group[k] = (int)groups.size() - 1;
    }
    grid_x_ = blocks;
    max_group_sys_ = 1;
    for (const BGroup &G : groups) max_group_sys_ = std::max(max_group_sys_, G.nsys);
    ngroups_ = (int)groups.size();
    std::vector<BVec> bvec(nsys);
    std::vector<int> chunk_sys;
    std::vector<int> part0(nsys), nparts(nsys);
    int parts = 0;
    for (int k = 0; k < nsys; ++k) {
        SysBufs &B = sys_[k]->B;
        BVec &v = bvec[k];
        v.p = B.p.v.p, v.p_scale = B.p.v.scale;
        v.rs = (float4 *)B.rs.v.p;
        v.Vh = sys_[k]->lat->g.Vh;
        v.chunk0 = (int)chunk_sys.size();
        for (int c = 0; c < (v.Vh + kChunk - 1) / kChunk; ++c) chunk_sys.push_back(k);
        part0[k] = parts;
        nparts[k] = (v.Vh + kSites - 1) / kSites;
        parts += nparts[k];
    }
    nchunks_ = (int)chunk_sys.size();
    wd_status st;
    if ((st = d_groups_.put(ctx_, groups)) != WD_OK) return st;
    for (int h = 0; h < 4; ++h) {
        std::vector<BSys> tab(nsys);
        std::vector<float> al(nsys), be(nsys);
        for (int k = 0; k < nsys; ++k) {
            const double a = 4.0 + sys_[k]->mass;
            const SysBufs &B = sys_[k]->B;
            // h = 0: p -> tmp_o (cb 1); 1: tmp_o -> t with x = p (cb 0); 2: t -> tmp_o; 3: tmp_o -> (update) with x = t
            const WdVec *vin[4] = {&B.p.v, &B.tmp_o.v, &B.t.v, &B.tmp_o.v};
            const WdVec *vout[4] = {&B.tmp_o.v, &B.t.v, &B.tmp_o.v, &B.t.v};
            const WdVec *vx[4] = {nullptr, &B.p.v, nullptr, &B.t.v};
            BSys &S = tab[k];
            S = BSys{vin[h]->p, vout[h]->p, vx[h] ? vx[h]->p : nullptr, vin[h]->scale, vout[h]->scale,
                     vx[h] ? vx[h]->scale : nullptr, B.p.v.p, B.p.v.scale, (float4 *)B.rs.v.p, (float4 *)B.xs.v.p,
                     part0[k], nparts[k]};
            al[k] = (h % 2 == 0) ? 1.0f : (float)(-0.25 / a);
            be[k] = (h % 2 == 0) ? 0.0f : (float)a;
        }
        if ((st = d_sys_[h].put(ctx_, tab)) != WD_OK) return st;
        if ((st = d_alpha_[h].put(ctx_, al)) != WD_OK) return st;
        if ((st = d_beta_[h].put(ctx_, be)) != WD_OK) return st;
    }
    if ((st = d_vec_.put(ctx_, bvec)) != WD_OK) return st;
    if ((st = d_chunk_sys_.put(ctx_, chunk_sys)) != WD_OK) return st;
    if ((st = d_partial_.reserve(ctx_, parts)) != WD_OK) return st;
    if ((st = d_rel_.reserve(ctx_, 2 * (size_t)nsys)) != WD_OK) return st;
    if ((st = upload_scalars()) != WD_OK) return st;

    // launch shape of the batched hop, timed on its first operator (p -> the
    // odd scratch, which every iteration rewrites before reading) outside the
    // capture; keyed by precision and the batch's system-sites to a power of 2
    int64_t sites = 0;
    for (const BGroup &G : groups) sites += (int64_t)G.g.Vh * G.nsys;
    int bucket = 1;
    while ((int64_t)bucket < sites && bucket < (1 << 30)) bucket <<= 1;
    return wd_tune_launch(ctx_, f16 ? "batch_hop_f16" : "batch_hop_f32", bucket, kBatchHopVariants,
                          [&](int v) -> wd_status {
                              hop_variant_ = v;
                              return hop(0, 1, 0, v, kBEpiPlain);
                          });
}

// k captured iterations (built on first use after each rebuild)
wd_status BatchEngine::graph(int k, cudaGraphExec_t *exec)
{
    auto it = graphs_.find(k);
    if (it != graphs_.end()) {
        *exec = it->second;
        return WD_OK;
    }
    const uint64_t before = ctx_->launches;
    cudaGraph_t g = nullptr;
    WD_CUDA(ctx_, cudaStreamSynchronize(ctx_->stream));
    WD_CUDA(ctx_, cudaStreamBeginCapture(ctx_->stream, cudaStreamCaptureModeThreadLocal));
    wd_status cap = WD_OK;
    for (int i = 0; i < k && cap == WD_OK; ++i) cap = iteration();
    const cudaError_t ce = cudaStreamEndCapture(ctx_->stream, &g);
    kernels_per_iter_ = (ctx_->launches - before) / (uint64_t)k;
    ctx_->launches = before;  // counted per replay
    if (cap != WD_OK) {
        if (g) cudaGraphDestroy(g);
        return cap;
    }
    if (ce != cudaSuccess) return wd_cuda_check(ctx_, ce, "cudaStreamEndCapture");
    cudaGraphExec_t e = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&e, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return wd_cuda_check(ctx_, ie, "cudaGraphInstantiate");
    graphs_[k] = e;
    *exec = e;
    return WD_OK;
}

// batched hop h (operand table h) with launch variant v and epilogue epi:
// (systems per block, min blocks per SM) = (8, none), (8, 3), (4, 6), (2, 12),
// (4, none), (4, 8), (4, 8) with the shared row-2 table.  A whole 24-source solve at 24^3x48 before the epilogue
// fusion (GB300, seconds): FP32 inner 0.298 / 0.270 / 0.265 / 0.268 / 0.274,
// FP16 inner 0.263 / 0.247 / 0.244 / 0.245 / 0.256.  The last, registers
// capped at 64 for 32 warps per SM (a few spilled registers; the kernel is
// bound by L2 latency, so more warps in flight pay): the plain hop at
// 24 x 24^3x48 0.604 ms (FP32) / 0.450 ms (FP16) against 0.632 / 0.498 for
// (4, 6) (the tuner's timings), the tuner's choice at every batch size
// measured, and whole batched solves 1-4 % faster.  Variant 6, FP16 links:
// (4, 8) with row 2 of the block's links rebuilt once per site and direction
// into shared memory and read by all four systems (k_batch_hop's R2): 0.437
// against 0.450 ms, the tuner's choice from 24 x 16^3x32 systems up (for
// FP32 links variant 6 is variant 5's launch).  Dropped: (8, 4) at 64
// registers (0.610 / 0.456 ms);
// the hop with each thread's operands staged in shared memory by cp.async,
// with 4 or 2 systems per block (FP32 0.276 / 0.279, FP16 0.243 / 0.243 s: no
// gain; the block's systems already share links through L1).
wd_status BatchEngine::hop(int h, int cb, int dag, int v, int epi)
{
    const BTable t{d_groups_.p, ngroups_, d_sys_[h].p, d_alpha_[h].p, d_beta_[h].p, d_sc_.p, d_partial_.p, cb};
    auto run = [&](auto sys, auto minb, auto share) -> wd_status {
        constexpr int S = decltype(sys)::value, M = decltype(minb)::value;
        const dim3 grid(grid_x_, (max_group_sys_ + S - 1) / S);
        auto go = [&](auto f16, auto e) {
            constexpr bool F = decltype(f16)::value;
            constexpr int E = decltype(e)::value;
            constexpr bool R = F && decltype(share)::value;  // the shared row-2 table: FP16 links only
            if (dag) k_batch_hop<true, F, S, M, E, R><<<grid, kSites * S, 0, ctx_->stream>>>(t);
            else k_batch_hop<false, F, S, M, E, R><<<grid, kSites * S, 0, ctx_->stream>>>(t);
        };
        using E0 = std::integral_constant<int, kBEpiPlain>;
        using E1 = std::integral_constant<int, kBEpiNorm>;
        using E2 = std::integral_constant<int, kBEpiUpdate>;
        if (L_ == WD_PREC_F16) {
            if (epi == kBEpiNorm) go(std::true_type(), E1());
            else if (epi == kBEpiUpdate) go(std::true_type(), E2());
            else go(std::true_type(), E0());
        } else {
            if (epi == kBEpiNorm) go(std::false_type(), E1());
            else if (epi == kBEpiUpdate) go(std::false_type(), E2());
            else go(std::false_type(), E0());
        }
        WD_LAUNCHED(ctx_);
        return WD_OK;
    };
    using I2 = std::integral_constant<int, 2>;
    using I4 = std::integral_constant<int, 4>;
    using I8 = std::integral_constant<int, 8>;
    using I0 = std::integral_constant<int, 0>;
    using N = std::false_type;
    switch (v) {
    case 1: return run(I8(), std::integral_constant<int, 3>(), N());
    case 2: return run(I4(), std::integral_constant<int, 6>(), N());
    case 3: return run(I2(), std::integral_constant<int, 12>(), N());
    case 4: return run(I4(), I0(), N());
    case 5: return run(I4(), std::integral_constant<int, 8>(), N());
    case 6: return run(I4(), std::integral_constant<int, 8>(), std::true_type());
    default: return run(I8(), I0(), N());
    }
}

wd_status BatchEngine::iteration()
{
    const int nsys = (int)sys_.size();
    const bool f16 = L_ == WD_PREC_F16;
    const int v = hop_variant_;
    wd_status e;
    // t = Mhat p with |t|^2 -> alpha
    if ((e = hop(0, 1, 0, v, kBEpiPlain)) != WD_OK || (e = hop(1, 0, 0, v, kBEpiNorm)) != WD_OK) return e;
    k_batch_scalars<<<nsys, kScalThreads, 0, ctx_->stream>>>(d_sys_[1].p, d_sc_.p, d_partial_.p, 0, 0.0);
    WD_LAUNCHED(ctx_);
    // q = Mhat^dag t applied as the update, |r_s|^2 -> beta (or a reliable update due)
    if ((e = hop(2, 1, 1, v, kBEpiPlain)) != WD_OK || (e = hop(3, 0, 1, v, kBEpiUpdate)) != WD_OK) return e;
    k_batch_scalars<<<nsys, kScalThreads, 0, ctx_->stream>>>(d_sys_[3].p, d_sc_.p, d_partial_.p, 1, delta_ * delta_);
    WD_LAUNCHED(ctx_);
    if (f16) k_batch_xpay<true><<<nchunks_, WD_RED_THREADS, 0, ctx_->stream>>>(d_vec_.p, d_chunk_sys_.p, d_sc_.p);
    else k_batch_xpay<false><<<nchunks_, WD_RED_THREADS, 0, ctx_->stream>>>(d_vec_.p, d_chunk_sys_.p, d_sc_.p);
    WD_LAUNCHED(ctx_);
    return WD_OK;
}

wd_status BatchEngine::rel_streams()
{
    if (rel_stream_[0]) return WD_OK;
    for (auto &q : rel_stream_) WD_CUDA(ctx_, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    for (auto &e : rel_ev_) WD_CUDA(ctx_, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return WD_OK;
}

// the reliable updates of systems upd, spread over the update streams
// (each system's kernels in order on one stream, with its own reduction
// scratch), joined back into the context's stream
wd_status BatchEngine::reliable_round(const std::vector<int> &upd)
{
    const int ns = std::min<int>(kRelStreams, (int)upd.size());
    if (ns <= 1) {
        for (int j : upd)
            if (wd_status st = reliable_enqueue(*sys_[j], false, d_rel_.p + 2 * j, d_rel_.p + 2 * j + 1))
                return st;
        return WD_OK;
    }
    wd_status st = rel_streams();
    if (st != WD_OK) return st;
    cudaStream_t main = ctx_->stream;
    WD_CUDA(ctx_, cudaEventRecord(rel_ev_[kRelStreams], main));
    for (int i = 0; i < ns; ++i) WD_CUDA(ctx_, cudaStreamWaitEvent(rel_stream_[i], rel_ev_[kRelStreams], 0));
    for (size_t u = 0; u < upd.size() && st == WD_OK; ++u) {
        const int j = upd[u];
        ctx_->stream = rel_stream_[u % ns];  // every launch of this system's update goes to its stream
        st = reliable_enqueue(*sys_[j], false, d_rel_.p + 2 * j, d_rel_.p + 2 * j + 1);
        ctx_->stream = main;
    }
    // join every stream that was given work, also after an error
    for (int i = 0; i < ns; ++i) {
        cudaEventRecord(rel_ev_[i], rel_stream_[i]);
        cudaStreamWaitEvent(main, rel_ev_[i], 0);
    }
    return st;
}

wd_status BatchEngine::upload_scalars()
{
    const int nsys = (int)sys_.size();
    h_sc_.assign(nsys, BScal{});
    for (int k = 0; k < nsys; ++k) {
        const EngineSys &s = *sys_[k];
        BScal &c = h_sc_[k];
        c.rr = s.rr;
        c.rr_max = s.rr_max;
        c.target2 = s.target * s.target;
        c.active = s.active ? 1 : 0;
        c.wait = 0;
        c.iters = s.iters;
    }
    scalars_dirty_ = false;
    return d_sc_.put(ctx_, h_sc_);
}

wd_status BatchEngine::step(std::vector<int> *finished)
{
    const auto t0 = std::chrono::steady_clock::now();
    wd_status st;
    // compact when systems joined or half the tables are masked
    size_t masked = 0;
    for (auto &s : sys_) masked += !s->active;
    if (rebuild_ || (masked > 0 && 2 * masked >= sys_.size())) {
        if ((st = rebuild()) != WD_OK) return st;
    } else if (scalars_dirty_) {
        if ((st = upload_scalars()) != WD_OK) return st;
    }
    const int nsys = (int)sys_.size();
    if (nsys == 0) return WD_OK;
    // iterations to queue: the shortest expected remainder of a cycle
    int k = kMaxPerGraph;
    for (auto &s : sys_)
        if (s->active) k = std::min(k, std::max(1, std::min(s->cycle - s->since, max_iter_ - s->iters)));
    cudaGraphExec_t exec = nullptr;
    if ((st = graph(k, &exec)) != WD_OK) return st;
    WD_CUDA(ctx_, cudaGraphLaunch(exec, ctx_->stream));
    ctx_->launches += kernels_per_iter_ * (uint64_t)k;
    h_sc_.resize(nsys);
    WD_CUDA(ctx_, cudaMemcpyAsync(h_sc_.data(), d_sc_.p, nsys * sizeof(BScal), cudaMemcpyDeviceToHost, ctx_->stream));
    WD_CUDA(ctx_, cudaStreamSynchronize(ctx_->stream));
    // systems the device masked for a reliable update take it now, all
    // enqueued back to back with one host wait for their norms
    std::vector<int> upd;
    std::vector<double> rr_old(nsys), rr_trig(nsys);
    for (int j = 0; j < nsys; ++j) {
        EngineSys &s = *sys_[j];
        if (!s.active) continue;
        const BScal &c = h_sc_[j];
        s.since += c.iters - s.iters;
        s.iters = c.iters;
        if (c.wait == 2) return wd_fail(ctx_, WD_ERR_NAN, "batched CG residual is not finite");
        if (c.wait == 0) s.rr = c.rr;  // the device's current iterate
        if (c.wait == 1) {
            upd.push_back(j);
            rr_old[j] = c.rr;
            rr_trig[j] = c.rr_new;
        } else if (s.iters >= max_iter_) {
            if ((st = finish(s)) != WD_OK) return st;  // give up: return what it has
        }
    }
    if (!upd.empty()) {
        if ((st = reliable_round(upd)) != WD_OK) return st;
        std::vector<double> rel(2 * (size_t)nsys);
        WD_CUDA(ctx_, cudaMemcpyAsync(rel.data(), d_rel_.p, rel.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                      ctx_->stream));
        WD_CUDA(ctx_, cudaStreamSynchronize(ctx_->stream));
        for (int j : upd) {
            EngineSys &s = *sys_[j];
            const double rrt = rel[2 * j], ss = rel[2 * j + 1];
            s.updates++;
            s.cycle = std::max(1, s.since);
            s.since = 0;
            s.true_res = std::sqrt(ss) / s.norm_b;
            if (s.true_res <= s.tol) {
                if ((st = finish(s)) != WD_OK) return st;
                continue;
            }
            if (std::sqrt(rr_trig[j]) <= s.target) {
                s.ratio = ss > 0 ? std::sqrt(rrt / ss) : s.ratio;
                s.target = std::fmin(s.target * 0.5, s.tol * s.norm_b * s.ratio * 0.5);
            }
            // continue from the recomputed residual: p = r_s + (|r_s|^2 / previous |r_s|^2) p
            if ((st = wd_mx_xpay(ctx_, s.lat->g.Vh, L_, s.B.rs.v, rrt / rr_old[j], s.B.p.v)) != WD_OK) return st;
            s.rr = s.rr_max = rrt;
            if (s.iters >= max_iter_ && (st = finish(s)) != WD_OK) return st;
        }
        scalars_dirty_ = true;
    }
    WD_CUDA(ctx_, cudaStreamSynchronize(ctx_->stream));
    solve_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (finished) {
        finished->clear();
        take_retired(finished);
    }
    return WD_OK;
}

}  // namespace

// ==================================================== one batch, all systems
extern "C" wd_status wd_solve_batch(wd_context *ctx, int nsys, const wd_lattice *const *lats,
                                    const wd_field *const *srcs, wd_field *const *dests, const double *masses,
                                    const wd_solver_params *prm, wd_solver_stats *stats)
{
    if (!ctx || nsys <= 0 || !lats || !srcs || !dests || !masses || !prm)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (prm->prec != WD_PREC_F32 && prm->prec != WD_PREC_F16)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "batched solves run a mixed FP32 or FP16 inner solver");
    if (prm->max_iter < 1 || !(prm->tol > 0)) return wd_fail(ctx, WD_ERR_BAD_ARG, "bad tolerance or max_iter");
    for (int i = 0; i < nsys; ++i) {
        if (!lats[i] || !srcs[i] || !dests[i]) return wd_fail(ctx, WD_ERR_BAD_ARG, "null system");
        if (srcs[i]->storage != WD_PREC_F64 || dests[i]->storage != WD_PREC_F64 ||
            srcs[i]->lat->volume != lats[i]->volume || dests[i]->lat->volume != lats[i]->volume)
            return wd_fail(ctx, WD_ERR_BAD_ARG, "batch fields must be FP64 fields of their system's lattice");
    }
    const wd_precision H = prm->prec_reliable == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
    const double delta = prm->delta > 0 && prm->delta < 1 ? prm->delta : 0.1;
    BatchEngine eng(ctx, prm->prec, H, delta, prm->max_iter);
    wd_status st;
    for (int i = 0; i < nsys; ++i)
        if ((st = eng.add(i, lats[i], srcs[i]->d, dests[i]->d, masses[i], prm->tol)) != WD_OK) return st;
    while (!eng.idle())
        if ((st = eng.step(nullptr)) != WD_OK) return st;
    const double secs = eng.solve_seconds;
    bool all = true;
    for (int i = 0; i < nsys; ++i) {
        wd_solver_stats s = eng.results[i];
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
        all = all && s.converged;
    }
    return all ? WD_OK : WD_ERR_NOT_CONVERGED;
}

// ================================================================ serving
//
// A request: nsrc right-hand sides on one resident lattice, one mass and
// tolerance.  Requests queue on submit; step() admits queued requests in
// arrival order while the HBM budget (links + every admitted request's
// fields and work buffers) and the slot count allow, advances all admitted
// systems together by one engine quantum, and retires finished systems.
// Requests admitted later join the running batch at the next quantum, so
// work of different requests overlaps on the device.  In FP64 mode (the
// plain drop-in), step() instead solves the oldest admitted system to the
// end with the FP64 even-odd CG.

namespace {
uint64_t gen_mix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ uint64_t dev_mix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// complex Gaussian entry for reference index i (the host generator's counter
// scheme), written at its device (structure-of-arrays) position
__global__ void k_gen_source(uint64_t key, int Vh, double2 *out)
{
    const int64_t n = (int64_t)Vh * 24;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h1 = dev_mix(key ^ (uint64_t)(2 * i)), h2 = dev_mix(key ^ (uint64_t)(2 * i + 1));
        const double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double u2 = ((double)(h2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double r = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        const int64_t site = i / 12, c = i % 12;
        const int64_t par = site / Vh, s = site % Vh;
        out[(par * 12 + c) * Vh + s] = make_double2(r * cs, r * sn);
    }
}
}  // namespace

struct wd_server {
    wd_context *ctx = nullptr;
    wd_server_config cfg{};
    std::unique_ptr<BatchEngine> eng;
    std::vector<wd_lattice *> lats;
    double gauge_bytes = 0, req_bytes = 0;
    struct Pending {
        int64_t id;
        int lat, nsrc;
        std::vector<std::vector<double>> host;
        std::vector<uint64_t> seeds;
        double mass, tol;
    };
    std::deque<Pending> queue;
    struct Req {
        int lat = 0, nsrc = 0, remaining = 0;
        std::vector<wd_field *> src, dest;
        std::vector<wd_solver_stats> st;
        double bytes = 0, mass = 0, tol = 0;
        bool done = false;
        std::chrono::steady_clock::time_point t_submit, t_done;
    };
    std::map<int64_t, Req> reqs;
    std::map<int, std::pair<int64_t, int>> tag_req;
    std::deque<int> fp64_todo;  // FP64 mode: tags waiting for their solve
    int next_tag = 0, active_systems = 0;
    int64_t next_id = 1;
};

static double field_bytes64(const wd_lattice *lat) { return (double)lat->volume * 12 * sizeof(double2); }

static double request_bytes(const wd_server *sv, const wd_lattice *lat, int nsrc)
{
    double per = 2 * field_bytes64(lat);
    if (sv->cfg.prec == WD_PREC_F64) per += 8 * 0.5 * field_bytes64(lat);  // the FP64 CG's half-lattice vectors
    else per += (double)system_bytes(lat, sv->cfg.prec, sv->cfg.prec_reliable == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64);
    return per * nsrc;
}

extern "C" void wd_server_config_default(wd_server_config *c)
{
    if (!c) return;
    c->prec = WD_PREC_F16;
    c->prec_reliable = WD_PREC_DF64;
    c->hbm_budget_bytes = 150e9;
    c->max_systems = 256;
    c->max_iter = 5000;
    c->delta = 0.1;
}

extern "C" wd_status wd_server_create(wd_context *ctx, const wd_server_config *cfg, wd_server **out)
{
    if (!ctx || !cfg || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (cfg->prec != WD_PREC_F64 && cfg->prec != WD_PREC_F32 && cfg->prec != WD_PREC_F16)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "server precision must be FP64 (plain) or FP32/FP16 (batched mixed)");
    if (!(cfg->hbm_budget_bytes > 0) || cfg->max_systems < 1 || cfg->max_iter < 1)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "bad server limits");
    wd_server *sv = new wd_server();
    sv->ctx = ctx;
    sv->cfg = *cfg;
    if (cfg->prec != WD_PREC_F64) {
        const wd_precision H = cfg->prec_reliable == WD_PREC_DF64 ? WD_PREC_DF64 : WD_PREC_F64;
        const double delta = cfg->delta > 0 && cfg->delta < 1 ? cfg->delta : 0.1;
        sv->eng = std::make_unique<BatchEngine>(ctx, cfg->prec, H, delta, cfg->max_iter);
    }
    *out = sv;
    return WD_OK;
}

extern "C" void wd_server_destroy(wd_server *sv)
{
    if (!sv) return;
    sv->eng.reset();
    for (auto &kv : sv->reqs) {
        for (wd_field *f : kv.second.src) wd_field_destroy(f);
        for (wd_field *f : kv.second.dest) wd_field_destroy(f);
    }
    for (wd_lattice *l : sv->lats) wd_lattice_destroy(l);
    delete sv;
}

extern "C" wd_status wd_server_add_lattice(wd_server *sv, const int dims[4], const double *const gauge[4], int *id)
{
    if (!sv || !id) return WD_ERR_BAD_ARG;
    wd_lattice *lat = nullptr;
    wd_status st = wd_lattice_create(sv->ctx, dims, gauge, &lat);
    if (st != WD_OK) return st;
    // derived link copies the server will use, built now so they count against the budget
    double bytes = (double)lat->volume * 4 * 9 * sizeof(double2);
    if (sv->cfg.prec != WD_PREC_F64) {
        st = wd_lattice_gauge_lp(sv->ctx, lat, sv->cfg.prec);
        bytes += (double)lat->volume * 4 * (sv->cfg.prec == WD_PREC_F16 ? 24 : 48);
        if (st == WD_OK && sv->cfg.prec == WD_PREC_F16) {  // reliable updates apply Mhat^dag with FP32 links
            st = wd_lattice_gauge_lp(sv->ctx, lat, WD_PREC_F32);
            bytes += (double)lat->volume * 4 * 48;
        }
        if (st == WD_OK && sv->cfg.prec_reliable == WD_PREC_DF64) {
            st = wd_lattice_gauge_df(sv->ctx, lat);
            bytes += (double)lat->volume * 4 * 9 * sizeof(float4);
        }
        if (st != WD_OK) {
            wd_lattice_destroy(lat);
            return st;
        }
    }
    sv->gauge_bytes += bytes;
    sv->lats.push_back(lat);
    *id = (int)sv->lats.size() - 1;
    return WD_OK;
}

extern "C" wd_status wd_server_submit(wd_server *sv, int lattice_id, int nsrc, const double *const *sources,
                                      const uint64_t *seeds, double mass, double tol, int64_t *id)
{
    if (!sv || !id || nsrc < 1 || lattice_id < 0 || lattice_id >= (int)sv->lats.size() || !(tol > 0))
        return sv ? wd_fail(sv->ctx, WD_ERR_BAD_ARG, "bad request") : WD_ERR_BAD_ARG;
    if (!sources && !seeds) return wd_fail(sv->ctx, WD_ERR_BAD_ARG, "a request needs sources or seeds");
    const wd_lattice *lat = sv->lats[lattice_id];
    if (sv->gauge_bytes + request_bytes(sv, lat, nsrc) > sv->cfg.hbm_budget_bytes || nsrc > sv->cfg.max_systems)
        return wd_fail(sv->ctx, WD_ERR_OOM, "request larger than the server's HBM budget or slot count");
    wd_server::Pending p;
    p.id = sv->next_id++;
    p.lat = lattice_id, p.nsrc = nsrc, p.mass = mass, p.tol = tol;
    const size_t n = (size_t)lat->volume * 24;
    for (int k = 0; k < nsrc; ++k) {
        if (sources) p.host.emplace_back(sources[k], sources[k] + n);
        else p.seeds.push_back(seeds[k]);
    }
    wd_server::Req r;
    r.lat = lattice_id, r.nsrc = nsrc, r.remaining = nsrc, r.mass = mass, r.tol = tol;
    r.st.resize(nsrc);
    r.t_submit = std::chrono::steady_clock::now();
    sv->reqs[p.id] = std::move(r);
    *id = p.id;
    sv->queue.push_back(std::move(p));
    return WD_OK;
}

// upload or generate one source into an FP64 field (unit L2 norm for generated ones)
static wd_status server_source(wd_server *sv, const wd_server::Pending &p, int k, wd_field *f)
{
    wd_context *ctx = sv->ctx;
    if (!p.host.empty()) return wd_field_upload(ctx, f, p.host[k].data());
    const int Vh = f->lat->g.Vh;
    k_gen_source<<<152 * 8, 256, 0, ctx->stream>>>(gen_mix(p.seeds[k] ^ 0xA5A5A5A5ull), Vh, f->d);
    WD_LAUNCHED(ctx);
    const int64_t n = f->lat->volume * 12;
    wd_status st = wd_red_norm2(ctx, f->d, n, 0);
    if (st != WD_OK) return st;
    double2 v;
    if ((st = wd_red_fetch(ctx, 1, &v)) != WD_OK) return st;
    return wd_blas_scale(ctx, v.x > 0 ? 1.0 / std::sqrt(v.x) : 1.0, f->d, f->d, n);
}

// systems k0.. of request r that could not be admitted complete as failed
// (not converged, no iterations), so the request still finishes
static void server_fail_from(wd_server::Req &r, int k0, int *completed)
{
    for (int k = k0; k < r.nsrc; ++k) r.st[k] = wd_solver_stats{};
    r.remaining -= r.nsrc - k0;
    if (r.remaining == 0) {
        r.done = true;
        r.t_done = std::chrono::steady_clock::now();
        for (wd_field *f : r.src) wd_field_destroy(f);
        r.src.clear();
        ++*completed;
    }
}

// Admits queued requests in order while the HBM budget and the slot count
// allow.  A request's fields and sources are created first, all or none; an
// allocation failure fails the whole request, a failure while handing its
// systems to the solver fails the systems not yet handed over.  Either way
// the request leaves the queue and the error is returned.
static wd_status server_admit(wd_server *sv, int *completed)
{
    while (!sv->queue.empty()) {
        wd_server::Pending &p = sv->queue.front();
        const wd_lattice *lat = sv->lats[p.lat];
        const double bytes = request_bytes(sv, lat, p.nsrc);
        if (sv->gauge_bytes + sv->req_bytes + bytes > sv->cfg.hbm_budget_bytes) break;
        if (sv->active_systems > 0 && sv->active_systems + p.nsrc > sv->cfg.max_systems) break;
        wd_server::Req &r = sv->reqs[p.id];
        wd_status st = WD_OK;
        for (int k = 0; k < p.nsrc && st == WD_OK; ++k) {
            wd_field *fs = nullptr, *fd = nullptr;
            st = wd_field_create(sv->ctx, lat, &fs);
            if (st == WD_OK) {
                r.src.push_back(fs);
                st = wd_field_create(sv->ctx, lat, &fd);
            }
            if (st == WD_OK) {
                r.dest.push_back(fd);
                st = server_source(sv, p, k, fs);
            }
        }
        if (st != WD_OK) {
            for (wd_field *f : r.dest) wd_field_destroy(f);
            r.dest.clear();
            server_fail_from(r, 0, completed);
            sv->queue.pop_front();
            return st;
        }
        r.bytes = bytes;
        sv->req_bytes += bytes;
        int k = 0;
        for (; k < p.nsrc; ++k) {
            const int tag = sv->next_tag++;
            if (sv->eng) st = sv->eng->add(tag, lat, r.src[k]->d, r.dest[k]->d, p.mass, p.tol);
            if (st != WD_OK) break;
            if (!sv->eng) sv->fp64_todo.push_back(tag);
            sv->tag_req[tag] = {p.id, k};
            sv->active_systems++;
        }
        sv->queue.pop_front();
        if (st != WD_OK) {
            server_fail_from(r, k, completed);
            return st;
        }
    }
    return WD_OK;
}

static void server_retire(wd_server *sv, int tag, const wd_solver_stats &s, int *completed)
{
    auto tr = sv->tag_req.find(tag);
    if (tr == sv->tag_req.end()) return;
    wd_server::Req &r = sv->reqs[tr->second.first];
    r.st[tr->second.second] = s;
    sv->tag_req.erase(tr);
    sv->active_systems--;
    if (--r.remaining == 0) {
        r.done = true;
        r.t_done = std::chrono::steady_clock::now();
        for (wd_field *f : r.src) wd_field_destroy(f);
        r.src.clear();
        ++*completed;
    }
}

extern "C" wd_status wd_server_step(wd_server *sv, int *completed)
{
    if (!sv) return WD_ERR_BAD_ARG;
    int done = 0;
    wd_status st = server_admit(sv, &done);
    if (st != WD_OK) {
        if (completed) *completed = done;
        return st;
    }
    std::vector<int> fin;
    if (sv->eng) {
        sv->eng->take_retired(&fin);  // systems already solved at admission
        if ((st = sv->eng->step(nullptr)) != WD_OK) return st;
        sv->eng->take_retired(&fin);
        for (int tag : fin) server_retire(sv, tag, sv->eng->results[tag], &done);
        for (int tag : fin) sv->eng->results.erase(tag);
    } else if (!sv->fp64_todo.empty()) {
        const int tag = sv->fp64_todo.front();
        sv->fp64_todo.pop_front();
        const auto &tr = sv->tag_req[tag];
        wd_server::Req &r = sv->reqs[tr.first];
        wd_solver_params p;
        wd_solver_params_default(&p);
        p.kind = WD_SOLVER_CG_EO;
        p.mass = r.mass, p.tol = r.tol, p.max_iter = sv->cfg.max_iter, p.prec = WD_PREC_F64;
        wd_solver_stats s{};
        st = wd_solve(sv->ctx, sv->lats[r.lat], r.src[tr.second], r.dest[tr.second], &p, &s);
        if (st != WD_OK && st != WD_ERR_NOT_CONVERGED) return st;
        server_retire(sv, tag, s, &done);
    }
    if (completed) *completed = done;
    return WD_OK;
}

extern "C" wd_status wd_server_poll(wd_server *sv, int64_t id, int *done, double *const *solutions,
                                    wd_solver_stats *stats, double *latency_s)
{
    if (!sv || !done) return WD_ERR_BAD_ARG;
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return wd_fail(sv->ctx, WD_ERR_BAD_ARG, "unknown or already collected request");
    wd_server::Req &r = it->second;
    *done = r.done ? 1 : 0;
    if (!r.done) return WD_OK;
    wd_status st = WD_OK;
    for (int k = 0; k < r.nsrc; ++k) {
        // a request that failed admission has no solution fields: its solutions stay untouched
        if (solutions && solutions[k] && k < (int)r.dest.size() && st == WD_OK)
            st = wd_field_download(sv->ctx, r.dest[k], solutions[k]);
        if (stats) stats[k] = r.st[k];
    }
    if (latency_s) *latency_s = std::chrono::duration<double>(r.t_done - r.t_submit).count();
    for (wd_field *f : r.dest) wd_field_destroy(f);
    sv->req_bytes -= r.bytes;
    sv->reqs.erase(it);
    return st;
}

extern "C" wd_status wd_server_status(const wd_server *sv, int *queued, int *active_systems, double *bytes_in_use)
{
    if (!sv) return WD_ERR_BAD_ARG;
    if (queued) *queued = (int)sv->queue.size();
    if (active_systems) *active_systems = sv->active_systems;
    if (bytes_in_use) *bytes_in_use = sv->gauge_bytes + sv->req_bytes;
    return WD_OK;
}
