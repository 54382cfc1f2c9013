// wd_dslash_lp.cu -- FP32 and FP16 hopping kernels (12-real links, FP32
// arithmetic) and the conversions between FP64 and the low-precision
// storage formats of wd_lp.cuh.
//
// Compulsory bytes per output site: FP32 8*48 + 96 + 96 = 576 B;
// FP16 8*24 + 52 + 52 = 296 B (+ one spinor read when the epilogue uses x).
// 1320 flop/site (+ 8 x 66 for the row-2 rebuild) is far below the FP32
// ridge: FP32 runs at the HBM bound, FP16 (half the bytes, the same
// arithmetic plus unpacking) at the instruction-issue bound.
#include <cudaTypedefs.h>
#include <algorithm>
#include "wd_hop.cuh"
#include "wd_lp_staged.cuh"
#include "wd_h16m.cuh"
#include "wd_h16_tma.cuh"
#include "wd_kernels.h"
#include "wd_reduce.cuh"
#include "wd_solver.h"
#include <type_traits>
#include "wd_tune.h"

namespace {

// THREADS per block; MINB blocks per SM as an occupancy hint (0: none)
template <class Sp, class Lk, int THREADS = 128, int MINB = 0>
struct HopLP {
    using C = float2;
    static constexpr int kThreads = THREADS;
    static constexpr int kMinBlocks = MINB;
    static constexpr bool kSiteScale = Sp::kScaled;
    WdGeom g;
    int cb;
    Sp in, out, x;
    Lk link;
    bool has_x;
    float alpha, beta;
    const int *stop = nullptr;  // gate: no-op launch while *stop != 0 (device-driven solver loops)

    __device__ __forceinline__ void load_in(int s, C *v) const { in.load(s, v); }
    __device__ __forceinline__ float load_in_raw(int s, C *v) const
    {
        if constexpr (Sp::kScaled) return in.load_raw(s, v);
        in.load(s, v);
        return 1.f;
    }
    __device__ __forceinline__ void load_link(int mu, int par, int s, C *U) const { link.load(mu, par, s, U); }
    __device__ __forceinline__ void epilogue(int s, const C *acc) const
    {
        C r[12];
        if (has_x) {
            C xv[12];
            float bx = beta;  // beta times the x site's scale
            if constexpr (Sp::kScaled) bx *= x.load_raw(s, xv);
            else x.load(s, xv);
#pragma unroll
            for (int c = 0; c < 12; ++c) r[c] = c_axpby(alpha, acc[c], bx, xv[c]);
        } else {
#pragma unroll
            for (int c = 0; c < 12; ++c) r[c] = c_scale(acc[c], alpha);
        }
        out.store(s, r);
    }
};

// links: FP64 planes [mu][par][9][Vh] -> rows 0,1 in FP32 / FP16
__global__ void k_gauge_f32(const double2 *__restrict__ g, float4 *__restrict__ out, int Vh)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int mp = blockIdx.y;  // mu*2 + par
    if (s >= Vh) return;
    const double2 *b = g + (size_t)mp * 9 * Vh + s;
    float4 *o = out + (size_t)mp * 3 * Vh + s;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double2 u0 = b[(size_t)(2 * j) * Vh], u1 = b[(size_t)(2 * j + 1) * Vh];
        o[(size_t)j * Vh] = make_float4((float)u0.x, (float)u0.y, (float)u1.x, (float)u1.y);
    }
}

__global__ void k_gauge_f16(const double2 *__restrict__ g, uint4 *__restrict__ a, uint2 *__restrict__ bb, int Vh)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int mp = blockIdx.y;
    if (s >= Vh) return;
    const double2 *b = g + (size_t)mp * 9 * Vh + s;
    float2 u[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double2 v = b[(size_t)k * Vh];
        u[k] = make_float2((float)v.x, (float)v.y);
    }
    a[(size_t)mp * Vh + s] = pack4(u);
    __half2 h4 = f2h(u[4]), h5 = f2h(u[5]);
    bb[(size_t)mp * Vh + s] = make_uint2(*reinterpret_cast<unsigned *>(&h4), *reinterpret_cast<unsigned *>(&h5));
}

// FP64 SoA block [12][Vh] <-> low-precision block, one thread per site
template <class Sp>
__global__ void k_from_f64(const double2 *__restrict__ in, Sp out, int Vh)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Vh) return;
    float2 v[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) {
        const double2 d = in[(size_t)c * Vh + s];
        v[c] = make_float2((float)d.x, (float)d.y);
    }
    out.store(s, v);
}

template <class Sp>
__global__ void k_to_f64(Sp in, double2 *__restrict__ out, int Vh, int accumulate)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Vh) return;
    float2 v[12];
    in.load(s, v);
#pragma unroll
    for (int c = 0; c < 12; ++c) {
        double2 d = make_double2(v[c].x, v[c].y);
        if (accumulate) {
            const double2 o = out[(size_t)c * Vh + s];
            d.x += o.x;
            d.y += o.y;
        }
        out[(size_t)c * Vh + s] = d;
    }
}

// reference AoS (both parities) <-> FP16 field
__global__ void k_aos_to_h16(const double2 *__restrict__ aos, SpF16 out, int Vh)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Vh) return;
    float2 v[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) {
        const double2 d = aos[(size_t)s * 12 + c];
        v[c] = make_float2((float)d.x, (float)d.y);
    }
    out.store(s, v);
}

__global__ void k_h16_to_aos(SpF16 in, double2 *__restrict__ aos, int Vh)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= Vh) return;
    float2 v[12];
    in.load(s, v);
#pragma unroll
    for (int c = 0; c < 12; ++c) aos[(size_t)s * 12 + c] = make_double2(v[c].x, v[c].y);
}

inline int site_blocks(int Vh) { return (Vh + 127) / 128; }

template <class P>
wd_status launch_hop(wd_context *ctx, const P &p, int dag)
{
    const int blocks = (p.g.Vh + P::kThreads - 1) / P::kThreads;
    if (dag) wd_hop_kernel<true><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
    else wd_hop_kernel<false><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// the FP16 kernel with FP16-operand arithmetic (wd_h16m.cuh), staged operands
template <bool DAG, class P>
__global__ void __launch_bounds__(P::kThreads, wd_min_blocks<P>::value) k_hop_h16m(const P p)
{
    using Sp = decltype(p.in);
    using Lk = decltype(p.link);
    __shared__ LpStage<Sp, Lk, P::kThreads> st;
    if (wd_gate_closed(p)) return;
    const int s = blockIdx.x * P::kThreads + threadIdx.x;
    if (s >= p.g.Vh) return;
    float2 acc[12];
    h16_hop_site_staged<DAG>(p, s, acc, st);
    p.epilogue(s, acc);
}

template <class P>
wd_status launch_hop_h16m(wd_context *ctx, const P &p, int dag)
{
    const int blocks = (p.g.Vh + P::kThreads - 1) / P::kThreads;
    if (dag) k_hop_h16m<true><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
    else k_hop_h16m<false><<<blocks, P::kThreads, 0, ctx->stream>>>(p);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

// ----------------------------------------------------------------------
// TMA-staged FP16 kernel (wd_h16_tma.cuh): tensor maps and launch.

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (no link against libcuda); null if the driver does not offer it
PFN_cuTensorMapEncodeTiled_v12000 tma_encoder()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

// a map of 32-bit words: dims innermost first, strides (bytes) of dims 1.., box
template <int R>
bool tma_map(CUtensorMap *m, const void *base, const cuuint64_t (&dims)[R], const cuuint64_t (&strides)[R - 1],
             const cuuint32_t (&box)[R])
{
    const auto fn = tma_encoder();
    if (!fn || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
    const cuuint32_t unit[5] = {1, 1, 1, 1, 1};  // element strides: every element
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, R, const_cast<void *>(base), dims, strides, box, unit,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr unsigned kTmaSmemMax = 232448;  // 227 KB: the largest dynamic shared memory of one block

// The maps and shared-memory layout of a BY x BZ tile.  False when the
// lattice or the operands do not fit the kernel's rules: Lxh a multiple of 4
// (16-byte scale rows) and at most 32, Ly and Lz multiples of the tile, at
// most 256 threads (sites) a tile, 16-byte aligned planes.
bool h16_tma_build(H16TmaMaps &M, const WdGeom &g, const SpF16 &in, int BY, int BZ)
{
    const cuuint64_t X = g.Lxh, Ly = g.L[1], Lz = g.L[2], Lt = g.L[3], Vh = g.Vh;
    if (X % 4 || X > 32 || Ly % BY || Lz % BZ || BY * BZ * X > 256) return false;
    const cuuint32_t x = (cuuint32_t)X, by = BY, bz = BZ;
    // spinor planes: words [3][Lt][Lz][Ly][4X]; scales [Lt][Lz][Ly][X]
    const cuuint64_t sd[5] = {4 * X, Ly, Lz, Lt, 3}, ss[4] = {16 * X, 16 * X * Ly, 16 * X * Ly * Lz, 16 * Vh};
    const cuuint64_t cd[4] = {X, Ly, Lz, Lt}, cs[3] = {4 * X, 4 * X * Ly, 4 * X * Ly * Lz};
    const cuuint32_t sbox[3][5] = {{4 * x, by, bz, 1, 3}, {4 * x, 1, bz, 1, 3}, {4 * x, by, 1, 1, 3}};
    const cuuint32_t cbox[3][4] = {{x, by, bz, 1}, {x, 1, bz, 1}, {x, by, 1, 1}};
    for (int k = 0; k < 3; ++k) {
        if (!tma_map<5>(&M.sp[k], in.p, sd, ss, sbox[k])) return false;
        if (!tma_map<4>(&M.sc[k], in.scale, cd, cs, cbox[k])) return false;
    }
    // regions: spinor planes (48 B a site) and scales (4 B) of the tile and
    // the faces; copy group of region r: (r + 1) / 2
    const unsigned RC = BY * BZ, rows[7] = {RC, (unsigned)BZ, (unsigned)BZ, (unsigned)BY, (unsigned)BY, RC, RC};
    unsigned off = 0;
    for (int k = 0; k < 4; ++k) M.tx_bytes[k] = 0;
    for (int r = 0; r < 7; ++r) {
        const unsigned sp = 48 * rows[r] * x, sc = 4 * rows[r] * x;
        M.off[r] = off;
        off += (sp + 127) & ~127u;
        M.off[kRegSc + r] = off;
        off += (sc + 127) & ~127u;
        M.tx_bytes[(r + 1) / 2] += sp + sc;
    }
    M.stage_bytes = off;
    return true;
}

// dynamic shared memory of a launch: the regions, four barriers, alignment slack
inline unsigned h16_tma_smem(const H16TmaMaps &m) { return m.stage_bytes + 32 + 128; }

// Tensor maps depend only on the spinor's addresses, the geometry and the
// tile: a small per-thread cache spares re-encoding them at every launch.
struct TmaKey {
    const void *in, *scale;
    int L[4], BY, BZ;
    bool operator==(const TmaKey &o) const
    {
        return in == o.in && scale == o.scale && L[0] == o.L[0] && L[1] == o.L[1] && L[2] == o.L[2] &&
               L[3] == o.L[3] && BY == o.BY && BZ == o.BZ;
    }
};

const H16TmaMaps *h16_tma_maps(const WdGeom &g, const SpF16 &in, int BY, int BZ)
{
    struct Entry {
        TmaKey key;
        bool ok;
        H16TmaMaps maps;
    };
    thread_local Entry cache[8];
    thread_local int used = 0, next = 0;
    const TmaKey key{in.p, in.scale, {g.L[0], g.L[1], g.L[2], g.L[3]}, BY, BZ};
    for (int i = 0; i < used; ++i)
        if (cache[i].key == key) return cache[i].ok ? &cache[i].maps : nullptr;
    Entry &e = cache[next];
    next = (next + 1) % 8;
    used = used < 8 ? used + 1 : 8;
    e.key = key;
    e.ok = h16_tma_build(e.maps, g, in, BY, BZ);
    return e.ok ? &e.maps : nullptr;
}

template <bool DAG, int BY, int BZ, class P>
void launch_h16_tma_k(wd_context *ctx, const H16TmaArgs<P> &a, int blocks, int threads, unsigned smem)
{
    auto k = k_hop_h16_tma<DAG, BY, BZ, P>;
    static unsigned attr_set = 0;  // devices on which the shared-memory limit is raised
    if (ctx->device < 32 && !(attr_set & (1u << ctx->device))) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTmaSmemMax);
        attr_set |= 1u << ctx->device;
    }
    k<<<blocks, threads, smem, ctx->stream>>>(a);
}

// The TMA-staged FP16 kernel (spinors staged, links loaded per thread), one
// block per tile; returns false (nothing launched) when the lattice or the
// operands do not fit it.  Tile: 4 x 4 rows up to Lxh = 16, 4 x 2 beyond.
template <class P>
bool launch_hop_h16_tma(wd_context *ctx, const P &p, int dag, wd_status *st)
{
    const WdGeom &g = p.g;
    const int BY = 4, BZ = g.Lxh <= 16 ? 4 : 2;
    const H16TmaMaps *m = h16_tma_maps(g, p.in, BY, BZ);
    if (!m || h16_tma_smem(*m) > kTmaSmemMax) return false;
    H16TmaArgs<HopLP<SpF16, LinkF16>> a;
    a.m = *m;
    auto &q = a.p;
    q.g = p.g, q.cb = p.cb, q.in = p.in, q.out = p.out, q.x = p.x, q.link = p.link;
    q.has_x = p.has_x, q.alpha = p.alpha, q.beta = p.beta, q.stop = p.stop;
    a.err = ctx->dev_err;
    const int threads = BY * BZ * g.Lxh, blocks = g.Vh / threads;
    const unsigned smem = h16_tma_smem(*m);
    using A = HopLP<SpF16, LinkF16>;
    if (BZ == 4) {
        if (dag) launch_h16_tma_k<true, 4, 4, A>(ctx, a, blocks, threads, smem);
        else launch_h16_tma_k<false, 4, 4, A>(ctx, a, blocks, threads, smem);
    } else {
        if (dag) launch_h16_tma_k<true, 4, 2, A>(ctx, a, blocks, threads, smem);
        else launch_h16_tma_k<false, 4, 2, A>(ctx, a, blocks, threads, smem);
    }
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    *st = e == cudaSuccess ? WD_OK : wd_cuda_check(ctx, e, "k_hop_h16_tma launch");
    return true;
}

// The launch variants the tuner times.  FP32: 128, 64 or 256 threads per
// block, or 128 with registers capped for 8 blocks per SM (GB300, D_eo at
// 32^3x64: all within 1 % of 102.5 us).  FP16: the FP16-operand kernel
// (wd_h16m.cuh) with each thread's next-direction operands staged in shared
// memory by cp.async, 128 threads (6 blocks per SM) or 64 (12), registers
// capped at 80: 63.8 / 63.8 us at 32^3x64, 0.291 / 0.293 ms at 48^3x96; 128
// threads capped at 64 registers for 8 blocks per SM (variant 3, a few bytes
// spilled): 63.6 us and 0.289 ms; or
// the TMA-staged kernel (wd_h16_tma.cuh; 75.8 us and 0.358 ms: every block
// stalls on its copies before its first direction, and at 3 blocks of 256
// threads an SM that start-up is not hidden -- issue slots busy 64 % against
// 74 % for the cp.async kernel).
// Replaced: the FP16 kernels converting every operand to FP32 first (staged
// 71.8 us, register-loading 73.8-79.9 us at 32^3x64; 0.331 ms at 48^3x96).
// Dropped: the staged FP32 kernel (103.1-104.0: 144 bytes per thread and
// slot leave less L1 for the neighbour spinors), the staged FP16 kernel
// without the register cap, a software-pipelined form issuing the next
// direction's register loads before the current direction's arithmetic (the
// compiler already hoists those loads), and TMA forms staging the links too
// (82.0 us: links have no reuse, and the extra 58 KB a tile leave 2 blocks an
// SM), walking tiles with double buffering (76.0 us, 2 blocks an SM), with
// 2 x 2 row tiles (75.9 us) or with one barrier for all copies (71.8-73.8 us).
template <class Sp, class Lk>
wd_status launch_tuned(wd_context *ctx, const char *name, const HopLP<Sp, Lk> &p, int dag)
{
    constexpr bool kF16 = std::is_same_v<Sp, SpF16>;
    return wd_tune_launch(ctx, name, p.g.Vh, 4, [&](int v) -> wd_status {
        auto make = [&](auto threads, auto minb) {
            HopLP<Sp, Lk, decltype(threads)::value, decltype(minb)::value> q;
            q.g = p.g, q.cb = p.cb, q.in = p.in, q.out = p.out, q.x = p.x, q.link = p.link;
            q.has_x = p.has_x, q.alpha = p.alpha, q.beta = p.beta, q.stop = p.stop;
            return q;
        };
        using I0 = std::integral_constant<int, 0>;
        using T64 = std::integral_constant<int, 64>;
        using T128 = std::integral_constant<int, 128>;
        if constexpr (kF16) {
            if (v == 2) {  // TMA-staged neighbour spinors
                wd_status st;
                if (launch_hop_h16_tma(ctx, p, dag, &st)) return st;
                v = 0;  // the lattice does not fit the TMA kernel
            }
            if (v == 1) return launch_hop_h16m(ctx, make(T64(), std::integral_constant<int, 12>()), dag);
            if (v == 3) return launch_hop_h16m(ctx, make(T128(), std::integral_constant<int, 8>()), dag);
            return launch_hop_h16m(ctx, make(T128(), std::integral_constant<int, 6>()), dag);
        } else {
            switch (v) {
            case 1: return launch_hop(ctx, make(T64(), I0()), dag);
            case 2: return launch_hop(ctx, make(std::integral_constant<int, 256>(), I0()), dag);
            case 3: return launch_hop(ctx, make(T128(), std::integral_constant<int, 8>()), dag);
            default: return launch_hop(ctx, make(T128(), I0()), dag);
            }
        }
    });
}

}  // namespace

wd_status wd_lattice_gauge_lp(wd_context *ctx, const wd_lattice *lat_c, wd_precision prec)
{
    wd_lattice *lat = const_cast<wd_lattice *>(lat_c);
    const int Vh = lat->g.Vh;
    dim3 grid((Vh + 127) / 128, 8);
    if (prec == WD_PREC_F32) {
        if (lat->gauge_f32) return WD_OK;
        WD_CUDA(ctx, cudaMalloc(&lat->gauge_f32, (size_t)8 * 3 * Vh * sizeof(float4)));
        k_gauge_f32<<<grid, 128, 0, ctx->stream>>>(lat->gauge, (float4 *)lat->gauge_f32, Vh);
    } else {
        if (lat->gauge_h12) return WD_OK;
        WD_CUDA(ctx, cudaMalloc(&lat->gauge_h12, (size_t)8 * Vh * (sizeof(uint4) + sizeof(uint2))));
        uint4 *a = (uint4 *)lat->gauge_h12;
        k_gauge_f16<<<grid, 128, 0, ctx->stream>>>(lat->gauge, a, (uint2 *)(a + (size_t)8 * Vh), Vh);
    }
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_hop_f32(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                     double alpha, double beta, const int *stop)
{
    wd_status st = wd_lattice_gauge_lp(ctx, lat, WD_PREC_F32);
    if (st != WD_OK) return st;
    HopLP<SpF32, LinkF32> p;
    p.g = lat->g;
    p.cb = cb;
    p.in = sp_f32(in, lat->g.Vh);
    p.out = sp_f32(out, lat->g.Vh);
    p.has_x = x != nullptr;
    p.x = x ? sp_f32(*x, lat->g.Vh) : p.out;
    p.link = LinkF32{(const float4 *)lat->gauge_f32, lat->g.Vh};
    p.alpha = (float)alpha;
    p.beta = (float)beta;
    p.stop = stop;
    return launch_tuned(ctx, "hop_f32", p, dag);
}

wd_status wd_hop_f16(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                     double alpha, double beta, const int *stop)
{
    wd_status st = wd_lattice_gauge_lp(ctx, lat, WD_PREC_F16);
    if (st != WD_OK) return st;
    HopLP<SpF16, LinkF16> p;
    p.g = lat->g;
    p.cb = cb;
    p.in = sp_f16(in, lat->g.Vh);
    p.out = sp_f16(out, lat->g.Vh);
    p.has_x = x != nullptr;
    p.x = x ? sp_f16(*x, lat->g.Vh) : p.out;
    const uint4 *a = (const uint4 *)lat->gauge_h12;
    p.link = LinkF16{a, (const uint2 *)(a + (size_t)8 * lat->g.Vh), lat->g.Vh};
    p.alpha = (float)alpha;
    p.beta = (float)beta;
    p.stop = stop;
    return launch_tuned(ctx, "hop_f16", p, dag);
}

wd_status wd_lp_from_f64(wd_context *ctx, int Vh, const double2 *in, WdVec out)
{
    if (out.prec == WD_PREC_F32) k_from_f64<<<site_blocks(Vh), 128, 0, ctx->stream>>>(in, sp_f32(out, Vh), Vh);
    else k_from_f64<<<site_blocks(Vh), 128, 0, ctx->stream>>>(in, sp_f16(out, Vh), Vh);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_lp_to_f64(wd_context *ctx, int Vh, WdVec in, double2 *out, int accumulate)
{
    if (in.prec == WD_PREC_F32) k_to_f64<<<site_blocks(Vh), 128, 0, ctx->stream>>>(sp_f32(in, Vh), out, Vh, accumulate);
    else k_to_f64<<<site_blocks(Vh), 128, 0, ctx->stream>>>(sp_f16(in, Vh), out, Vh, accumulate);
    WD_LAUNCHED(ctx);
    return WD_OK;
}

wd_status wd_spinor_ref_to_h16(wd_context *ctx, const WdGeom &g, const double2 *ref, WdVec f)
{
    for (int par = 0; par < 2; ++par) {
        const WdVec b = wd_offset(f, (int64_t)par * 12 * g.Vh, (int64_t)par * g.Vh);
        k_aos_to_h16<<<site_blocks(g.Vh), 128, 0, ctx->stream>>>(ref + (size_t)par * 12 * g.Vh, sp_f16(b, g.Vh), g.Vh);
        WD_LAUNCHED(ctx);
    }
    return WD_OK;
}

wd_status wd_spinor_h16_to_ref(wd_context *ctx, const WdGeom &g, WdVec f, double2 *ref)
{
    for (int par = 0; par < 2; ++par) {
        const WdVec b = wd_offset(f, (int64_t)par * 12 * g.Vh, (int64_t)par * g.Vh);
        k_h16_to_aos<<<site_blocks(g.Vh), 128, 0, ctx->stream>>>(sp_f16(b, g.Vh), ref + (size_t)par * 12 * g.Vh, g.Vh);
        WD_LAUNCHED(ctx);
    }
    return WD_OK;
}

// ===================================================================
// Reducing operator steps of the mixed-precision CG (wd_mixed.cu): the
// second hop of t = Mhat p also reduces |t|^2, the second hop of
// q = Mhat^dag t applies the CG update instead of storing q.  One block
// partial per block; the last block to finish (a one-shot atomic counter, no
// waiting) folds the partials in a fixed order -- the result does not depend
// on which block finishes last -- and updates the solver's device scalars.
namespace {

// kEpiNorm / kEpiUpdate: the CG iteration's steps (device scalars in dev);
// kEpiNormResult: out stored and |out|^2 written to *result
enum { kEpiNorm = 0, kEpiUpdate = 1, kEpiNormResult = 2 };

template <class Sp, class Lk, int THREADS, int MINB, int EPI>
struct HopLPRed : HopLP<Sp, Lk, THREADS, MINB> {
    WdMxDev *dev;
    double *partial;
    unsigned *counter;  // kEpiNormResult
    double *result;     // kEpiNormResult
    Sp pvec;       // update: p at the output site (x_s += alpha p)
    SpF32 rs, xs;  // update: iterated residual and solution increment

    // out = alpha acc + beta x, then the site's contribution to the reduction
    __device__ __forceinline__ float epilogue_red(int s, const float2 *acc) const
    {
        float2 r[12], xv[12];
        float bx = this->beta;  // beta times the x site's scale
        if constexpr (Sp::kScaled) bx *= this->x.load_raw(s, xv);
        else this->x.load(s, xv);
#pragma unroll
        for (int c = 0; c < 12; ++c) r[c] = c_axpby(this->alpha, acc[c], bx, xv[c]);
        float n = 0.f;
        if constexpr (EPI != kEpiUpdate) {
#pragma unroll
            for (int c = 0; c < 12; ++c) n = fmaf(r[c].x, r[c].x, fmaf(r[c].y, r[c].y, n));
            this->out.store(s, r);
        } else {
            const float a = dev->alpha;
            rs.load(s, xv);
#pragma unroll
            for (int c = 0; c < 12; ++c) {
                xv[c] = make_float2(fmaf(-a, r[c].x, xv[c].x), fmaf(-a, r[c].y, xv[c].y));
                n = fmaf(xv[c].x, xv[c].x, fmaf(xv[c].y, xv[c].y, n));
            }
            rs.store(s, xv);
            pvec.load(s, r);
            xs.load(s, xv);
#pragma unroll
            for (int c = 0; c < 12; ++c) xv[c] = make_float2(fmaf(a, r[c].x, xv[c].x), fmaf(a, r[c].y, xv[c].y));
            xs.store(s, xv);
        }
        return n;
    }
};

// t reduced: alpha = rr / |t|^2
__device__ __forceinline__ void mx_fin_norm(WdMxDev *d, double tt)
{
    d->tt = tt;
    if (!(tt > 0.0) || !isfinite(tt)) {
        d->stop = 2;
        return;
    }
    d->alpha = (float)(d->rr / tt);
}

// |r_s|^2 after the update: the reliable-update rule of wd_mixed.cu
__device__ __forceinline__ void mx_fin_update(WdMxDev *d, double rr_new)
{
    d->rr_new = rr_new;
    d->iters += 1;
    if (!isfinite(rr_new)) {
        d->stop = 2;
        return;
    }
    if (rr_new < d->delta2 * d->rr_max || rr_new <= d->target2) {
        d->stop = 1;  // the host runs the update; rr keeps the previous iterate's value
        return;
    }
    d->beta = (float)(rr_new / d->rr);
    d->rr = rr_new;
}

// STAGED: the FP16 kernel's staged operands and FP16-operand arithmetic
// (wd_h16m.cuh); otherwise the register-loading FP32 kernel
template <bool DAG, bool STAGED, int EPI, class P>
__device__ __forceinline__ float red_site(const P &p, int s)
{
    float v = 0.f;
    if constexpr (STAGED) {
        using Sp = decltype(p.in);
        using Lk = decltype(p.link);
        __shared__ LpStage<Sp, Lk, P::kThreads> st;
        if (s < p.g.Vh) {
            float2 acc[12];
            h16_hop_site_staged<DAG>(p, s, acc, st);
            v = p.epilogue_red(s, acc);
        }
    } else {
        if (s < p.g.Vh) {
            float2 acc[12];
            wd_hop_site<DAG>(p, s, acc);
            v = p.epilogue_red(s, acc);
        }
    }
    return v;
}

template <bool DAG, bool STAGED, int EPI, class P>
__global__ void __launch_bounds__(P::kThreads, wd_min_blocks<P>::value) k_hop_lp_red(const P p)
{
    constexpr int T = P::kThreads;
    if (EPI != kEpiNormResult && p.dev->stop) return;  // the same value in every block of the launch
    const int s = blockIdx.x * T + threadIdx.x;
    const float v = red_site<DAG, STAGED, EPI>(p, s);
    unsigned *counter = EPI == kEpiNorm ? &p.dev->count_t : EPI == kEpiUpdate ? &p.dev->count_r : p.counter;
    double tot;
    if (!wd_grid_sum<T>((double)v, p.partial, counter, &tot)) return;
    if constexpr (EPI == kEpiNorm) mx_fin_norm(p.dev, tot);
    else if constexpr (EPI == kEpiUpdate) mx_fin_update(p.dev, tot);
    else *p.result = tot;
}

// the launch shape the tuner chose for the plain hop of this storage and size
// (FP16's 8-blocks-per-SM shape too: 128 threads like variant 0, so the same
// reduction partials and bits; mixed FP16 solves 0.8-1.2 % faster with it)
template <int EPI, class Sp, class Lk>
wd_status launch_red(wd_context *ctx, const char *name, const HopLP<Sp, Lk> &b, int dag, WdMxDev *dev,
                     double *partial, Sp pvec, SpF32 rs, SpF32 xs, unsigned *counter = nullptr,
                     double *result = nullptr)
{
    constexpr bool kF16 = std::is_same_v<Sp, SpF16>;
    int v = wd_tune_choice(ctx, name, b.g.Vh);
    if (v < 0 || (v == 3 && !kF16)) v = 0;  // FP32 3 caps registers at 64: the reducing epilogues would spill
    auto run = [&](auto threads, auto minb, auto staged) -> wd_status {
        constexpr int TH = decltype(threads)::value, MB = decltype(minb)::value;
        constexpr bool ST = decltype(staged)::value;
        HopLPRed<Sp, Lk, TH, MB, EPI> q;
        q.g = b.g, q.cb = b.cb, q.in = b.in, q.out = b.out, q.x = b.x, q.link = b.link;
        q.has_x = true, q.alpha = b.alpha, q.beta = b.beta;
        q.dev = dev, q.partial = partial, q.pvec = pvec, q.rs = rs, q.xs = xs;
        q.counter = counter, q.result = result;
        const int blocks = (b.g.Vh + TH - 1) / TH;
        if (dag) k_hop_lp_red<true, ST, EPI><<<blocks, TH, 0, ctx->stream>>>(q);
        else k_hop_lp_red<false, ST, EPI><<<blocks, TH, 0, ctx->stream>>>(q);
        WD_LAUNCHED(ctx);
        return WD_OK;
    };
    using I0 = std::integral_constant<int, 0>;
    using T64 = std::integral_constant<int, 64>;
    using T128 = std::integral_constant<int, 128>;
    using Yes = std::true_type;
    using No = std::false_type;
    if constexpr (kF16) {
        if (v == 1) return run(T64(), std::integral_constant<int, 12>(), Yes());
        if (v == 3) return run(T128(), std::integral_constant<int, 8>(), Yes());
        return run(T128(), std::integral_constant<int, 6>(), Yes());
    } else {
        switch (v) {
        case 1: return run(T64(), I0(), No());
        case 2: return run(std::integral_constant<int, 256>(), I0(), No());
        default: return run(T128(), I0(), No());
        }
    }
}

template <class Sp, class Lk>
HopLP<Sp, Lk> red_base(const wd_lattice *lat, Sp in, Sp out, Sp x, Lk link, double mass)
{
    const double a = 4.0 + mass;
    HopLP<Sp, Lk> b;
    b.g = lat->g;
    b.cb = 0;
    b.in = in, b.out = out, b.x = x, b.link = link;
    b.has_x = true;
    b.alpha = (float)(-0.25 / a);
    b.beta = (float)a;
    return b;
}

template <int EPI>
wd_status hop_lp_red(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, WdVec x, WdVec p, WdVec rs,
                     WdVec xs, double mass, int dag, WdMxDev *dev, double *partial)
{
    const int Vh = lat->g.Vh;
    if (in.prec != x.prec || in.prec != p.prec || (in.prec != WD_PREC_F32 && in.prec != WD_PREC_F16))
        return wd_fail(ctx, WD_ERR_BAD_ARG, "reducing hop: FP32 or FP16 operands of one storage");
    wd_status st = wd_lattice_gauge_lp(ctx, lat, in.prec);
    if (st != WD_OK) return st;
    const SpF32 r32 = sp_f32(rs, Vh), x32 = sp_f32(xs, Vh);
    if (in.prec == WD_PREC_F32) {
        const LinkF32 lk{(const float4 *)lat->gauge_f32, Vh};
        return launch_red<EPI>(ctx, "hop_f32", red_base(lat, sp_f32(in, Vh), sp_f32(out, Vh), sp_f32(x, Vh), lk, mass),
                               dag, dev, partial, sp_f32(p, Vh), r32, x32);
    }
    const uint4 *a = (const uint4 *)lat->gauge_h12;
    const LinkF16 lk{a, (const uint2 *)(a + (size_t)8 * Vh), Vh};
    return launch_red<EPI>(ctx, "hop_f16", red_base(lat, sp_f16(in, Vh), sp_f16(out, Vh), sp_f16(x, Vh), lk, mass), dag,
                           dev, partial, sp_f16(p, Vh), r32, x32);
}

}  // namespace

wd_status wd_hop_lp_norm(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec t, WdVec p, double mass,
                         WdMxDev *dev, double *partial)
{
    WdVec none;
    none.prec = WD_PREC_F32;
    return hop_lp_red<kEpiNorm>(ctx, lat, in, t, p, p, none, none, mass, 0, dev, partial);
}

wd_status wd_hop_lp_update(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec t, WdVec p, WdVec rs, WdVec xs,
                           double mass, WdMxDev *dev, double *partial)
{
    // out is not written by the update epilogue
    return hop_lp_red<kEpiUpdate>(ctx, lat, in, t, t, p, rs, xs, mass, 1, dev, partial);
}

wd_status wd_hop_f32_norm(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, WdVec x, double mass, int dag,
                          double *partial, unsigned *counter, double *result)
{
    const int Vh = lat->g.Vh;
    if (in.prec != WD_PREC_F32 || out.prec != WD_PREC_F32 || x.prec != WD_PREC_F32)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "wd_hop_f32_norm: FP32 operands");
    wd_status st = wd_lattice_gauge_lp(ctx, lat, WD_PREC_F32);
    if (st != WD_OK) return st;
    const LinkF32 lk{(const float4 *)lat->gauge_f32, Vh};
    const SpF32 none = sp_f32(out, Vh);
    return launch_red<kEpiNormResult>(ctx, "hop_f32",
                                      red_base(lat, sp_f32(in, Vh), sp_f32(out, Vh), sp_f32(x, Vh), lk, mass), dag,
                                      nullptr, partial, none, none, none, counter, result);
}
