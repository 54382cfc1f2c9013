// wd_h16_tma.cuh -- the FP16 hopping kernel with its neighbour spinors
// staged in shared memory by the Tensor Memory Accelerator: each neighbour
// spinor is loaded once per tile and reused by every output site of the tile
// that touches it, and no thread computes a neighbour spinor's address.
//
// A block owns a tile of output sites of parity cb: all Lxh half-x sites of
// the rows y0..y0+BY-1, z0..z0+BZ-1 of one time slice t0, one thread per
// site.  The neighbours the tile reads (parity 1-cb) are the tile's own rows
// (x neighbours, and y/z neighbours inside the tile) and six one-row-thick
// faces: y0-1 and y0+BY (BZ rows each), z0-1 and z0+BZ (BY rows each), and
// the tile's rows in the time slices t0-1 and t0+1.  A face is a single layer,
// so a face across the periodic boundary is just the wrapped coordinate: no
// box ever leaves the lattice.  One thread issues 14 bulk tensor copies
// (cp.async.bulk.tensor: spinor planes and scales over the tile and the six
// faces) in four groups, each completing on its own mbarrier; every thread
// then computes its site with the arithmetic of wd_h16m.cuh in the same
// direction order, so results are bit-identical to the other FP16 kernels.
// Links have no reuse between sites and are loaded per thread.
//
// Every wait on a barrier is bounded (wd_mbar.cuh, 0.5 s): after that the thread
// sets *err, waits once more (bounded) for copies still in flight and returns
// without computing, so a copy that never completes cannot hang the GPU; the
// host reports the flag as an error (wd_context_device_check).
#pragma once
#include <cuda.h>
#include "wd_h16m.cuh"
#include "wd_mbar.cuh"

// shared-memory regions: spinor planes of the tile (0) and of the faces y-,
// y+, z-, z+, t-, t+ (1..6); their scales (7..13)
enum { kRegSc = 7, kRegCount = 14 };

struct H16TmaMaps {
    CUtensorMap sp[3];       // spinor planes [3][Lt][Lz][Ly][4 Lxh] words: tile (= t face), y face, z face boxes
    CUtensorMap sc[3];       // scales [Lt][Lz][Ly][Lxh]: the same boxes
    unsigned off[kRegCount];  // byte offset of each region
    unsigned stage_bytes;     // bytes of all regions (a multiple of 128); the barriers follow
    unsigned tx_bytes[4];     // bytes of each copy group: tile, y faces, z faces, t faces
};

template <class P>
struct H16TmaArgs {
    H16TmaMaps m;
    P p;       // geometry, output, x and the epilogue
    int *err;  // set when a wait gives up
};

__device__ __forceinline__ void wd_tma_load4(unsigned dst, const CUtensorMap *m, int c0, int c1, int c2, int c3,
                                             unsigned mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(m), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void wd_tma_load5(unsigned dst, const CUtensorMap *m, int c0, int c1, int c2, int c3,
                                             int c4, unsigned mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(m), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(mbar)
        : "memory");
}

// The operands of direction D for the thread at half-x index xh, tile rows
// (ly, lz): neighbour spinor (half2 bits) and scale from shared memory, link
// rows 0 and 1 from the link planes in global memory.
template <int D, int BY, int BZ, class P>
__device__ __forceinline__ void tma_operands(const H16TmaMaps &m, const P &p, const unsigned char *sm, int s,
                                             const WdSite &c, int xh_f, int xh_b, int ly, int lz, unsigned *sp,
                                             float &sc, unsigned *U)
{
    const int Lxh = p.g.Lxh, xh = c.xh;
    constexpr int MU = D / 2;
    constexpr bool FWD = (D % 2) == 0;
    constexpr int RC = BY * BZ;
    // spinor region and row within it
    int reg, row, rows, x = xh;
    if constexpr (MU == 0) {
        reg = 0, row = lz * BY + ly, rows = RC, x = FWD ? xh_f : xh_b;
    } else if constexpr (MU == 1) {
        const bool in = FWD ? ly + 1 < BY : ly > 0;
        reg = in ? 0 : (FWD ? 2 : 1);
        row = in ? lz * BY + ly + (FWD ? 1 : -1) : lz;
        rows = in ? RC : BZ;
    } else if constexpr (MU == 2) {
        const bool in = FWD ? lz + 1 < BZ : lz > 0;
        reg = in ? 0 : (FWD ? 4 : 3);
        row = in ? (lz + (FWD ? 1 : -1)) * BY + ly : ly;
        rows = in ? RC : BY;
    } else {
        reg = FWD ? 6 : 5, row = lz * BY + ly, rows = RC;
    }
    const uint4 *spr = reinterpret_cast<const uint4 *>(sm + m.off[reg]);
    const float *scr = reinterpret_cast<const float *>(sm + m.off[kRegSc + reg]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const uint4 v = spr[(j * rows + row) * Lxh + x];
        sp[4 * j] = v.x, sp[4 * j + 1] = v.y, sp[4 * j + 2] = v.z, sp[4 * j + 3] = v.w;
    }
    sc = scr[row * Lxh + x];
    // links: forward U_mu(x) at this site (parity cb), backward U_mu(x - mu)
    // at the neighbour (parity 1-cb)
    const int ls = FWD ? s : wd_neighbour(p.g, s, c, MU, false);
    const size_t i = (size_t)(MU * 2 + (FWD ? p.cb : 1 - p.cb)) * p.g.Vh + ls;
    const uint4 la = __ldg(p.link.a + i);
    const uint2 lb = __ldg(p.link.b + i);
    U[0] = la.x, U[1] = la.y, U[2] = la.z, U[3] = la.w, U[4] = lb.x, U[5] = lb.y;
}

template <int D, bool DAG, int BY, int BZ, class P>
__device__ __forceinline__ void tma_dir(const H16TmaMaps &m, const P &p, const unsigned char *sm, int s,
                                        const WdSite &c, int xh_f, int xh_b, int ly, int lz, float2 *acc)
{
    unsigned sp[12], U[9];
    float sc;
    tma_operands<D, BY, BZ>(m, p, sm, s, c, xh_f, xh_b, ly, lz, sp, sc, U);
    h16_dir_terms<D / 2, (D % 2) == 0, DAG>(sp, sc, U, acc);
}

// Thread 0: arm the barriers and issue the copies of one tile, in the order
// the directions use them: group 0 the tile's own rows (x, inner y and z
// neighbours), 1 the y faces, 2 the z faces, 3 the t faces; each group
// completes on its own barrier (mbar + 8 * group).
template <int BY, int BZ>
__device__ __forceinline__ void tma_issue(const H16TmaMaps &m, const WdGeom &g, int tile, unsigned base, unsigned mbar)
{
    const int nty = g.L[1] / BY, ntz = g.L[2] / BZ;
    const int y0 = tile % nty * BY, z0 = (tile / nty) % ntz * BZ, t0 = tile / (nty * ntz);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar + 8 * k), "r"(m.tx_bytes[k])
                     : "memory");
    const int ym = (y0 + g.L[1] - 1) % g.L[1], yp = (y0 + BY) % g.L[1];
    const int zm = (z0 + g.L[2] - 1) % g.L[2], zp = (z0 + BZ) % g.L[2];
    const int tm = (t0 + g.L[3] - 1) % g.L[3], tp = (t0 + 1) % g.L[3];
    // spinor planes and scales: tile, y-, y+, z-, z+, t-, t+
    const int cy[7] = {y0, ym, yp, y0, y0, y0, y0};
    const int cz[7] = {z0, z0, z0, zm, zp, z0, z0};
    const int ct[7] = {t0, t0, t0, t0, t0, tm, tp};
    const int box[7] = {0, 1, 1, 2, 2, 0, 0};
#pragma unroll
    for (int r = 0; r < 7; ++r) {
        const unsigned bar = mbar + 8 * ((r + 1) / 2);  // group of region r
        wd_tma_load5(base + m.off[r], &m.sp[box[r]], 0, cy[r], cz[r], ct[r], 0, bar);
        wd_tma_load4(base + m.off[kRegSc + r], &m.sc[box[r]], 0, cy[r], cz[r], ct[r], bar);
    }
}

// One block per tile, BY * BZ * Lxh <= 256 threads, one per site: thread 0
// issues the tile's copies; every thread computes its site direction by
// direction, waiting for each copy group just before the first direction
// that reads it, so the later groups arrive while the earlier directions
// compute.  Links are loaded per thread from global memory (they have no
// reuse).  Dynamic shared memory: m.stage_bytes, the four barriers, 128 bytes
// of alignment slack.  Registers are capped at 80 (3 blocks of 256 threads
// an SM).
template <bool DAG, int BY, int BZ, class P>
__global__ void __launch_bounds__(256, 3) k_hop_h16_tma(const __grid_constant__ H16TmaArgs<P> a)
{
    extern __shared__ unsigned char sm_raw[];
    if (wd_gate_closed(a.p)) return;
    const H16TmaMaps &m = a.m;
    const WdGeom &g = a.p.g;
    unsigned char *sm = sm_raw + ((128u - (wd_smem_u32(sm_raw) & 127u)) & 127u);
    const unsigned base = wd_smem_u32(sm);
    const unsigned mbar = base + m.stage_bytes;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar + 8 * k) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tma_issue<BY, BZ>(m, g, blockIdx.x, base, mbar);
    }
    __syncthreads();  // the barriers are initialised before anyone waits on them
    const int nty = g.L[1] / BY, ntz = g.L[2] / BZ;
    const int y0 = blockIdx.x % nty * BY, z0 = (blockIdx.x / nty) % ntz * BZ, t0 = blockIdx.x / (nty * ntz);
    const int Lxh = g.Lxh;
    const int r = threadIdx.x / Lxh;
    const int ly = r % BY, lz = r / BY;
    WdSite c;
    c.xh = threadIdx.x % Lxh, c.y = y0 + ly, c.z = z0 + lz, c.t = t0;
    c.xodd = (c.y + c.z + c.t + a.p.cb) & 1;
    const int s = c.xh + Lxh * (c.y + g.L[1] * (c.z + g.L[2] * t0));
    // half-x index of the x neighbours (the rule of wd_neighbour)
    const int xh_f = c.xodd ? (c.xh + 1 == Lxh ? 0 : c.xh + 1) : c.xh;
    const int xh_b = c.xodd ? c.xh : (c.xh == 0 ? Lxh - 1 : c.xh - 1);
    float2 acc[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) acc[j] = make_float2(0.f, 0.f);
    bool ok = wd_mbar_wait(mbar, 0);
    if (ok) {
        tma_dir<0, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        tma_dir<1, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        ok = wd_mbar_wait(mbar + 8, 0);
    }
    if (ok) {
        tma_dir<2, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        tma_dir<3, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        ok = wd_mbar_wait(mbar + 16, 0);
    }
    if (ok) {
        tma_dir<4, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        tma_dir<5, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
        ok = wd_mbar_wait(mbar + 24, 0);
    }
    if (!ok) {
        atomicExch(a.err, 1);
        // once more, bounded, for copies still in flight
        for (int k = 0; k < 4; ++k) wd_mbar_wait(mbar + 8 * k, 0);
        return;
    }
    tma_dir<6, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
    tma_dir<7, DAG, BY, BZ>(m, a.p, sm, s, c, xh_f, xh_b, ly, lz, acc);
    a.p.epilogue(s, acc);
}
