// wd_reduce.cuh -- warp/block reduction helpers shared by the BLAS and
// solver kernels.  Partials are FP64; block size WD_RED_THREADS.
#pragma once
#include "wd_kernels.h"

__device__ __forceinline__ double wd_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-reduce (a, b) and write one partial per block.
__device__ __forceinline__ void wd_block_partial(double a, double b, double2 *partial)
{
    __shared__ double sa[WD_RED_THREADS / 32], sb[WD_RED_THREADS / 32];
    a = wd_warp_sum(a);
    b = wd_warp_sum(b);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = l < WD_RED_THREADS / 32 ? sa[l] : 0.0;
        b = l < WD_RED_THREADS / 32 ? sb[l] : 0.0;
        a = wd_warp_sum(a);
        b = wd_warp_sum(b);
        if (l == 0) partial[blockIdx.x] = make_double2(a, b);
    }
}

// Grid-wide sum with no waiting: each block adds its threads' v and writes one
// partial; the block that finishes last (a one-shot atomic counter, which it
// resets to 0) folds partial[0 .. gridDim.x) in a fixed order, so the total
// does not depend on which block that is.  Returns true in thread 0 of that
// block, with the total in *total.  T = threads per block (a multiple of 32);
// every thread of the block must call it; partial holds gridDim.x doubles.
template <int T>
__device__ __forceinline__ bool wd_grid_sum(double v, double *partial, unsigned *counter, double *total)
{
    __shared__ double sw[T / 32];
    __shared__ int last;
    v = wd_warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sw[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
#pragma unroll
        for (int i = 0; i < T / 32; ++i) b += sw[i];
        partial[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += T) t += __ldcg(partial + i);
    t = wd_warp_sum(t);
    __syncthreads();
    if (l == 0) sw[w] = t;
    __syncthreads();
    if (threadIdx.x != 0) return false;
    double tot = 0.0;
#pragma unroll
    for (int i = 0; i < T / 32; ++i) tot += sw[i];
    *counter = 0;
    *total = tot;
    return true;
}
