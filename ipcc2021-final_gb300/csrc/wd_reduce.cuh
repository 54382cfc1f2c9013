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
