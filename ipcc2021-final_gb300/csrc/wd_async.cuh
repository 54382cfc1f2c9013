// wd_async.cuh -- per-thread asynchronous copies global -> shared memory
// (cp.async, LDGSTS) for kernels that stage the next direction's operands
// while they compute the current one.  Each copy moves one 4-, 8- or 16-byte
// element; both addresses must be aligned to its size.  A thread's copies
// become visible to that thread after cp.async.wait_group retires their
// group; other threads would also need a barrier (the kernels using these
// read back only their own copies).
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ unsigned wd_smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// L1-allocating copy of BYTES = 4, 8 or 16
template <int BYTES>
__device__ __forceinline__ void wd_cp_async_ca(void *smem, const void *gmem)
{
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(wd_smem_addr(smem)), "l"(gmem), "n"(BYTES)
                 : "memory");
}
// L2-only copy of 16 bytes (data read once)
__device__ __forceinline__ void wd_cp_async_cg16(void *smem, const void *gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(wd_smem_addr(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void wd_cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's committed groups are still pending
template <int N>
__device__ __forceinline__ void wd_cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
