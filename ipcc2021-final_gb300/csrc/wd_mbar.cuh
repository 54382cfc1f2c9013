// wd_mbar.cuh -- shared-memory mbarrier helpers with bounded waits.
//
// Every wait polls mbarrier.try_wait for at most kMbarWaitNs of wall time
// (%globaltimer) and then gives up, returning false, so a phase that never
// completes cannot hang the GPU; callers record the failure in a device
// error flag that the host reads (wd_context_device_check).
#pragma once
#include <cuda_runtime.h>

constexpr unsigned long long kMbarWaitNs = 500000000ull;  // 0.5 s: phases complete in microseconds
constexpr long long kMbarWaitPolls = 1ll << 26;

__device__ __forceinline__ unsigned wd_smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long wd_globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void wd_mbar_init(unsigned mbar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// one arrival (release: this thread's earlier shared-memory writes are
// visible to threads that then observe the phase complete)
__device__ __forceinline__ void wd_mbar_arrive(unsigned mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// true once phase `parity` of the mbarrier has completed; false after
// kMbarWaitNs of wall time (or kMbarWaitPolls polls, whichever comes first)
__device__ __forceinline__ bool wd_mbar_wait(unsigned mbar, unsigned parity)
{
    const unsigned long long t0 = wd_globaltimer_ns();
    for (long long i = 0; i < kMbarWaitPolls; ++i) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (wd_globaltimer_ns() - t0 > kMbarWaitNs) return false;
    }
    return false;
}
