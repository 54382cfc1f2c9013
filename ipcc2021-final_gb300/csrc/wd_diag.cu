// wd_diag.cu -- device throughput probe: independent FMA chains in FP64 and
// FP32, timed with CUDA events.  Gives the compute roof the hopping kernels
// are compared against (the FP64 pipe of GB300 is far narrower than FP32).
// Also a testing aid for the bounded device waits (wd_debug_expire_wait).
#include "wd_kernels.h"
#include "wd_mbar.cuh"

namespace {
// One warp waits on a barrier nothing arrives at: the bounded wait gives up
// and the kernel records it in the device error flag.
__global__ void __launch_bounds__(32) k_expire_wait(int *err, unsigned long long *waited_ns)
{
    __shared__ unsigned long long bar;
    const unsigned mbar = wd_smem_u32(&bar);
    if (threadIdx.x == 0) wd_mbar_init(mbar, 1);
    __syncwarp();
    const unsigned long long t0 = wd_globaltimer_ns();
    const bool done = wd_mbar_wait(mbar, 0);
    if (threadIdx.x == 0) {
        if (!done) atomicExch(err, 1);
        *waited_ns = wd_globaltimer_ns() - t0;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T *out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = x[k] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" wd_status wd_diag_fma_peak(wd_context *ctx, double *fp64_tflops, double *fp32_tflops)
{
    if (!ctx || !fp64_tflops || !fp32_tflops) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    cudaDeviceProp prop;
    WD_CUDA(ctx, cudaGetDeviceProperties(&prop, ctx->device));
    const int blocks = prop.multiProcessorCount * 8, threads = 256;
    void *buf = nullptr;
    WD_CUDA(ctx, cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best64 = 0, best32 = 0;
    for (int rep = 0; rep < 3; ++rep) {
        const int it64 = 2048, it32 = 16384;
        float ms = 0;
        cudaEventRecord(e0, ctx->stream);
        k_fma_chains<double><<<blocks, threads, 0, ctx->stream>>>((double *)buf, it64, 0.999, 1e-3);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best64 = fmax(best64, 2.0 * 8 * it64 * (double)blocks * threads / (ms * 1e-3) / 1e12);
        cudaEventRecord(e0, ctx->stream);
        k_fma_chains<float><<<blocks, threads, 0, ctx->stream>>>((float *)buf, it32, 0.999f, 1e-3f);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best32 = fmax(best32, 2.0 * 8 * it32 * (double)blocks * threads / (ms * 1e-3) / 1e12);
        ctx->launches += 2;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaGetLastError();
    cudaFree(buf);
    if (e != cudaSuccess) return wd_cuda_check(ctx, e, "fma probe");
    *fp64_tflops = best64;
    *fp32_tflops = best32;
    return WD_OK;
}

extern "C" wd_status wd_debug_expire_wait(wd_context *ctx, double *waited_seconds)
{
    if (!ctx || !waited_seconds) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    unsigned long long *d = nullptr, ns = 0;
    WD_CUDA(ctx, cudaMalloc(&d, sizeof(unsigned long long)));
    k_expire_wait<<<1, 32, 0, ctx->stream>>>(ctx->dev_err, d);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ns, d, sizeof(ns), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return wd_cuda_check(ctx, e, "bounded-wait probe");
    *waited_seconds = (double)ns * 1e-9;
    return WD_OK;
}
