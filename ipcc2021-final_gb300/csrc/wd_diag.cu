// wd_diag.cu -- device throughput probe: independent FMA chains in FP64 and
// FP32, timed with CUDA events.  Gives the compute roof the hopping kernels
// are compared against (the FP64 pipe of GB300 is far narrower than FP32).
#include "wd_kernels.h"

namespace {
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
