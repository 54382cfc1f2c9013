// wd_noalloc.cu -- the complex dot product sum_i conj(a_i) b_i for callers
// that cannot allocate device memory.
//
// Who needs it: host codes that own all of HBM through their own pool (a
// lattice code that reserves the device up front for resident gauge fields
// and solver vectors), and latency-critical loops that must not call
// cudaMalloc/cudaFree because those calls synchronise the whole device and
// stall every other stream.  wd_dot (the vector_p replacement) needs a
// context, whose creation allocates its reduction scratch; this entry point
// needs nothing but the caller's inputs and output.
//
// Its per-chunk partial sums live in g_dot_scratch, a file-scope __device__
// array of WD_NOALLOC_MAX_CHUNKS entries (512 KiB).  Every GPU that loads
// this library holds that array until the process exits.  Host code cannot
// use the array's name as a device address (on the host it is only a
// stand-in symbol), so the first call on each device, with that device
// current, looks the address up with cudaGetSymbolAddress and keeps it.
// That first call should come before any stream capture.  The address is
// kept for the life of the process, so a device reset (cudaDeviceReset)
// after the first call on that device is not supported.
//
// All calls share the one array: two calls whose kernels overlap on the GPU
// (different streams, or different host threads without ordering) race on it
// and both results are then undefined.  Nothing in the array needs to start
// at zero: each call writes every partial it later reads, in stream order.
#include <cstdio>
#include <mutex>
#include "wd_kernels.h"

#define WD_NOALLOC_CHUNK 4096
#define WD_NOALLOC_MAX_CHUNKS 32768
#define WD_NOALLOC_MAX_DEVICES 64

namespace {

static __device__ __align__(256) double2 g_dot_scratch[WD_NOALLOC_MAX_CHUNKS];

__device__ __forceinline__ double nsum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// One block folds one chunk of WD_NOALLOC_CHUNK entries into partial[chunk].
__global__ void __launch_bounds__(256) k_dot_chunks(const double2 *__restrict__ a,
                                                    const double2 *__restrict__ b, int64_t n,
                                                    double2 *__restrict__ partial)
{
    __shared__ double sre[8], sim[8];
    const int64_t base = (int64_t)blockIdx.x * WD_NOALLOC_CHUNK;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < WD_NOALLOC_CHUNK; k += blockDim.x) {
        const int64_t i = base + k;
        if (i < n) {
            const double2 u = a[i], v = b[i];
            re = fma(u.x, v.x, re);
            re = fma(u.y, v.y, re);
            im = fma(u.x, v.y, im);
            im = fma(-u.y, v.x, im);
        }
    }
    re = nsum(re);
    im = nsum(im);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sre[w] = re;
        sim[w] = im;
    }
    __syncthreads();
    if (w == 0) {
        re = l < 8 ? sre[l] : 0.0;
        im = l < 8 ? sim[l] : 0.0;
        re = nsum(re);
        im = nsum(im);
        if (l == 0) partial[blockIdx.x] = make_double2(re, im);
    }
}

// One block adds nparts partials in a fixed order and writes out[0..1].
__global__ void __launch_bounds__(1024) k_dot_finish(const double2 *__restrict__ partial, int nparts,
                                                     double *__restrict__ out)
{
    __shared__ double sre[32], sim[32];
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        re += partial[i].x;
        im += partial[i].y;
    }
    re = nsum(re);
    im = nsum(im);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sre[w] = re;
        sim[w] = im;
    }
    __syncthreads();
    if (w == 0) {
        re = sre[l];
        im = sim[l];
        re = nsum(re);
        im = nsum(im);
        if (l == 0) {
            out[0] = re;
            out[1] = im;
        }
    }
}

std::mutex g_setup_mu;
double2 *g_scratch_ptr[WD_NOALLOC_MAX_DEVICES] = {};

// Device address of g_dot_scratch on the current device (looked up once).
wd_status scratch_for_current_device(double2 **ptr)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return WD_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= WD_NOALLOC_MAX_DEVICES) return WD_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_dot_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            fprintf(stderr, "wd_dot_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                    cudaGetErrorString(e));
            return WD_ERR_CUDA;
        }
        g_scratch_ptr[dev] = (double2 *)p;
    }
    *ptr = g_scratch_ptr[dev];
    return WD_OK;
}

}  // namespace

extern "C" wd_status wd_dot_noalloc(const double *a, const double *b, int64_t n, double *out, void *stream)
{
    if (!a || !b || !out) return WD_ERR_BAD_ARG;
    const int64_t max_n = (int64_t)WD_NOALLOC_MAX_CHUNKS * WD_NOALLOC_CHUNK;
    if (n < 0 || n > max_n) {
        fprintf(stderr,
                "wd_dot_noalloc: n = %lld complex entries is outside [0, %lld], the capacity of its "
                "fixed scratch array\n",
                (long long)n, (long long)max_n);
        return WD_ERR_BAD_ARG;
    }
    if (((uintptr_t)a | (uintptr_t)b) % 16 != 0 || (uintptr_t)out % 8 != 0) {
        fprintf(stderr, "wd_dot_noalloc: a and b must be 16-byte aligned, out 8-byte aligned\n");
        return WD_ERR_BAD_ARG;
    }
    double2 *scratch = nullptr;
    const wd_status st = scratch_for_current_device(&scratch);
    if (st != WD_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int nchunks = (int)((n + WD_NOALLOC_CHUNK - 1) / WD_NOALLOC_CHUNK);
    if (nchunks > 0)
        k_dot_chunks<<<nchunks, 256, 0, s>>>((const double2 *)a, (const double2 *)b, n, scratch);
    k_dot_finish<<<1, 1024, 0, s>>>(scratch, nchunks, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "wd_dot_noalloc: launch failed: %s\n", cudaGetErrorString(e));
        return WD_ERR_CUDA;
    }
    return WD_OK;
}
