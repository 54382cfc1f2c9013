// wd_api.cu -- C ABI: contexts, resident lattices and fields, operators and
// the host-buffer entry points that replace the reference's functions.
#include <algorithm>
#include <cstring>
#include <cstdio>
#include <string>
#include "wd_kernels.h"
#include "wd_precision.h"
#include "wd_solver.h"

// ------------------------------------------------------------------ errors
wd_status wd_fail(wd_context *ctx, wd_status s, const std::string &msg)
{
    if (ctx) ctx->last_error = msg;
    return s;
}

wd_status wd_cuda_check(wd_context *ctx, cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the sticky-free allocation error
        return wd_fail(ctx, WD_ERR_OOM, m);
    }
    return wd_fail(ctx, WD_ERR_CUDA, m);
}

extern "C" const char *wd_status_string(wd_status s)
{
    switch (s) {
    case WD_OK: return "ok";
    case WD_ERR_BAD_DIMS: return "bad lattice dimensions";
    case WD_ERR_OOM: return "out of device memory";
    case WD_ERR_NOT_CONVERGED: return "solver did not converge";
    case WD_ERR_TIMEOUT: return "device wait timed out";
    case WD_ERR_CUDA: return "CUDA error";
    case WD_ERR_BAD_ARG: return "bad argument";
    case WD_ERR_NO_DEVICE: return "no usable CUDA device";
    case WD_ERR_NAN: return "non-finite residual";
    }
    return "unknown status";
}

extern "C" const char *wd_last_error(const wd_context *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

// ----------------------------------------------------------------- context
extern "C" wd_status wd_context_create(int device, wd_context **out)
{
    if (!out) return WD_ERR_BAD_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
        cudaGetLastError();
        return WD_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return WD_ERR_NO_DEVICE;
    // the kernels are built for sm_103a only
    if (prop.major != 10 || prop.minor != 3) return WD_ERR_NO_DEVICE;
    wd_context *ctx = new wd_context();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->h2d_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking);
    for (int i = 0; i < WD_MAX_CHUNKS && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&ctx->chunk_done[i], cudaEventDisableTiming);
    for (int i = 0; i < WD_MAX_UPLOADS && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&ctx->chunk_in[i], cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaMalloc(&ctx->red_partial, sizeof(double2) * (WD_RED_BLOCKS + WD_RED_SLOTS));
    if (e == cudaSuccess) e = cudaHostAlloc(&ctx->red_result, sizeof(double2) * WD_RED_SLOTS, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&ctx->state_host, WD_STATE_HOST_BYTES, 0);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dev_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->dev_err, 0, sizeof(int));
    if (e != cudaSuccess) {
        wd_context_destroy(ctx);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? WD_ERR_OOM : WD_ERR_CUDA;
    }
    *out = ctx;
    return WD_OK;
}

static void host_cache_drop(wd_context *ctx)
{
    for (auto &f : ctx->host_f) {
        wd_field_destroy(f);
        f = nullptr;
    }
    if (ctx->host_lat) wd_lattice_destroy(ctx->host_lat);
    ctx->host_lat = nullptr;
    for (auto &p : ctx->host_gauge_ptr) p = nullptr;
}

wd_status wd_dev_alloc(wd_context *ctx, void **p, size_t bytes)
{
    if (wd_alloc_fails(ctx)) return wd_fail(ctx, WD_ERR_OOM, "work buffer: injected allocation failure");
    bytes = (bytes + 255) & ~(size_t)255;
    // best fit among cached blocks no more than twice the request
    auto it = ctx->pool_free.lower_bound(bytes);
    if (it != ctx->pool_free.end() && it->first <= 2 * bytes) {
        *p = it->second;
        ctx->pool_used[it->second] = it->first;
        ctx->pool_free.erase(it);
        return WD_OK;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        wd_pool_release(ctx);
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) return wd_cuda_check(ctx, e, "cudaMalloc(work buffer)");
    ctx->pool_used[*p] = bytes;
    ctx->pool_bytes += bytes;
    return WD_OK;
}

void wd_dev_free(wd_context *ctx, void *p)
{
    if (!p) return;
    auto it = ctx->pool_used.find(p);
    if (it == ctx->pool_used.end()) return;
    ctx->pool_free.emplace(it->second, p);
    ctx->pool_used.erase(it);
}

void wd_pool_release(wd_context *ctx)
{
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->pool_free) {
        cudaFree(kv.second);
        ctx->pool_bytes -= kv.first;
    }
    ctx->pool_free.clear();
}

extern "C" void wd_context_destroy(wd_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    host_cache_drop(ctx);
    wd_pool_release(ctx);
    for (auto &kv : ctx->pool_used) cudaFree(kv.first);
    ctx->pool_used.clear();
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->red_partial);
    cudaFree(ctx->dev_err);
    cudaFree(ctx->staging);
    if (ctx->red_result) cudaFreeHost(ctx->red_result);
    if (ctx->state_host) cudaFreeHost(ctx->state_host);
    for (auto &ev : ctx->chunk_done)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : ctx->chunk_in)
        if (ev) cudaEventDestroy(ev);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->h2d_stream) cudaStreamDestroy(ctx->h2d_stream);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" wd_status wd_context_sync(wd_context *ctx)
{
    if (!ctx) return WD_ERR_BAD_ARG;
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" void *wd_context_stream(wd_context *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" wd_status wd_context_device_check(wd_context *ctx)
{
    if (!ctx) return WD_ERR_BAD_ARG;
    int flag = 0;
    WD_CUDA(ctx, cudaMemcpyAsync(&flag, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!flag) return WD_OK;
    WD_CUDA(ctx, cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
    return wd_fail(ctx, WD_ERR_TIMEOUT, "a kernel's bounded device wait gave up (its output is undefined)");
}

extern "C" int wd_debug_fail_allocations_after(wd_context *ctx, int n)
{
    if (!ctx) return -1;
    const int prev = ctx->fail_alloc_after;
    ctx->fail_alloc_after = n < 0 ? -1 : n;
    return prev;
}
extern "C" uint64_t wd_context_launches(const wd_context *ctx) { return ctx ? ctx->launches : 0; }

static wd_status ensure_staging(wd_context *ctx, size_t bytes)
{
    if (ctx->staging_bytes >= bytes) return WD_OK;
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->staging);
    ctx->staging = nullptr;
    ctx->staging_bytes = 0;
    WD_CUDA(ctx, cudaMalloc(&ctx->staging, bytes));
    ctx->staging_bytes = bytes;
    return WD_OK;
}

// ---------------------------------------------------------------- lattice
static wd_status make_geom(wd_context *ctx, const int *dims, WdGeom *g, int64_t *vol)
{
    if (!dims) return wd_fail(ctx, WD_ERR_BAD_ARG, "dims is null");
    int64_t v = 1;
    for (int i = 0; i < 4; ++i) {
        if (dims[i] <= 0) return wd_fail(ctx, WD_ERR_BAD_DIMS, "lattice extent must be positive");
        v *= dims[i];
        g->L[i] = dims[i];
    }
    if (dims[0] % 2) return wd_fail(ctx, WD_ERR_BAD_DIMS, "Lx must be even for the even-odd layout");
    if (v > WD_MAX_SITES) return wd_fail(ctx, WD_ERR_BAD_DIMS, "lattice too large");
    g->Lxh = dims[0] / 2;
    g->Vh = (int)(v / 2);
    *vol = v;
    return WD_OK;
}

static wd_status upload_gauge(wd_context *ctx, wd_lattice *lat, const double *const gauge[4])
{
    const WdGeom &g = lat->g;
    const size_t bytes = (size_t)lat->volume * 9 * sizeof(double2);
    wd_status st = ensure_staging(ctx, bytes);
    if (st != WD_OK) return st;
    for (int mu = 0; mu < 4; ++mu) {
        if (!gauge[mu]) return wd_fail(ctx, WD_ERR_BAD_ARG, "gauge pointer is null");
        WD_CUDA(ctx, cudaMemcpyAsync(ctx->staging, gauge[mu], bytes, cudaMemcpyHostToDevice, ctx->stream));
        st = wd_gauge_ref_to_soa(ctx, g, mu, (const double2 *)ctx->staging, lat->gauge);
        if (st != WD_OK) return st;
    }
    wd_lattice_invalidate_derived(lat);
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_lattice_create(wd_context *ctx, const int dims[4], const double *const gauge[4],
                                       wd_lattice **out)
{
    if (!ctx || !out || !gauge) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    wd_lattice *lat = new wd_lattice();
    lat->ctx = ctx;
    wd_status st = make_geom(ctx, dims, &lat->g, &lat->volume);
    if (st != WD_OK) {
        delete lat;
        return st;
    }
    cudaError_t e = cudaMalloc(&lat->gauge, (size_t)lat->volume * 4 * 9 * sizeof(double2));
    if (e != cudaSuccess) {
        delete lat;
        return wd_cuda_check(ctx, e, "cudaMalloc(gauge)");
    }
    st = upload_gauge(ctx, lat, gauge);
    if (st != WD_OK) {
        wd_lattice_destroy(lat);
        return st;
    }
    *out = lat;
    return WD_OK;
}

extern "C" wd_status wd_lattice_update(wd_context *ctx, wd_lattice *lat, const double *const gauge[4])
{
    if (!ctx || !lat || !gauge) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    return upload_gauge(ctx, lat, gauge);
}

extern "C" void wd_lattice_destroy(wd_lattice *lat)
{
    if (!lat) return;
    cudaFree(lat->gauge);  // cudaFree waits for work in flight on the device
    wd_lattice_invalidate_derived(lat);
    delete lat;
}

extern "C" int64_t wd_lattice_volume(const wd_lattice *lat) { return lat ? lat->volume : 0; }

// ------------------------------------------------------------------ fields
static size_t field_bytes(const wd_lattice *lat, wd_precision prec)
{
    size_t b = (size_t)lat->volume * 12 * wd_entry_bytes(prec);
    if (prec == WD_PREC_F16) b += (size_t)lat->volume * sizeof(float);
    return b;
}

extern "C" wd_status wd_field_create_prec(wd_context *ctx, const wd_lattice *lat, wd_precision prec, wd_field **out)
{
    if (!ctx || !lat || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (prec < WD_PREC_F64 || prec > WD_PREC_F16) return wd_fail(ctx, WD_ERR_BAD_ARG, "unknown precision");
    *out = nullptr;
    if (wd_alloc_fails(ctx)) return wd_fail(ctx, WD_ERR_OOM, "field: injected allocation failure");
    wd_field *f = new wd_field();
    f->lat = lat;
    f->storage = prec;
    const size_t bytes = field_bytes(lat, prec);
    cudaError_t e = cudaMalloc(&f->data, bytes);
    if (e != cudaSuccess) {
        delete f;
        return wd_cuda_check(ctx, e, "cudaMalloc(field)");
    }
    if (prec == WD_PREC_F64) f->d = (double2 *)f->data;
    if (prec == WD_PREC_F16) f->scale = (float *)((char *)f->data + (size_t)lat->volume * 12 * wd_entry_bytes(prec));
    e = cudaMemsetAsync(f->data, 0, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(f->data);
        delete f;
        return wd_cuda_check(ctx, e, "cudaMemsetAsync(field)");
    }
    *out = f;
    return WD_OK;
}

extern "C" wd_status wd_field_create(wd_context *ctx, const wd_lattice *lat, wd_field **out)
{
    return wd_field_create_prec(ctx, lat, WD_PREC_F64, out);
}

extern "C" wd_precision wd_field_precision(const wd_field *f) { return f ? f->storage : WD_PREC_F64; }

extern "C" void wd_field_destroy(wd_field *f)
{
    if (!f) return;
    cudaFree(f->data);  // cudaFree waits for work in flight on the device
    delete f;
}

// FP64 SoA staging <-> any storage (F16 goes through the FP32 layout kernel of wd_mixed.cu)
extern "C" wd_status wd_field_upload(wd_context *ctx, wd_field *f, const double *host)
{
    if (!ctx || !f || !host) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    const size_t bytes = (size_t)f->lat->volume * 12 * sizeof(double2);
    wd_status st = ensure_staging(ctx, bytes);
    if (st != WD_OK) return st;
    WD_CUDA(ctx, cudaMemcpyAsync(ctx->staging, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (f->storage == WD_PREC_F16)
        st = wd_spinor_ref_to_h16(ctx, f->lat->g, (const double2 *)ctx->staging, wd_whole(f));
    else
        st = wd_spinor_ref_to_soa(ctx, f->lat->g, (const double2 *)ctx->staging, wd_whole(f));
    if (st != WD_OK) return st;
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_field_download(wd_context *ctx, const wd_field *f, double *host)
{
    if (!ctx || !f || !host) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    const size_t bytes = (size_t)f->lat->volume * 12 * sizeof(double2);
    wd_status st = ensure_staging(ctx, bytes);
    if (st != WD_OK) return st;
    if (f->storage == WD_PREC_F16)
        st = wd_spinor_h16_to_ref(ctx, f->lat->g, wd_whole(f), (double2 *)ctx->staging);
    else
        st = wd_spinor_soa_to_ref(ctx, f->lat->g, wd_whole(f), (double2 *)ctx->staging);
    if (st != WD_OK) return st;
    WD_CUDA(ctx, cudaMemcpyAsync(host, ctx->staging, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_field_zero(wd_context *ctx, wd_field *f)
{
    if (!ctx || !f) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    WD_CUDA(ctx, cudaMemsetAsync(f->data, 0, field_bytes(f->lat, f->storage), ctx->stream));
    return WD_OK;
}

extern "C" wd_status wd_field_copy(wd_context *ctx, wd_field *dst, const wd_field *src)
{
    if (!ctx || !dst || !src) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (dst->lat->volume != src->lat->volume || dst->storage != src->storage)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "field size or storage mismatch");
    WD_CUDA(ctx, cudaMemcpyAsync(dst->data, src->data, field_bytes(src->lat, src->storage), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    return WD_OK;
}

// --------------------------------------------------------------- operators
static wd_status check_fields(wd_context *ctx, const wd_lattice *lat, const wd_field *a, const wd_field *b)
{
    if (!ctx || !lat || !a || !b) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (a->lat->volume != lat->volume || b->lat->volume != lat->volume)
        return wd_fail(ctx, WD_ERR_BAD_ARG, "field does not belong to this lattice size");
    if (a == b) return wd_fail(ctx, WD_ERR_BAD_ARG, "input and output must be different fields");
    if (a->storage != b->storage) return wd_fail(ctx, WD_ERR_BAD_ARG, "input and output storage differ");
    return WD_OK;
}

// out_cb = alpha * D_{cb,1-cb} in_{1-cb} + beta * x_cb on blocks of one storage format.
wd_status wd_hop_v(wd_context *ctx, const wd_lattice *lat, WdVec in, WdVec out, const WdVec *x, int cb, int dag,
                   double alpha, double beta)
{
    if (in.prec != out.prec || (x && x->prec != in.prec))
        return wd_fail(ctx, WD_ERR_BAD_ARG, "hopping term operands have different storage");
    switch (in.prec) {
    case WD_PREC_F64:
        return wd_hop_f64(ctx, lat, (const double2 *)in.p, (double2 *)out.p, x ? (const double2 *)x->p : nullptr, cb,
                          dag, alpha, beta);
    case WD_PREC_DF64:
        return wd_hop_df(ctx, lat, (const float4 *)in.p, (float4 *)out.p, x ? (const float4 *)x->p : nullptr, cb, dag,
                         alpha, beta);
    case WD_PREC_F32: return wd_hop_f32(ctx, lat, in, out, x, cb, dag, alpha, beta);
    case WD_PREC_F16: return wd_hop_f16(ctx, lat, in, out, x, cb, dag, alpha, beta);
    }
    return wd_fail(ctx, WD_ERR_BAD_ARG, "unknown precision");
}

// Runs `op` on df copies when an FP64 field is asked for double-float
// arithmetic; otherwise the arithmetic must match the storage.
template <class Op>
static wd_status with_arith(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                            wd_precision prec, bool out_needs_init, Op op)
{
    if (prec == in->storage) return op(in, out);
    if (!(in->storage == WD_PREC_F64 && prec == WD_PREC_DF64))
        return wd_fail(ctx, WD_ERR_BAD_ARG, "arithmetic precision does not match the fields' storage");
    wd_field *ti = nullptr, *to = nullptr;
    wd_status st = wd_field_create_prec(ctx, lat, WD_PREC_DF64, &ti);
    if (st == WD_OK) st = wd_field_create_prec(ctx, lat, WD_PREC_DF64, &to);
    const int64_t n = lat->volume * 12;
    if (st == WD_OK) st = wd_convert_f64_to_df(ctx, in->d, (float4 *)ti->data, n);
    if (st == WD_OK && out_needs_init) st = wd_convert_f64_to_df(ctx, out->d, (float4 *)to->data, n);
    if (st == WD_OK) st = op(ti, to);
    if (st == WD_OK) st = wd_convert_df_to_f64(ctx, (const float4 *)to->data, out->d, n);
    wd_field_destroy(ti);
    wd_field_destroy(to);
    return st;
}

extern "C" wd_status wd_dslash_offd(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                                    int dag, int cb, wd_precision prec)
{
    wd_status st = check_fields(ctx, lat, in, out);
    if (st != WD_OK) return st;
    if (cb != 0 && cb != 1) return wd_fail(ctx, WD_ERR_BAD_ARG, "cb must be 0 or 1");
    return with_arith(ctx, lat, in, out, prec, false, [&](const wd_field *i, wd_field *o) -> wd_status {
        // the reference zeroes the whole destination (src/dslash_new.cpp:1398)
        wd_status s = wd_v_zero(ctx, wd_block(o, 1 - cb), (int64_t)12 * lat->g.Vh);
        if (s != WD_OK) return s;
        return wd_hop_v(ctx, lat, wd_block(i, 1 - cb), wd_block(o, cb), nullptr, cb, dag, -0.5, 0.0);
    });
}

extern "C" wd_status wd_dslash_eo(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                                  int dag, int cb, wd_precision prec)
{
    wd_status st = check_fields(ctx, lat, in, out);
    if (st != WD_OK) return st;
    if (cb != 0 && cb != 1) return wd_fail(ctx, WD_ERR_BAD_ARG, "cb must be 0 or 1");
    return with_arith(ctx, lat, in, out, prec, true, [&](const wd_field *i, wd_field *o) -> wd_status {
        return wd_hop_v(ctx, lat, wd_block(i, 1 - cb), wd_block(o, cb), nullptr, cb, dag, -0.5, 0.0);
    });
}

extern "C" wd_status wd_dslash_eeoo(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                                    double mass)
{
    wd_status st = check_fields(ctx, lat, in, out);
    if (st != WD_OK) return st;
    const int64_t n = lat->volume * 12;
    if (in->storage == WD_PREC_F64) return wd_blas_scale(ctx, 4.0 + mass, in->d, out->d, n);
    if (in->storage == WD_PREC_DF64) {
        st = wd_v_zero(ctx, wd_whole(out), n);
        if (st != WD_OK) return st;
        return wd_v_axpby(ctx, make_double2(4.0 + mass, 0.0), wd_whole(in), make_double2(0.0, 0.0), wd_whole(out), n);
    }
    return wd_fail(ctx, WD_ERR_BAD_ARG, "DslashEEOO needs FP64 or double-float fields");
}

extern "C" wd_status wd_dslash_full(wd_context *ctx, const wd_lattice *lat, const wd_field *in, wd_field *out,
                                    double mass, int dag, wd_precision prec)
{
    wd_status st = check_fields(ctx, lat, in, out);
    if (st != WD_OK) return st;
    const double a = 4.0 + mass;
    return with_arith(ctx, lat, in, out, prec, false, [&](const wd_field *i, wd_field *o) -> wd_status {
        for (int cb = 0; cb < 2; ++cb) {
            const WdVec x = wd_block(i, cb);
            wd_status s = wd_hop_v(ctx, lat, wd_block(i, 1 - cb), wd_block(o, cb), &x, cb, dag, -0.5, a);
            if (s != WD_OK) return s;
        }
        return WD_OK;
    });
}

extern "C" wd_status wd_norm2(wd_context *ctx, const wd_field *a, double *out)
{
    if (!ctx || !a || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    wd_status st = wd_v_norm2(ctx, wd_whole(a), a->lat->volume * 12, 0);
    if (st != WD_OK) return st;
    double2 r;
    st = wd_red_fetch(ctx, 1, &r);
    *out = r.x;
    return st;
}

extern "C" wd_status wd_dot(wd_context *ctx, const wd_field *a, const wd_field *b, double out[2])
{
    if (!ctx || !a || !b || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (a->lat->volume != b->lat->volume) return wd_fail(ctx, WD_ERR_BAD_ARG, "field size mismatch");
    wd_status st = wd_v_dot(ctx, wd_whole(a), wd_whole(b), a->lat->volume * 12, 0);
    if (st != WD_OK) return st;
    double2 r;
    st = wd_red_fetch(ctx, 1, &r);
    out[0] = r.x;
    out[1] = r.y;
    return st;
}

// ------------------------------------------------------- host-buffer path
// The reference's functions take host arrays on every call.  The device copy
// of the links is kept between calls and refreshed when the caller passes a
// different gauge array (pointer identity), different extents, or when a
// fingerprint of 1024 sampled doubles per direction changes (catches links
// reloaded in place; a change that touches none of the sampled entries is
// missed, so callers that edit single links call wd_lattice_update on a
// lattice of their own).
static uint64_t gauge_fingerprint(const int dims[4], const double *const gauge[4])
{
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2] * dims[3] * 18;
    const int64_t step = n > 1024 ? n / 1024 : 1;
    uint64_t h = 1469598103934665603ull;
    for (int mu = 0; mu < 4; ++mu)
        for (int64_t i = 0; i < n; i += step) {
            uint64_t v;
            memcpy(&v, gauge[mu] + i, sizeof(v));
            h = (h ^ v) * 1099511628211ull;
        }
    return h;
}

// *deferred (optional): when the cached lattice was built from the same
// arrays, the fingerprint check is left to the caller (*deferred = true), to
// run on the host while the device works (host_pipeline's overlap step);
// the caller re-checks with host_refresh_if_changed.
static wd_status host_prepare(wd_context *ctx, const int dims[4], const double *const gauge[4],
                              bool *deferred = nullptr)
{
    if (deferred) *deferred = false;
    if (!ctx || !dims || !gauge) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    for (int i = 0; i < 4; ++i)
        if (!gauge[i] || dims[i] <= 0) return wd_fail(ctx, WD_ERR_BAD_ARG, "bad gauge pointer or extent");
    bool same = ctx->host_lat != nullptr;
    if (same)
        for (int i = 0; i < 4; ++i)
            same = same && ctx->host_lat->g.L[i] == dims[i] && ctx->host_gauge_ptr[i] == gauge[i];
    if (same && deferred) {
        *deferred = true;
        return WD_OK;
    }
    const uint64_t print = gauge_fingerprint(dims, gauge);
    if (same && print == ctx->host_gauge_print) return WD_OK;
    if (same) {  // same arrays, new contents: refresh the links only
        wd_status st = upload_gauge(ctx, ctx->host_lat, gauge);
        if (st == WD_OK) ctx->host_gauge_print = print;
        return st;
    }
    host_cache_drop(ctx);
    wd_status st = wd_lattice_create(ctx, dims, gauge, &ctx->host_lat);
    if (st != WD_OK) return st;
    for (int i = 0; i < 3; ++i) {
        st = wd_field_create(ctx, ctx->host_lat, &ctx->host_f[i]);
        if (st != WD_OK) {
            host_cache_drop(ctx);
            return st;
        }
    }
    for (int i = 0; i < 4; ++i) ctx->host_gauge_ptr[i] = gauge[i];
    ctx->host_gauge_print = print;
    return WD_OK;
}

// Host-array operators as a three-stage pipeline over time slabs: uploads of
// the source parities the operator reads (h2d stream), the arithmetic on
// output chunks (two compute streams) and downloads of finished chunks (copy
// stream) overlap.  Output chunk [t0, t1) reads source slices t0-1 .. t1 (the
// hopping term reaches one slice in t), so it waits only for the upload
// holding slice t1; uploads go in units of at most Lt/32 slices, enqueued
// just ahead of the first chunk that needs them, so the first compute starts
// after about a chunk and a unit have arrived.  Chunk 0 reads slice Lt-1 and
// runs last.  The kernels read and write the reference's site-major layout
// in the staging buffers (source parities | output parities), so data goes
// from copy to arithmetic to copy with no layout conversion.  `in_mask` and
// `out_mask` select parity blocks (bit p = parity p); compute(stream, p, lo,
// hi, in, out) enqueues output parity p's sites [lo, hi).
// Host memory that is neither pinned nor registered with CUDA (malloc'ed, as
// the reference allocates its fields).
static bool host_pageable(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

// overlap() runs on the calling thread once everything is enqueued, while
// the device works.
template <class Compute, class Overlap>
static wd_status host_pipeline(wd_context *ctx, const double *src, double *dest, int in_mask, int out_mask,
                               Compute compute, Overlap overlap)
{
    const wd_lattice *lat = ctx->host_lat;
    const WdGeom &g = lat->g;
    const int Vh = g.Vh, Lt = g.L[3];
    const int slab = g.Lxh * g.L[1] * g.L[2];  // sites of one parity per time slice
    const size_t half = (size_t)12 * Vh;       // complex entries of one parity
    wd_status st = ensure_staging(ctx, 4 * half * sizeof(double2));
    if (st != WD_OK) return st;
    double2 *in_aos = (double2 *)ctx->staging, *out_aos = in_aos + 2 * half;
    // compute chunks of about 64k sites (at most WD_MAX_CHUNKS); upload units.
    // The chunk computed first (1) and the one computed last (0) are a
    // quarter of the others, and chunk 2 half: the first kernel then waits
    // only for a few slices to arrive, and the last download after the final
    // kernel is short (pipeline fill and drain).
    int n = std::min(std::min(WD_MAX_CHUNKS, Lt), Vh / 65536);
    if (n < 3) n = 1;
    int sz[WD_MAX_CHUNKS];
    if (n >= 4 && Lt >= 2 * n) {
        const int small = std::max(1, Lt / (4 * n));
        sz[0] = sz[1] = small;
        sz[2] = 2 * small;
        const int rest = Lt - 4 * small, m = n - 3;
        for (int k = 3; k < n; ++k) sz[k] = rest / m + (k - 3 < rest % m ? 1 : 0);
    } else {
        for (int k = 0; k < n; ++k) sz[k] = (int)((int64_t)(k + 1) * Lt / n - (int64_t)k * Lt / n);
    }
    int tb[WD_MAX_CHUNKS + 1];
    tb[0] = 0;
    for (int k = 0; k < n; ++k) tb[k + 1] = tb[k] + sz[k];
    const int us = n == 1 ? Lt : (Lt + WD_MAX_UPLOADS - 1) / WD_MAX_UPLOADS;  // slices per upload unit
    const int nu = (Lt + us - 1) / us;  // upload units (<= WD_MAX_UPLOADS), unit u = slices [u*us, (u+1)*us)
    // Pageable host buffers: a copy from or to them through the copy engines
    // is staged and holds the calling thread (measured: 5.3 ms per
    // DslashoffdNew at 32^3x64 against 1.9 ms pinned), so where the device
    // reaches pageable memory itself (address translation over the CPU-GPU
    // link) kernels on the same streams move the data instead, asynchronously
    // and at the link's rate.
    const bool src_direct = ctx->pageable_access && host_pageable(src);
    const bool dest_direct = ctx->pageable_access && host_pageable(dest);
    auto move = [&](double2 *to, const double2 *from, size_t n, cudaMemcpyKind kind, bool direct,
                    cudaStream_t stream) -> wd_status {
        if (direct) return wd_copy_kernel(ctx, stream, from, to, (int64_t)n);
        WD_CUDA(ctx, cudaMemcpyAsync(to, from, n * sizeof(double2), kind, stream));
        return WD_OK;
    };
    int uploaded = 0;                   // units enqueued so far
    auto upload_through = [&](int unit) -> wd_status {
        for (; uploaded <= unit; ++uploaded) {
            const size_t lo = (size_t)uploaded * us * slab * 12;
            const size_t hi = (size_t)std::min((uploaded + 1) * us, Lt) * slab * 12;
            for (int p = 0; p < 2; ++p)
                if (in_mask & (1 << p)) {
                    wd_status e = move(in_aos + p * half + lo, (const double2 *)src + p * half + lo, hi - lo,
                                       cudaMemcpyHostToDevice, src_direct, ctx->h2d_stream);
                    if (e != WD_OK) return e;
                }
            WD_CUDA(ctx, cudaEventRecord(ctx->chunk_in[uploaded], ctx->h2d_stream));
        }
        return WD_OK;
    };
    auto enqueue = [&]() -> wd_status {
        // uploads start after the work already queued on the context's stream
        WD_CUDA(ctx, cudaEventRecord(ctx->chunk_done[0], ctx->stream));
        WD_CUDA(ctx, cudaStreamWaitEvent(ctx->h2d_stream, ctx->chunk_done[0], 0));
        // chunks 1..n-1, then 0; consecutive chunks alternate between two compute
        // streams, so one chunk's last partial wave of blocks overlaps the next's first
        for (int i = 0; i < n; ++i) {
            const int j = n == 1 ? 0 : (i + 1) % n;
            const int need = (j == 0 || tb[j + 1] >= Lt) ? nu - 1 : tb[j + 1] / us;
            if ((st = upload_through(need)) != WD_OK) return st;
            cudaStream_t cs = (i & 1) ? ctx->aux_stream : ctx->stream;
            WD_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->chunk_in[need], 0));
            const int lo = tb[j] * slab, hi = tb[j + 1] * slab;
            for (int p = 0; p < 2; ++p)
                if (out_mask & (1 << p))
                    if ((st = compute(cs, p, lo, hi, in_aos, out_aos)) != WD_OK) return st;
            WD_CUDA(ctx, cudaEventRecord(ctx->chunk_done[j], cs));
            WD_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->chunk_done[j], 0));
            for (int p = 0; p < 2; ++p)
                if (out_mask & (1 << p))
                    if ((st = move((double2 *)dest + p * half + (size_t)lo * 12, out_aos + p * half + (size_t)lo * 12,
                                   (size_t)(hi - lo) * 12, cudaMemcpyDeviceToHost, dest_direct, ctx->copy_stream)) !=
                        WD_OK)
                        return st;
        }
        return WD_OK;
    };
    st = enqueue();
    if (st == WD_OK) overlap();
    // a parity of dest the operator does not write is zero.  Four threads: the
    // copies to and from host memory run meanwhile, and a wider team both
    // competes with them for host memory bandwidth and, on a busy host, waits
    // on descheduled threads (measured at 32^3x64: 2.03 ms per call with 2-8
    // threads, up to 4.4 ms with 16 on 16 cores).
    for (int p = 0; p < 2 && st == WD_OK; ++p)
        if (!(out_mask & (1 << p))) {
            double *zero = dest + (size_t)p * half * 2;
            const int64_t nz = (int64_t)half * 2;
#pragma omp parallel for schedule(static) num_threads(4)
            for (int64_t i = 0; i < nz; ++i) zero[i] = 0.0;
        }
    // drain every stream the pipeline used -- after an enqueue error too, so
    // that no copy or kernel still reads src or writes dest once the call
    // returns and the caller may free them
    const cudaStream_t used[4] = {ctx->copy_stream, ctx->stream, ctx->aux_stream, ctx->h2d_stream};
    for (cudaStream_t q : used) {
        const cudaError_t e = cudaStreamSynchronize(q);
        if (e != cudaSuccess && st == WD_OK) st = wd_cuda_check(ctx, e, "cudaStreamSynchronize");
    }
    return st;
}

// DslashoffdNew on host arrays: only the source parity the term reads (1-cb)
// is uploaded, and the other parity of dest -- zero by the reference's
// semantics, src/dslash_new.cpp:1398 -- is cleared on the host meanwhile.
// Runs a host-buffer operator with the cached links, checking the links'
// fingerprint on the host while the device works; if the caller's links
// changed in place since they were uploaded, they are uploaded again and the
// operator runs once more on the new links.
template <class Run>
static wd_status host_run_checked(wd_context *ctx, const int dims[4], const double *const gauge[4], bool deferred,
                                  Run run)
{
    uint64_t print = 0;
    wd_status st = run([&] {
        if (deferred) print = gauge_fingerprint(dims, gauge);
    });
    if (st != WD_OK || !deferred || print == ctx->host_gauge_print) return st;
    if ((st = upload_gauge(ctx, ctx->host_lat, gauge)) != WD_OK) return st;
    ctx->host_gauge_print = print;
    return run([] {});
}

extern "C" wd_status wd_host_dslash_offd(wd_context *ctx, const int dims[4], const double *const gauge[4],
                                         const double *src, double *dest, int dag, int cb)
{
    bool deferred = false;
    wd_status st = host_prepare(ctx, dims, gauge, &deferred);
    if (st != WD_OK) return st;
    if (!src || !dest) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (cb != 0 && cb != 1) return wd_fail(ctx, WD_ERR_BAD_ARG, "cb must be 0 or 1");
    const size_t half = (size_t)12 * ctx->host_lat->g.Vh;
    return host_run_checked(ctx, dims, gauge, deferred, [&](auto overlap) {
        return host_pipeline(
            ctx, src, dest, 1 << (1 - cb), 1 << cb,
            [&](cudaStream_t cs, int p, int lo, int hi, const double2 *in, double2 *out) {
                return wd_hop_f64_aos_range(ctx, cs, ctx->host_lat, in + (1 - p) * half, out + p * half, nullptr, p,
                                            dag, -0.5, 0.0, lo, hi);
            },
            overlap);
    });
}

// DslashNew / Dslash on host arrays (src/invert.cpp:123-156): both parities go
// up and come back; each output parity p is (4+m) src_p - 1/2 D_{p,1-p} src_{1-p}
// in one kernel per chunk.
extern "C" wd_status wd_host_dslash_full(wd_context *ctx, const int dims[4], const double *const gauge[4],
                                         const double *src, double *dest, double mass, int dag)
{
    bool deferred = false;
    wd_status st = host_prepare(ctx, dims, gauge, &deferred);
    if (st != WD_OK) return st;
    if (!src || !dest) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    const size_t half = (size_t)12 * ctx->host_lat->g.Vh;
    const double a = 4.0 + mass;
    return host_run_checked(ctx, dims, gauge, deferred, [&](auto overlap) {
        return host_pipeline(
            ctx, src, dest, 3, 3,
            [&](cudaStream_t cs, int p, int lo, int hi, const double2 *in, double2 *out) {
                return wd_hop_f64_aos_range(ctx, cs, ctx->host_lat, in + (1 - p) * half, out + p * half, in + p * half,
                                            p, dag, -0.5, a, lo, hi);
            },
            overlap);
    });
}

extern "C" wd_status wd_host_cg(wd_context *ctx, const int dims[4], const double *const gauge[4],
                                const double *src, double *dest, const wd_solver_params *params,
                                wd_solver_stats *stats)
{
    wd_status st = host_prepare(ctx, dims, gauge);
    if (st != WD_OK) return st;
    if (!src || !dest || !params) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if ((st = wd_field_upload(ctx, ctx->host_f[0], src)) != WD_OK) return st;
    if ((st = wd_field_upload(ctx, ctx->host_f[1], dest)) != WD_OK) return st;
    wd_status solve = wd_solve(ctx, ctx->host_lat, ctx->host_f[0], ctx->host_f[1], params, stats);
    if (solve != WD_OK && solve != WD_ERR_NOT_CONVERGED) return solve;
    st = wd_field_download(ctx, ctx->host_f[1], dest);
    return st != WD_OK ? st : solve;
}

// reductions of host arrays: staged through the context's staging buffer
static wd_status host_reduce(wd_context *ctx, int64_t n, const double *a, const double *b, double2 *out)
{
    if (!ctx || !a || n < 0) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    const size_t bytes = (size_t)n * sizeof(double2);
    wd_status st = ensure_staging(ctx, b ? 2 * bytes : bytes);
    if (st != WD_OK) return st;
    double2 *da = (double2 *)ctx->staging, *db = da + n;
    WD_CUDA(ctx, cudaMemcpyAsync(da, a, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (b) {
        WD_CUDA(ctx, cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, ctx->stream));
        st = wd_red_dot(ctx, da, db, n, 0);
    } else {
        st = wd_red_norm2(ctx, da, n, 0);
    }
    if (st != WD_OK) return st;
    return wd_red_fetch(ctx, 1, out);
}

extern "C" wd_status wd_host_norm2(wd_context *ctx, int64_t n, const double *a, double *out)
{
    if (!out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    double2 r;
    wd_status st = host_reduce(ctx, n, a, nullptr, &r);
    *out = r.x;
    return st;
}

extern "C" wd_status wd_host_dot(wd_context *ctx, int64_t n, const double *a, const double *b, double out[2])
{
    if (!out || !b) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    double2 r;
    wd_status st = host_reduce(ctx, n, a, b, &r);
    out[0] = r.x;
    out[1] = r.y;
    return st;
}

extern "C" wd_status wd_host_check(wd_context *ctx, const int dims[4], const double *const gauge[4],
                                   const double *b, const double *x, double mass, double out[12])
{
    wd_status st = host_prepare(ctx, dims, gauge);
    if (st != WD_OK) return st;
    if (!b || !x || !out) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if ((st = wd_field_upload(ctx, ctx->host_f[0], b)) != WD_OK) return st;
    if ((st = wd_field_upload(ctx, ctx->host_f[1], x)) != WD_OK) return st;
    return wd_check(ctx, ctx->host_lat, ctx->host_f[0], ctx->host_f[1], mass, out);
}

extern "C" wd_status wd_host_dslash_eeoo(wd_context *ctx, const int dims[4], const double *src, double *dest,
                                         double mass, int parity)
{
    if (!ctx || !dims || !src || !dest) return wd_fail(ctx, WD_ERR_BAD_ARG, "null argument");
    if (parity < -1 || parity > 1) return wd_fail(ctx, WD_ERR_BAD_ARG, "parity must be -1, 0 or 1");
    WdGeom g;
    int64_t V;
    wd_status st = make_geom(ctx, dims, &g, &V);
    if (st != WD_OK) return st;
    // reference layout: parity p occupies complex entries [p*Vh*12, (p+1)*Vh*12)
    const int64_t n = V * 12, nh = n / 2;
    if ((st = ensure_staging(ctx, n * sizeof(double2))) != WD_OK) return st;
    double2 *d = (double2 *)ctx->staging;
    WD_CUDA(ctx, cudaMemcpyAsync(d, src, n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    const int64_t lo = parity == 1 ? nh : 0, hi = parity == 0 ? nh : n;
    if ((st = wd_blas_scale(ctx, 4.0 + mass, d + lo, d + lo, hi - lo)) != WD_OK) return st;
    if (parity >= 0) WD_CUDA(ctx, cudaMemsetAsync(d + (parity == 0 ? nh : 0), 0, nh * sizeof(double2), ctx->stream));
    WD_CUDA(ctx, cudaMemcpyAsync(dest, d, n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    WD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return WD_OK;
}
