// wd_tune.cu -- launch-shape autotuner for the hopping kernels.
//
// A tunable kernel has a few compiled launch variants (threads per block,
// sites per block, occupancy hints).  The first call for a (device, kernel,
// half-volume) times every variant with CUDA events on the context's stream
// (one warm-up launch, then the best of three) and keeps the fastest; later
// calls reuse the choice.  Launches must be idempotent (out = f(in, x) with
// out distinct from the inputs), which every hop launch is.  WD_TUNE=0
// disables tuning (variant 0 everywhere); WD_TUNE_CACHE=<file> loads and
// appends decisions so later processes skip the timing.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include "wd_tune.h"

namespace {

struct Tuner {
    std::mutex mu;
    std::map<std::tuple<int, std::string, int>, int> best;  // (device, kernel, Vh) -> variant
    std::map<std::tuple<int, std::string, int>, float> best_ms;
    std::map<std::string, int> variants;  // kernel -> number of launch variants (seen at launch)
    bool loaded = false;
    int enabled = -1;

    bool on()
    {
        if (enabled < 0) {
            const char *e = std::getenv("WD_TUNE");
            enabled = (e && e[0] == '0') ? 0 : 1;
        }
        return enabled == 1;
    }
    void load()
    {
        if (loaded) return;
        loaded = true;
        const char *path = std::getenv("WD_TUNE_CACHE");
        if (!path) return;
        FILE *f = std::fopen(path, "r");
        if (!f) return;
        char name[128];
        int dev, vh, var;
        float ms;
        while (std::fscanf(f, "%d %127s %d %d %f", &dev, name, &vh, &var, &ms) == 5) {
            best[{dev, name, vh}] = var;
            best_ms[{dev, name, vh}] = ms;
        }
        std::fclose(f);
    }
    void save(int dev, const std::string &name, int vh, int var, float ms)
    {
        const char *path = std::getenv("WD_TUNE_CACHE");
        if (!path) return;
        FILE *f = std::fopen(path, "a");
        if (!f) return;
        std::fprintf(f, "%d %s %d %d %.6f\n", dev, name.c_str(), vh, var, ms);
        std::fclose(f);
    }
};

Tuner &tuner()
{
    static Tuner t;
    return t;
}

}  // namespace

wd_status wd_tune_launch(wd_context *ctx, const char *kernel, int Vh, int nvariants,
                         const std::function<wd_status(int)> &launch)
{
    Tuner &T = tuner();
    int choice = 0;
    {
        std::lock_guard<std::mutex> lock(T.mu);
        T.load();
        T.variants[kernel] = nvariants;
        auto it = T.best.find({ctx->device, kernel, Vh});
        if (it != T.best.end()) choice = it->second;
        else if (!T.on() || nvariants <= 1) choice = 0;
        else choice = -1;
    }
    if (choice < 0) {  // never time inside a stream capture
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) choice = 0;
    }
    if (choice >= 0) return launch(choice < nvariants ? choice : 0);
    // time every variant: one warm-up launch, best of three timed launches
    cudaEvent_t e0, e1;
    WD_CUDA(ctx, cudaEventCreate(&e0));
    WD_CUDA(ctx, cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int best_v = 0;
    wd_status st = WD_OK;
    for (int v = 0; v < nvariants && st == WD_OK; ++v) {
        st = launch(v);
        for (int r = 0; r < 3 && st == WD_OK; ++r) {
            cudaEventRecord(e0, ctx->stream);
            st = launch(v);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                best_v = v;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != WD_OK) return st;
    {
        std::lock_guard<std::mutex> lock(T.mu);
        T.best[{ctx->device, kernel, Vh}] = best_v;
        T.best_ms[{ctx->device, kernel, Vh}] = best_ms;
        T.save(ctx->device, kernel, Vh, best_v, best_ms);
    }
    return launch(best_v);  // the call's own launch, with the chosen shape
}

int wd_tune_choice(wd_context *ctx, const char *kernel, int Vh)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    T.load();
    auto it = T.best.find({ctx->device, kernel, Vh});
    if (it != T.best.end()) return it->second;
    return T.on() ? -1 : 0;
}

extern "C" int wd_tune_report(char *buf, int len)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    std::string s;
    for (auto &kv : T.best) {
        char line[200];
        std::snprintf(line, sizeof(line), "%d %s %d %d %.4f\n", std::get<0>(kv.first), std::get<1>(kv.first).c_str(),
                      std::get<2>(kv.first), kv.second, T.best_ms[kv.first]);
        s += line;
    }
    if (buf && len > 0) {
        const int n = (int)s.size() < len - 1 ? (int)s.size() : len - 1;
        s.copy(buf, n);
        buf[n] = 0;
    }
    return (int)s.size();
}

extern "C" int wd_tune_pin(int device, const char *kernel, int half_volume, int variant)
{
    if (!kernel || half_volume <= 0) return -1;
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    T.load();
    const auto key = std::make_tuple(device, std::string(kernel), half_volume);
    if (variant < 0) {
        T.best.erase(key);
        T.best_ms.erase(key);
        return 0;
    }
    auto it = T.variants.find(kernel);
    if (it != T.variants.end() && variant >= it->second) return -1;
    T.best[key] = variant;
    T.best_ms[key] = -1.0f;  // pinned, not timed
    return 0;
}

extern "C" int wd_tune_variants(const char *kernel)
{
    if (!kernel) return 0;
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    auto it = T.variants.find(kernel);
    return it == T.variants.end() ? 0 : it->second;
}

extern "C" void wd_tune_enable(int on)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    T.enabled = on ? 1 : 0;
}
