// wd_tune.h -- launch-shape autotuner (wd_tune.cu).
#pragma once
#include <functional>
#include "wd_internal.cuh"

// Launch one of nvariants shapes of `kernel` for half-volume Vh: the cached
// best, or, on the first call, time them all and keep the fastest.
// launch(v) must enqueue variant v on ctx->stream and be idempotent.
wd_status wd_tune_launch(wd_context *ctx, const char *kernel, int Vh, int nvariants,
                         const std::function<wd_status(int)> &launch);
