// wd_tune.h -- launch-shape autotuner (wd_tune.cu).
#pragma once
#include <functional>
#include "wd_internal.cuh"

// Launch one of nvariants shapes of `kernel` for half-volume Vh: the cached
// best, or, on the first call, time them all and keep the fastest.
// launch(v) must enqueue variant v on ctx->stream and be idempotent.
wd_status wd_tune_launch(wd_context *ctx, const char *kernel, int Vh, int nvariants,
                         const std::function<wd_status(int)> &launch);

// The launch variant the tuner keeps for (kernel, Vh) on this context's
// device, or -1 when it has not chosen one yet.  Kernels that fuse work into
// a tuned kernel's epilogue (and so cannot be timed repeatedly) take the
// plain kernel's shape.
int wd_tune_choice(wd_context *ctx, const char *kernel, int Vh);
