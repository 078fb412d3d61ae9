/*
 * cvtpm_tools.h — measurement helpers exported by libcvtpm.so beside the
 * drop-in ABI of cvtpm.h.  They have no counterpart in the reference: they
 * supply denominators for roofline reporting.
 */
#ifndef CVTPM_TOOLS_H
#define CVTPM_TOOLS_H

#include "cvtpm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FP32 CUDA-core peak of `device`: a grid of independent FFMA chains
 * (2 flops each), timed with CUDA events on `stream`.  Writes TFLOP/s. */
cvtpm_status cvtpm_tool_fp32_peak(int device, void* stream, float* tflops);

/* The blocked PD smoother alone: `steps` (even) steps on the left view's
 * smoother input and edge weights of the last depthMap call on `ctx`, run
 * on `stream` into the context's scratch; writes the time per step (us,
 * best of two timed runs after a warm-up).  depthMap runs the two views'
 * smoothers concurrently, so its per-phase timings cannot give this. */
cvtpm_status cvtpm_tool_pd_time(cvtpm_ctx* ctx, int steps, void* stream, float* us_per_step);

#ifdef __cplusplus
}
#endif
#endif
