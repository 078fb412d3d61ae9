/*
 * cvtpm.h — C ABI of the GB300 slanted-plane PatchMatch stereo library
 * (libcvtpm.so).  Plain C: pointers, sizes and status codes; no C++ or torch
 * types cross this boundary and no exception escapes it.
 *
 * It replaces the OpenCL path behind
 *   cvt::PMHuberStereo::depthMap(Image& dmap, const Image& left,
 *       const Image& right, size_t patchsize, float depthmax,
 *       size_t iterations, size_t viewsamples, float dscale = -1.0f,
 *       Image* normalmap = NULL)
 * declared at cvt/vision/PMHuberStereo.h:40 and implemented at
 * cvt/vision/PMHuberStereo.cpp:64-291 (kernels in cvt/cl/kernel/pmhstereo.cl,
 * cvt/cl/kernel/PDHuberWeighted.cl, cvt/cl/kernel/RNG.cl; smoother in
 * cvt/gfx/PDROF.h:50-96).
 *
 * Conventions
 *  - Images are row-major RGBA float32 (4 floats per pixel, the reference's
 *    IFormat::RGBA_FLOAT), with a row pitch in BYTES that is a multiple of 16.
 *    The disparity map is GRAY float32 (IFormat::GRAY_FLOAT) with its own pitch.
 *  - Device pointers belong to the caller.  Scratch memory belongs to the
 *    context, is allocated on first use for a given size and reused.
 *  - Work is stream-ordered on the cudaStream_t passed as `void* stream`
 *    (NULL = legacy default stream).  Only the *_host entry points and
 *    cvtpm_synchronize block the calling thread.
 *  - One context per host thread at a time; contexts are independent.
 */
#ifndef CVTPM_H
#define CVTPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cvtpm_status {
    CVTPM_OK = 0,
    CVTPM_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad pitch, bad enum      */
    CVTPM_ERR_SIZE = 2,             /* width/height/patchsize out of range    */
    CVTPM_ERR_INCONSISTENT = 3,     /* left/right sizes differ (the reference
                                       throws CVTException, PMHuberStereo.cpp:66-68) */
    CVTPM_ERR_CUDA = 4,             /* a CUDA runtime call failed             */
    CVTPM_ERR_ALLOC = 5,            /* device allocation failed               */
    CVTPM_ERR_TIMEOUT = 6,          /* a bounded device wait gave up          */
    CVTPM_ERR_NOT_SUPPORTED = 7,
    CVTPM_ERR_IO = 8                /* a file could not be opened, read or
                                       written, or its header is corrupt    */
} cvtpm_status;

enum { CVTPM_RNG_MWC64X = 0, CVTPM_RNG_PHILOX = 1 };
/* EXACT: the reference's operation order, no contraction (bit-faithful to the
 * .cl arithmetic).  FAST: FMA-contracted tap arithmetic with a precomputed
 * (value, forward difference) layout of the other view; its CPU mirror is the
 * oracle run with the same setting. */
enum { CVTPM_ARITH_EXACT = 0, CVTPM_ARITH_FAST = 1 };
enum { CVTPM_SCHEDULE_JACOBI = 0, CVTPM_SCHEDULE_REDBLACK = 1 };
enum { CVTPM_PROFILE_SMOOTHSTEP = 0, CVTPM_PROFILE_CONSTANT = 1 };
enum { CVTPM_PRESET_REFERENCE = 0, CVTPM_PRESET_BASELINE = 1 };

/* Every constant of the path.  cvtpm_params_default() fills them. */
typedef struct cvtpm_params {
    int   patchsize;        /* window radius P, window (2P+1)^2; 1..31      */
    float depthmax;         /* maximum disparity in pixels (> 0)            */
    int   iterations;       /* PatchMatch iterations (>= 1)                 */
    int   viewsamples;      /* accepted and ignored: 4 slots, as in the
                               reference (pmhstereo.cl:40)                  */
    float dscale;           /* output scale; <= 0 means 1/depthmax
                               (PMHuberStereo.cpp:75-76)                    */
    float maxdispdiff;      /* LR check, px (PMHuberStereo.cpp:70: 0.5)     */
    float maxanglediff;     /* LR check, degrees (:71: 10)                  */
    float thetascale;       /* PD lambda = theta*thetascale + 5 (:72,:243)  */
    int   pd_iterations;    /* PD steps per view per iteration (:243: 250)  */
    float color_weight;     /* COLORWEIGHT (pmhstereo.cl:34: 26)            */
    float color_alpha;      /* COLORGRADALPHA, colour share (:35: 0.05)     */
    float color_maxdiff;    /* COLORMAXDIFF (:36: 0.04)                     */
    float grad_maxdiff;     /* GRADMAXDIFF (:37: 0.01)                      */
    int   weight_profile;   /* CVTPM_PROFILE_*                              */
    int   rng;              /* CVTPM_RNG_*                                  */
    uint64_t seed;          /* Philox key (ignored by MWC64X)               */
    int   arith;            /* CVTPM_ARITH_*                                */
    int   schedule;         /* CVTPM_SCHEDULE_*: JACOBI is the reference's;
                               REDBLACK (added) updates the pixels with
                               (x+y) even from the old field, then the odd
                               ones from the updated field               */
} cvtpm_params;

/* Per-pixel integer outputs of a run, for bit-exact comparison. */
typedef struct cvtpm_trace {
    uint8_t* winners;       /* 2*W*H: index of the winning hypothesis in the
                               last propagation pass, left view then right;
                               0 kept, 1-8 neighbours, 9 smooth, 10-15 random
                               neighbours, 16 random plane, 17-20 view,
                               21-22 refinements                            */
    uint8_t* valid;         /* W*H: final LR-consistency mask of the left view */
    float*   states;        /* 2*W*H*4: final plane states (s0,s1,s2,cost),
                               left then right                              */
} cvtpm_trace;

typedef struct cvtpm_ctx cvtpm_ctx;

/* Counters of the calls since the last cvtpm_reset_stats (no reference
 * counterpart: observability for benchmarks and tests). */
typedef struct cvtpm_stats {
    uint64_t calls;              /* depthmap calls                              */
    uint64_t launches;           /* kernels this library launched               */
    uint64_t propagate_launches;
    uint64_t cost_evals;         /* (pixel, candidate) cost evaluations of the
                                    propagation passes, counted on the device   */
    uint64_t cost_taps;          /* in-image window taps of those evaluations   */
    uint64_t pd_launches;
    uint64_t pd_steps;           /* PD smoother steps (several per launch)      */
    float    propagate_ms;       /* CUDA-event time of the propagation launches */
    float    pd_ms;              /* CUDA-event time of the PD smoother loops    */
} cvtpm_stats;

/* One stereo pair of a batch. */
typedef struct cvtpm_pair {
    const float* left;      /* device RGBA f32 */
    const float* right;
    int width, height;
    size_t pitch;           /* bytes, both images */
    float depthmax;
    float* dmap;            /* device GRAY f32 out */
    size_t dmap_pitch;      /* bytes */
} cvtpm_pair;

const char*  cvtpm_version(void);
const char*  cvtpm_status_string(cvtpm_status s);
cvtpm_status cvtpm_params_default(cvtpm_params* p, int preset);

/* Context (replaces the CLKernel members built in PMHuberStereo's
 * constructor, PMHuberStereo.cpp:42-58). */
cvtpm_status cvtpm_create(cvtpm_ctx** ctx, int device);
cvtpm_status cvtpm_destroy(cvtpm_ctx* ctx);
cvtpm_status cvtpm_set_params(cvtpm_ctx* ctx, const cvtpm_params* p);
cvtpm_status cvtpm_get_params(const cvtpm_ctx* ctx, cvtpm_params* p);
/* The message of the context's last failure; with ctx == NULL, the message
 * of the calling thread's last failed context-free call (image conversion,
 * file readers and writers, cvtpm_cost_eval_noalloc). */
const char*  cvtpm_last_error(const cvtpm_ctx* ctx);
cvtpm_status cvtpm_synchronize(cvtpm_ctx* ctx, void* stream);

/* PMHuberStereo::depthMap (PMHuberStereo.h:40, PMHuberStereo.cpp:64-291).
 * patchsize, depthmax, iterations, viewsamples and dscale override the
 * context's parameters for this call, as the reference's arguments do.
 * normalmap may be NULL (reference default).  trace may be NULL.
 * Stream order: the call's work is ordered after earlier work on `stream`
 * and everything it writes is complete, in `stream`'s order, when later
 * work on `stream` runs.  Inside, the right view's smoother runs on a
 * second stream of the context, forked from `stream` by an event and joined
 * back before the call's last launch, so the call also works under stream
 * capture.  Calls on one context from different streams must be ordered by
 * the caller. */
cvtpm_status cvtpm_depthmap(cvtpm_ctx* ctx,
                            float* dmap, size_t dmap_pitch,
                            const float* left, const float* right,
                            int width, int height, size_t pitch,
                            int patchsize, float depthmax, int iterations,
                            int viewsamples, float dscale,
                            float* normalmap, size_t normalmap_pitch,
                            const cvtpm_trace* trace, void* stream);

/* The same call on HOST buffers: copies in, runs, copies out, synchronizes. */
cvtpm_status cvtpm_depthmap_host(cvtpm_ctx* ctx,
                                 float* dmap, size_t dmap_pitch,
                                 const float* left, const float* right,
                                 int width, int height, size_t pitch,
                                 int patchsize, float depthmax, int iterations,
                                 int viewsamples, float dscale,
                                 float* normalmap, size_t normalmap_pitch,
                                 void* stream);

/* The state of a depthMap run between two iterations: everything the
 * iterations from `iteration` on read (the random streams are keyed by
 * pixel, iteration and view, so they need no state).  Device memory of the
 * caller, 16-byte aligned; W*H*4 floats per view, left view first. */
typedef struct cvtpm_checkpoint {
    int iteration;          /* the next iteration to run, 0..iterations     */
    float* states;          /* 2*W*H*4: plane states (s0, s1, s2, cost)     */
    float* smooth;          /* 2*W*H*4: PD-smoothed fields (nx, ny, d/dmax, 1) */
} cvtpm_checkpoint;

/* cvtpm_depthmap in pieces, for checkpointing long runs or inspecting the
 * field between iterations; no counterpart in the reference, which runs
 * the whole schedule in one call.  resume (may be NULL: start with the
 * random init) continues from resume->iteration; the run stops before
 * iteration `stop` (stop < 0 or >= iterations: runs to the end) and, with
 * save given, writes the state there into save->states / save->smooth and
 * sets save->iteration.  dmap (and normalmap, trace) are produced only by a
 * call that runs to the end (dmap may be NULL otherwise).  A run split at
 * any iteration into a saving call and a resuming call gives the bits of the
 * uninterrupted call.  The other arguments are cvtpm_depthmap's. */
cvtpm_status cvtpm_depthmap_resumable(cvtpm_ctx* ctx,
                                      float* dmap, size_t dmap_pitch,
                                      const float* left, const float* right,
                                      int width, int height, size_t pitch,
                                      int patchsize, float depthmax, int iterations,
                                      int viewsamples, float dscale,
                                      float* normalmap, size_t normalmap_pitch,
                                      const cvtpm_trace* trace,
                                      const cvtpm_checkpoint* resume, int stop,
                                      cvtpm_checkpoint* save, void* stream);

/* PMHuberStereo::depthMapInpaint (PMHuberStereo.h:41, PMHuberStereo.cpp:
 * 293-506) on device images: the depthMap schedule with the occlusion-masked
 * Huber-ROF smoother (100 steps, lambda = 20*theta + 5), theta ramped from
 * iteration 4, the final consistency check with 1 px / 5 degrees on state
 * buffer 1 (as the reference, whatever the iteration count) and the
 * disparity in pixels (scale 1).  dmap is W*H floats (pitch in bytes).
 * Parameters other than patchsize/depthmax/iterations come from the
 * context (cvtpm_set_params); maxdispdiff, maxanglediff, thetascale,
 * pd_iterations and dscale are not used.  trace (optional) as for
 * cvtpm_depthmap. */
cvtpm_status cvtpm_depthmap_inpaint(cvtpm_ctx* ctx,
                                    float* dmap, size_t dmap_pitch,
                                    const float* left, const float* right,
                                    int width, int height, size_t pitch,
                                    int patchsize, float depthmax, int iterations,
                                    int viewsamples, const cvtpm_trace* trace,
                                    void* stream);

/* Fixed-plane cost evaluator: the aggregated ASW cost
 * patch_eval_color_grad_weighted (pmhstereo.cl:170-228) of every pixel of
 * view `lr` (1 = left is image 1, 0 = right is image 1) for the given state
 * field (float4 s0,s1,s2,unused per pixel, x_other = s0*x + s1*y + s2).
 * img1/img2 are RGBA f32 device images; gradients are computed internally
 * (pmhstereo_gradxy, pmhstereo.cl:785-831).  cost is W*H floats.  states
 * must be 16-byte aligned and cost 4-byte aligned (CVTPM_ERR_INVALID_ARGUMENT
 * otherwise, before any launch). */
cvtpm_status cvtpm_cost_eval(cvtpm_ctx* ctx,
                             const float* img1, const float* img2,
                             int width, int height, size_t pitch,
                             const float* states, int lr, float* cost,
                             void* stream);

/* Adjoint of the aggregated cost (pmhstereo.cl:170-228) with respect to the
 * planes and both images; no counterpart in the reference, which never
 * differentiates its cost.  planes are per-pixel (a, b, c, unused), 16-byte
 * aligned, in the disparity convention d = a*x + b*y + c of view 1
 * (x_other = x - d for lr = 1, x + d for lr = 0).  cost (W*H, may be NULL)
 * receives the cost, evaluated in the FAST arithmetic (fixed-point tap
 * positions) whatever params.arith says.  With dcost (W*H, dL/dcost) given,
 * dplanes (W*H*4: dL/da, dL/db, dL/dc, 0), dimg1 and dimg2 (W*H*4 RGBA,
 * alpha 0) receive the gradients; each may be NULL.  Without dcost no
 * gradient may be requested.  Window weights are recomputed, not stored.
 * The image gradients are summed with float atomics, so their last bits vary
 * from run to run. */
cvtpm_status cvtpm_cost_adjoint(cvtpm_ctx* ctx,
                                const float* img1, const float* img2,
                                int width, int height, size_t pitch,
                                const float* planes, int lr,
                                const float* dcost,
                                float* cost, float* dplanes,
                                float* dimg1, float* dimg2, void* stream);

/* Plane polishing, no counterpart in the reference: `steps` Levenberg-
 * Marquardt trial steps per pixel on the plane (a, b, c, unused) of view lr
 * (convention of cvtpm_cost_adjoint), minimising its aggregated cost
 * (FAST evaluation, fixed-point taps).  The gradient is the adjoint's; the
 * curvature is the Gauss-Newton matrix of the truncated-L1 terms read as
 * reweighted least squares.  A step is kept only if the cost decreases, so
 * no pixel's cost grows; pixels without support (cost 1e5) are unchanged.
 * planes is updated in place (16-byte aligned); cost (W*H, may be NULL)
 * receives the final costs. */
cvtpm_status cvtpm_polish_planes(cvtpm_ctx* ctx, const float* img1, const float* img2,
                                 int width, int height, size_t pitch,
                                 float* planes, int lr, int steps, float* cost,
                                 void* stream);

/* Device memory the context may use for the propagation's shared-window
 * neighbour costs (FAST and EXACT): 32 bytes per pixel (the costs of the 8 neighbour
 * candidates).  Within the budget (and 60 % of the free memory) the 8
 * neighbour candidates of a pass are evaluated once per plane over the union
 * of their windows; otherwise per pixel.  Results are identical either way.
 * Default: no limit; 0 turns the shared windows off.  No counterpart in the
 * reference. */
cvtpm_status cvtpm_set_memory_budget(cvtpm_ctx* ctx, size_t bytes);

/* Enable CUDA-event timing of the propagation and PD phases (on the call's
 * stream); cvtpm_get_stats waits for the recorded events. */
cvtpm_status cvtpm_set_timing(cvtpm_ctx* ctx, int enable);
cvtpm_status cvtpm_reset_stats(cvtpm_ctx* ctx);
cvtpm_status cvtpm_get_stats(cvtpm_ctx* ctx, cvtpm_stats* out);

/* cvtpm_cost_eval without any device allocation and without a context.  No
 * counterpart in the reference: it serves callers that may not allocate
 * device memory (hosts that own every allocation through their own pool or
 * budget, real-time code that reserves memory up front) and can only pass
 * their own input and output buffers.  Its intermediate images live in a
 * fixed 16 MiB device array inside the library (present on every GPU that
 * loads it, until exit): width*height is limited to about 135 000 pixels
 * (366 x 366 is the largest square); larger images return CVTPM_ERR_SIZE.  The first call on
 * a device looks the array up (make it before any stream capture).  A call
 * whose color_weight or weight_profile differs from the previous call's on
 * that device uploads the spatial-profile table and synchronises `stream`
 * before it launches.  Calls share the array, so calls that overlap on the
 * GPU race; serialise them.  states must be 16-byte aligned and cost 4-byte
 * aligned (CVTPM_ERR_INVALID_ARGUMENT otherwise, before any launch).  Same
 * arguments and results as cvtpm_cost_eval, with the parameters passed
 * explicitly. */
cvtpm_status cvtpm_cost_eval_noalloc(const cvtpm_params* params,
                                     const float* img1, const float* img2,
                                     int width, int height, size_t pitch,
                                     const float* states, float* cost,
                                     void* stream);

/* PMHuberStereo::depthMap for many pairs of uneven size and disparity range
 * (pair.depthmax) in one CUDA-graph launch; no counterpart in the reference,
 * which handles one pair per call.  Each pair's result is bit-identical to
 * cvtpm_depthmap on that pair with the context's parameters (normal map and
 * trace are not produced).
 *
 * Default (lane count 0, Jacobi schedule): phase-batched.  Every phase of
 * the depthMap schedule (prep, init, per iteration the neighbour costs,
 * propagation and view lists of each view, the consistency checks, fills
 * and PD smoother steps, the final fill) is ONE launch covering all pairs:
 * persistent blocks walk a flat list of (pair, tile) work items, with the
 * pairs' arguments in the kernel parameter (up to 64 pairs per launch).  So
 * a batch takes the launches of one plain call, not one call per pair.  The
 * first call of a batch shape runs the autotuner on the batch's own data:
 * it times the propagation with persistent grids of 1 or 2 times the
 * resident blocks per SM or one block per work item, and the PD smoother
 * with 16- or 8-row tiles and 4 or 2 steps per launch (the steps are the
 * halo width of its shared-memory tile), and keeps the fastest of each;
 * the choice is cached per shape (widths, heights, disparity ranges and
 * parameters) in the context.  Each pair gets its own scratch.
 *
 * With a lane count k >= 1 (cvtpm_set_batch_lanes), or with the red/black
 * schedule: the pairs are spread over k lanes, each with its own scratch
 * and stream, and each pair's plain launch sequence is captured on its
 * lane's branch of the graph.
 *
 * Either graph is replayed while the context's parameters and the pair
 * descriptors (pointers, sizes, depthmax) stay the same.  Capture and tuning
 * synchronise `stream` once; replays do not. */
cvtpm_status cvtpm_depthmap_batched(cvtpm_ctx* ctx, const cvtpm_pair* pairs,
                                    int npairs, void* stream);

#define CVTPM_BATCH_MAX_CAND 16
typedef struct cvtpm_batch_info {
    int lanes;                 /* lanes of the current graph (0: phase-batched) */
    int shared_windows;        /* shared-window neighbour costs in use for every pair */
    int tuned;                 /* 1 if the autotuner ran for the current graph */
    int ncand;
    int cand_lanes[CVTPM_BATCH_MAX_CAND];     /* lane count of a lane candidate, 0 for a phase-batched one */
    float cand_ms[CVTPM_BATCH_MAX_CAND];      /* its timed proxy: a one-iteration batch (lanes), one
                                                 propagation phase or one 8-step PD apply (phase-batched) */
    long long graph_nodes;
    long long replays;
    int phased;                /* 1: phase-batched graph */
    int grid_mult;             /* chosen persistent grid (x resident blocks per SM; 0: a block per item) */
    int pd_rows;               /* chosen PD tile height */
    int pd_halo;               /* chosen PD steps per launch (= halo width) */
    int cand_grid_mult[CVTPM_BATCH_MAX_CAND];
    int cand_pd_rows[CVTPM_BATCH_MAX_CAND];
    int cand_pd_halo[CVTPM_BATCH_MAX_CAND];
    long long launches;        /* kernel launches in the phase-batched graph */
    float tune_ms;             /* host time the last tuning took */
    float mode_ms[2];          /* the mode proxies of the last tuning (ms; 0: not run): the tuning subset for one
                                  iteration, [0] phase-batched with the chosen knobs, [1] one lane */
} cvtpm_batch_info;

/* The lane count of cvtpm_depthmap_batched: 0 (default) lets the autotuner
 * choose between the phase-batched launches and one lane of per-pair launch
 * sequences (mode_ms: the phase-batched schedule is taken when its proxy is
 * at least 3 % faster); k >= 1 fixes k lanes of per-pair launch sequences. */
cvtpm_status cvtpm_set_batch_lanes(cvtpm_ctx* ctx, int lanes);
/* Pin the phase-batched launch knobs instead of tuning them: grid_mult 0
 * (a block per work item), 1 or 2 (persistent grid of that many times the
 * resident blocks per SM); pd_rows 16 or 8; pd_halo 4 or 2.  grid_mult -1
 * returns to autotuning.  Results never depend on the knobs. */
cvtpm_status cvtpm_set_batch_knobs(cvtpm_ctx* ctx, int grid_mult, int pd_rows, int pd_halo);
cvtpm_status cvtpm_get_batch_info(const cvtpm_ctx* ctx, cvtpm_batch_info* out);

/* ------------------------------------------------------------------
 * Input side: the reference's image formats and files.
 *
 * cvt::PMHuberStereo::depthMap accepts left/right cvt::Image objects of any
 * format backed by OpenCL images (PMHuberStereo.cpp:64-68 checks only sizes
 * and the memory type; the two may differ in format); its kernels read them
 * with read_imagef, which returns RGBA floats.  The identifiers below are
 * cvt::IFormatID (cvt/gfx/IFormat.h:36-63) and each is read the way its
 * OpenCL image format (IFormat::toCLImageFormat, IFormat.h:293-328) makes
 * read_imagef return it:
 *   GRAY_*, BAYER_*  CL_INTENSITY  (I, I, I, I)
 *   GRAYALPHA_*      CL_RG         (R, G, 0, 1)
 *   RGBA_*           CL_RGBA       (R, G, B, A)
 *   BGRA_*           CL_BGRA       stored B, G, R, A; returned (R, G, B, A)
 *   YUYV, UYVY       CL_RA         (R, 0, 0, A): byte 0 and byte 1 of a pixel
 * with UINT8 = CL_UNORM_INT8 (c / 255), UINT16 = CL_UNORM_INT16
 * (c / 65535), INT16 = CL_SNORM_INT16 (max(-1, c / 32767)), FLOAT as is
 * (OpenCL 1.2, 8.3.1.1; the division is correctly rounded).  16-bit
 * channels are in host byte order.
 * ------------------------------------------------------------------ */
enum {
    CVTPM_IFORMAT_GRAY_UINT8 = 1, CVTPM_IFORMAT_GRAY_UINT16, CVTPM_IFORMAT_GRAY_INT16, CVTPM_IFORMAT_GRAY_FLOAT,
    CVTPM_IFORMAT_GRAYALPHA_UINT8, CVTPM_IFORMAT_GRAYALPHA_UINT16, CVTPM_IFORMAT_GRAYALPHA_INT16,
    CVTPM_IFORMAT_GRAYALPHA_FLOAT,
    CVTPM_IFORMAT_RGBA_UINT8, CVTPM_IFORMAT_RGBA_UINT16, CVTPM_IFORMAT_RGBA_INT16, CVTPM_IFORMAT_RGBA_FLOAT,
    CVTPM_IFORMAT_BGRA_UINT8, CVTPM_IFORMAT_BGRA_UINT16, CVTPM_IFORMAT_BGRA_INT16, CVTPM_IFORMAT_BGRA_FLOAT,
    CVTPM_IFORMAT_BAYER_RGGB_UINT8, CVTPM_IFORMAT_BAYER_GRBG_UINT8, CVTPM_IFORMAT_BAYER_GBRG_UINT8,
    CVTPM_IFORMAT_YUYV_UINT8, CVTPM_IFORMAT_UYVY_UINT8
};

/* A cvt::Image's storage: format, size and row stride in bytes.  `data` is
 * device memory for the conversion and depthMap calls, host memory for the
 * file readers and writers. */
typedef struct cvtpm_image {
    int format;             /* CVTPM_IFORMAT_* */
    int width, height;
    size_t stride;          /* bytes per row, >= width * bytes per pixel */
    void* data;
} cvtpm_image;

/* Bytes per pixel of a format (0 for an unknown one). */
size_t cvtpm_iformat_bpp(int format);

/* src (device) as read_imagef sees it, into RGBA float32 rows of dst_pitch
 * bytes (a multiple of 16).  No counterpart function in the reference: there
 * the OpenCL image sampler does this on every read. */
cvtpm_status cvtpm_image_to_rgbaf(const cvtpm_image* src, float* dst, size_t dst_pitch, void* stream);

/* PMHuberStereo::depthMap with left/right in any of the formats above
 * (device memory; formats may differ, sizes may not).  The images are
 * converted into context scratch, then the call is cvtpm_depthmap's. */
cvtpm_status cvtpm_depthmap_image(cvtpm_ctx* ctx,
                                  float* dmap, size_t dmap_pitch,
                                  const cvtpm_image* left, const cvtpm_image* right,
                                  int patchsize, float depthmax, int iterations,
                                  int viewsamples, float dscale,
                                  float* normalmap, size_t normalmap_pitch,
                                  const cvtpm_trace* trace, void* stream);

/* Files (host memory).  Readers fill the descriptor in two steps: with
 * img->data == NULL they set format, width, height and the stride of a tight
 * copy (width * bytes per pixel) and return; then, with data pointing to
 * height * stride bytes, they read the pixels.
 *
 * CVTRaw (plugins/iloader/CVTRaw/CVTRawLoader.cpp,
 * plugins/isaver/CVTRaw/CVTRawSaver.cpp): a header of four uint32 in host
 * byte order, width, height, stride and IFormatID, then height rows of
 * `stride` bytes. */
cvtpm_status cvtpm_raw_read(const char* path, cvtpm_image* img);
cvtpm_status cvtpm_raw_write(const char* path, const cvtpm_image* img);

/* PPM / PGM (plugins/iloader/PPM/PPMLoader.cpp): P2 and P5 (gray) read as
 * GRAY_UINT8, P3 and P6 (RGB) as RGBA_UINT8 with alpha 255; lines starting
 * with '#' are comments; maximum values above 255 are refused
 * (CVTPM_ERR_NOT_SUPPORTED), as in the reference, whose 16-bit formats have
 * no reader. */
cvtpm_status cvtpm_ppm_read(const char* path, cvtpm_image* img);

/* PFM (plugins/isaver/PFM/PFMSaver.cpp): GRAY_FLOAT as "Pf", RGBA_FLOAT and
 * BGRA_FLOAT as "PF" with the alpha channel dropped (BGRA written in its
 * stored order, as the reference's alpha stripping keeps the channel order);
 * rows bottom to top; scale -1.0 on little-endian hosts.  Other formats:
 * CVTPM_ERR_NOT_SUPPORTED. */
cvtpm_status cvtpm_pfm_write(const char* path, const cvtpm_image* img);

/* PNG (plugins/iloader/PNG/PNGLoader.cpp, plugins/isaver/PNG/PNGSaver.cpp;
 * no libpng: the zlib/DEFLATE streams are decoded and encoded here).  Read
 * in the two-call protocol above: gray 1-8 bit -> GRAY_UINT8 (low depths
 * scaled), gray 16 -> GRAY_UINT16, gray+alpha -> GRAYALPHA_UINT8/16, RGB 8
 * and palette -> RGBA_UINT8, RGB 16 -> RGBA_UINT16 (alpha 255 as the
 * reference's 0xff filler), RGBA -> RGBA_UINT8/16; a tRNS chunk becomes the
 * alpha channel (gray + tRNS -> GRAYALPHA); Adam7 interlacing is undone;
 * 16-bit samples in host order.  Unsupported PNG types give
 * CVTPM_ERR_NOT_SUPPORTED, corrupt files (bad CRC, Adler-32, codes)
 * CVTPM_ERR_IO. */
cvtpm_status cvtpm_png_read(const char* path, cvtpm_image* img);
/* Writes GRAY, GRAYALPHA, RGBA or BGRA (as RGBA) host images of 8 or 16
 * bits; float images are converted to 8 bits as the reference's
 * Image::convert: colour and gray through cvtpm_float_to_srgb_u8, alpha and
 * GRAYALPHA_FLOAT channels as (uint8)(clamp(v * 255 + 0.5, 0, 255)).  Other
 * formats: CVTPM_ERR_NOT_SUPPORTED. */
cvtpm_status cvtpm_png_write(const char* path, const cvtpm_image* img);
/* The reference's float-to-8-bit sRGB conversion (F_TO_SRGB_U8,
 * cvt/util/SIMD.cpp): the table entry round(255 * sRGB(i / 8192)) at
 * i = (int)(v * 8192), 0 below 0 (and for NaN), 255 from 1 on. */
uint8_t cvtpm_float_to_srgb_u8(float v);

/* ------------------------------------------------------------------
 * Input side: stereo rectification (cvt/vision/StereoCameraCalibration.h,
 * cvt/vision/StereoRectification.h, cvt/gfx/ifilter/IWarp.cpp).
 * ------------------------------------------------------------------ */

/* A camera of cvt::CameraCalibration: intrinsics and lens distortion. */
typedef struct cvtpm_camera {
    float intrinsics[9];    /* row-major 3x3: fx, skew, cx / 0, fy, cy / 0, 0, 1 */
    float radial[3];        /* k1, k2, k3 */
    float tangential[2];    /* p1, p2 */
} cvtpm_camera;

/* What StereoCameraCalibration::undistortRectify produces besides the maps. */
typedef struct cvtpm_rectification {
    cvtpm_camera first, second;  /* rectified cameras: common focal length, no distortion */
    float extrinsics[16];        /* rectified stereo extrinsics (row-major 4x4) */
    float rot_first[9];          /* rectifying rotations (row-major), as  */
    float rot_second[9];         /* rectificationMatrices returns them    */
} cvtpm_rectification;

/* StereoCameraCalibration(first, second, extrinsics).undistortRectify(out,
 * warp_first, warp_second, width, height, vertical)
 * (StereoCameraCalibration.h:124-130, 166-277): `extrinsics` is the stereo
 * extrinsics (row-major 4x4, the pose of the second camera relative to the
 * first, as StereoCameraCalibration stores and loads it).  The rectified
 * calibration is computed on the host; with warp_first / warp_second non-NULL
 * the two warp maps (IFormat::GRAYALPHA_FLOAT, width x height, rows of
 * warp_pitch bytes: per output pixel the (x, y) to sample the source at) are
 * written on the device, stream-ordered on `stream`.  As in the reference,
 * the rectifying rotations are always those of horizontal stereo
 * (undistortRectify calls rectificationMatrices without its `verticalstereo`
 * flag); `vertical` only selects which principal-point coordinate the two
 * cameras share. */
cvtpm_status cvtpm_stereo_rectify(const cvtpm_camera* first, const cvtpm_camera* second, const float* extrinsics,
                                  int vertical, cvtpm_rectification* out, int width, int height,
                                  float* warp_first, float* warp_second, size_t warp_pitch, void* stream);

/* IWarp::apply(dst, src, warp) (cvt/gfx/ifilter/IWarp.cpp:49-66, 254-376):
 * dst (warp's size, src's format) = src resampled at the warp map's (x, y),
 * bilinear, with the reference's fill outside the image.  Formats:
 * GRAY_FLOAT (fill 0), RGBA_FLOAT / BGRA_FLOAT (fill 0, 0, 0, 1), GRAY_UINT8
 * (fill 0, 16-bit fixed-point weights), RGBA_UINT8 / BGRA_UINT8 (fill
 * opaque black, 8-bit fixed-point weights).  Map coordinates that are not
 * finite or beyond the fixed-point range (|x|, |y| >= 32768 for GRAY_UINT8,
 * >= 2^23 for the 4-channel 8-bit formats, >= 2^31 for float) give the fill
 * value (the reference's float-to-int conversion is undefined there).  All
 * device memory. */
cvtpm_status cvtpm_warp_apply(const cvtpm_image* dst, const cvtpm_image* src, const float* warp, size_t warp_pitch,
                              void* stream);

/* ------------------------------------------------------------------
 * Output side: TSDF fusion of depth maps (cvt::TSDFVolume,
 * cvt/vision/TSDFVolume.h, TSDFVolume.cpp; kernels
 * cvt/cl/kernel/TSDFVolume/TSDFVolume.cl).  Matrices are row-major 4x4
 * (cvt::Matrix4f).  The volume is width*height*depth float2 (tsdf, weight) in
 * device memory, x fastest.
 * ------------------------------------------------------------------ */
typedef struct cvtpm_tsdf cvtpm_tsdf;

/* TSDFVolume(gridtoworld, width, height, depth, truncation)
 * (TSDFVolume.cpp:31-45); the volume is not cleared (call cvtpm_tsdf_clear). */
cvtpm_status cvtpm_tsdf_create(cvtpm_tsdf** vol, int device, const float* grid_to_world,
                               int width, int height, int depth, float truncation);
cvtpm_status cvtpm_tsdf_destroy(cvtpm_tsdf* vol);
/* Size and the device pointer of the volume. */
cvtpm_status cvtpm_tsdf_info(const cvtpm_tsdf* vol, int* width, int* height, int* depth, void** data);
/* clear(weight) (:47-58): every voxel (1, weight). */
cvtpm_status cvtpm_tsdf_clear(cvtpm_tsdf* vol, float weight, void* stream);
/* The projection of addDepthMap / rayCastDepthMap from intrinsics (3x3) and
 * extrinsics (4x4): intrinsics.toMatrix4() * extrinsics (:79-84, :87-92). */
cvtpm_status cvtpm_tsdf_projection(const float* intrinsics, const float* extrinsics, float* proj);
/* Vision::disparityToDepthmap(depthmap, disparity, dispscale, focallength,
 * baseline, dispthres) (cvt/vision/Vision.cpp:147-168), the step between
 * depthMap and addDepthMap: depth = (focallength * baseline) / (disparity *
 * dispscale) where the scaled disparity exceeds dispthres (the reference's
 * default 0.01), else 0.  GRAY_FLOAT images on the device, rows of the given
 * pitches in bytes.  With depthMap's default dscale (1 / depthmax), pass
 * dispscale = depthmax. */
cvtpm_status cvtpm_disparity_to_depth(float* depth, size_t depth_pitch, const float* disparity, size_t disp_pitch,
                                      int width, int height, float dispscale, float focallength, float baseline,
                                      float dispthres, void* stream);
/* addDepthMap(proj, depthmap, scale) (:61-77): depth map GRAY_FLOAT on the
 * device (rows of dpitch bytes), depth = value * scale. */
cvtpm_status cvtpm_tsdf_add_depthmap(cvtpm_tsdf* vol, const float* proj, const float* depthmap,
                                     int dwidth, int dheight, size_t dpitch, float scale, void* stream);
/* rayCastDepthMap(depthmap, proj, scale) (:94-110): depth of the first
 * surface along each pixel's ray, 0 where there is none.  A ray whose march
 * cannot advance in float (a camera about 2^24 voxels from the volume) stops
 * after 2 * max(width, height, depth) + 16 steps with 0, where the
 * reference's loop does not end. */
cvtpm_status cvtpm_tsdf_raycast(cvtpm_tsdf* vol, const float* proj, float* depthmap,
                                int dwidth, int dheight, size_t dpitch, float scale, void* stream);
/* The slice kernels TSDFVolume_sliceX/Y/Z (axis 0/1/2, plane `index`) into
 * RGBA float rows of `pitch` bytes: (c, c, c, 1), c = clamp(tsdf + 0.5, 0, 1);
 * the image is height x depth (x), width x depth (y) or width x height (z).
 * (The reference's host functions sliceX/Y/Z are empty.) */
cvtpm_status cvtpm_tsdf_slice(cvtpm_tsdf* vol, int axis, int index, float* rgba, size_t pitch, void* stream);
/* saveRaw(path, weighted) (:130-152): (tsdf, weight) pairs or the tsdf
 * values alone; synchronizes the device. */
cvtpm_status cvtpm_tsdf_save_raw(cvtpm_tsdf* vol, const char* path, int weighted);

/* ------------------------------------------------------------------
 * The comparison baseline: cvt::StereoGCVFilter
 * (cvt/gfx/ifilter/StereoGCVFilter.cpp), cost-volume stereo with a
 * colour-guided filter over integral images.  Images are tight RGBA float
 * rows on the device (pitch = width * 16).  The depth is normalised:
 * |d - dmin| / |dmax - dmin| for the best d of dmin, dmin + dt, ... (0 where
 * no cost fell below its start).  As in the reference, the map belongs to
 * cam1 and its match in cam0 lies at x - d: with a left/right pair, pass the
 * right image as cam0 and the left as cam1 for the left view's disparity.
 * The disparities are processed in batches; scratch is (22 + 10 x batch)
 * floats per pixel (2 more for apply), allocated on the call's stream from a
 * stream-ordered memory pool of the library's and returned to it when the
 * call's kernels end (the pool keeps the memory for later calls).  Calls are
 * stream-ordered.  The batch does not change results.
 * ------------------------------------------------------------------ */

/* Disparities per batch for later calls: 0 (the default) takes as many as
 * 4 GiB of scratch holds, at most 256; 1..256 sets it.  Process-wide. */
cvtpm_status cvtpm_gcv_set_batch(int disparities);

/* The scratch pool keeps what its largest call reserved (22 + 10 x batch
 * floats per pixel per call in flight: about 1.9 GB for an apply at
 * 1242x375 with the automatic batch of 128 disparities) until the process
 * exits.  This returns the unused part beyond keep_bytes to the device
 * (cudaMemPoolTrimTo); later calls reserve again.  No counterpart in the
 * reference. */
cvtpm_status cvtpm_gcv_trim(int device, size_t keep_bytes);

/* The plan of a depthmap call of these arguments: the number of
 * disparities, the batch, the scratch bytes and the kernel launches (each
 * optional).  An apply call runs two such depth maps and one more launch. */
cvtpm_status cvtpm_gcv_plan(int width, int height, float dmin, float dmax, float dt, int* steps, int* batch,
                            size_t* scratch_bytes, int* launches);

/* StereoGCVFilter::depthmap(dst, cam0, cam1, dmin, dmax, dt) (:97-242). */
cvtpm_status cvtpm_gcv_depthmap(float* dst, size_t dst_pitch, const float* cam0, const float* cam1,
                                int width, int height, size_t pitch, float dmin, float dmax, float dt,
                                void* stream);

/* StereoGCVFilter::apply(dst, cam0, cam1, dmin, dmax, dt) (:75-95): both
 * views' depth maps (d0, d1 tight float rows, or NULL) and their
 * consistency check into a GRAY_UINT8 image (CL_UNORM_INT8 write:
 * convert_uchar_sat_rte(v * 255)).  The reference also saves d0 and d1 as
 * PNG files; that is not done. */
cvtpm_status cvtpm_gcv_apply(uint8_t* dst, size_t dst_pitch, float* d0, float* d1, size_t dpitch,
                             const float* cam0, const float* cam1, int width, int height, size_t pitch,
                             float dmin, float dmax, float dt, void* stream);

#ifdef __cplusplus
}
#endif
#endif
