/*
 * pm_kernels.cuh — launch interface between the host schedule (pm_capi.cu)
 * and the kernels (pm_kernels.cu).
 */
#ifndef CVT_GB300_PM_KERNELS_CUH
#define CVT_GB300_PM_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "cvtpm.h"
#include "pm_device.cuh"

/* Everything one init / propagation / cost launch needs. */
struct PmPassArgs {
    PmCostConsts k;
    PmView v1, v2;             /* v1: the view being estimated; v2: the other view */
    int lr, iter, rng;
    uint32_t key0, key1;
    float depthmax, theta;
    const float4* old;         /* previous states of v1            */
    const float4* smooth;      /* PD-smoothed (nx, ny, d/dmax, 1)  */
    const short4* viewin;      /* up to 4 source x per pixel, or NULL */
    const float4* viewsrc;     /* states the view list refers to    */
    float4* out;
    uint8_t* winners;
    unsigned long long* counters;   /* [0] cost evaluations, [1] in-image taps; may be NULL */
    float* nbcost;             /* FAST: costs of candidates 1-8 by shared windows, [8][W*H], or NULL */
    int color;                 /* -1: every pixel (Jacobi); 0 / 1: pixels with (x + y) & 1 == color */
};

/* ------------------------------------------------------------------
 * Batched launches (cvtpm_depthmap_batched).  One launch runs one phase of
 * the depthMap schedule for many pairs: its blocks walk a flat list of work
 * items, pair i owning items first[i] .. first[i+1]-1, whose item t is the
 * tile (t % tx[i], t / tx[i]) of that pair (a row, for the row-scan
 * kernels).  Blocks are persistent: block b takes items b, b + gridDim.x,
 * ...  The pairs' arguments travel in the kernel parameter (at most
 * PM_BATCH_MAX pairs per launch), read through a block-uniform index.
 * ------------------------------------------------------------------ */
#define PM_BATCH_MAX 64

template <typename A>
struct PmBatch {
    int n;                          /* pairs of this launch */
    int first[PM_BATCH_MAX + 1];    /* first item of each pair; first[n] = items */
    int tx[PM_BATCH_MAX];           /* tiles per row of each pair */
    A a[PM_BATCH_MAX];
};

struct PmPrepArgs { const float4* img; size_t pitch4; int W, H; float4* col; float4* grad; float* wgt; };
struct PmRecArgs { const float4* col; const float4* grad; int W, H, rp; float4 *A, *B, *C; float2* D; };
struct PmViewListArgs { const float4* src; int W, H; short4* list; };
struct PmConsArgs { const float4 *L, *R; int W, H; float maxdisp, athr; int lr; float4* out; uint8_t* valid; };
struct PmFillArgs { const float4* in; int W, H; float depthmax; int lr; float4* out; };
struct PmOutArgs { const float4* in; int W, H; float scale; float* dmap; size_t dpitch; float4* nmap; size_t npitch; };
struct PmPdArgs {
    float4 *uout, *pout;
    const float4 *uin, *pin, *f;
    const float* wgt;
    int pzero, nsteps, W, H;
    float lambda;
};

/* Launch knobs the batch autotuner chooses. */
struct PmBatchKnobs {
    int grid_mult;     /* persistent grid: this many x the blocks resident per SM x the SMs; 0 = one block per item */
    int pd_rows;       /* PD tile height: 16 or 8 */
    int pd_halo;       /* PD steps per launch, which is also the tile's halo width: 4 or 2 */
};

/* Tile geometry of each batched kernel (items per pair = tiles). */
enum PmBatchKernel { PMB_PREP, PMB_RECORDS, PMB_PIXEL, PMB_NBCOST, PMB_ROW, PMB_PD };
void pm_batch_tiles(PmBatchKernel k, int W, int H, const PmBatchKnobs& kn, int* tx, int* tiles);

cudaError_t pm_batch_prep(const PmBatch<PmPrepArgs>& b, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_records(const PmBatch<PmRecArgs>& b, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_init(const PmBatch<PmPassArgs>& b, bool exact, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_nbcost(const PmBatch<PmPassArgs>& b, bool exact, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_propagate(const PmBatch<PmPassArgs>& b, bool exact, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_view_list(const PmBatch<PmViewListArgs>& b, int maxW, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_consistency(const PmBatch<PmConsArgs>& b, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_fill_state(const PmBatch<PmFillArgs>& b, int maxW, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_pd(const PmBatch<PmPdArgs>& b, const PmBatchKnobs& kn, cudaStream_t st);
cudaError_t pm_batch_fill_output(const PmBatch<PmOutArgs>& b, int maxW, const PmBatchKnobs& kn, cudaStream_t st);
/* Shared-memory limits of the batched PD kernels; once per device before
 * the first launch or capture. */
cudaError_t pm_batch_prepare_kernels();

cudaError_t pm_upload_tables(const unsigned long long* pow2, const float* prof, cudaStream_t st);
cudaError_t pm_launch_prep(const float4* img, size_t pitch4, int W, int H, float4* col, float4* grad,
                           float* wgt, cudaStream_t st);
cudaError_t pm_launch_records(const float4* col, const float4* grad, int W, int H, int rp, float4* A, float4* B,
                              float4* C, float2* D, cudaStream_t st);
cudaError_t pm_launch_init(const PmPassArgs& a, bool exact, cudaStream_t st);
cudaError_t pm_launch_cost_field(const PmPassArgs& a, bool exact, const float4* states, float* cost,
                                 cudaStream_t st);
cudaError_t pm_launch_propagate(const PmPassArgs& a, bool exact, cudaStream_t st);
cudaError_t pm_launch_view_list(const float4* src, int W, int H, short4* list, cudaStream_t st);
cudaError_t pm_launch_consistency(const float4* L, const float4* R, int W, int H, float maxdisp,
                                  float maxangle, int lr, float4* out, uint8_t* valid, cudaStream_t st);
cudaError_t pm_launch_fill_state(const float4* in, int W, int H, float depthmax, int lr, float4* out,
                                 cudaStream_t st);
cudaError_t pm_launch_fill_output(const float4* in, int W, int H, float scale, float* dmap, size_t dpitch,
                                  float4* nmap, size_t npitch, cudaStream_t st);
/* mask == NULL: PDHuberWeighted; else PDHuberWeightedInpaint with lambda * mask. */
cudaError_t pm_launch_pd_step(float4* uout, float4* pout, const float4* last, const float4* pin,
                              const float4* f, const float* wgt, const float* mask, float lambda, int W, int H,
                              cudaStream_t st);
cudaError_t pm_launch_occmap(const float4* L, const float4* R, int W, int H, float maxdiff, int lr, float* mask,
                             cudaStream_t st);
cudaError_t pm_launch_normal_depth(const float4* in, int W, int H, float depthmax, int lr, float4* out,
                                   cudaStream_t st);

/* Kernel attributes (dynamic shared memory limits) for the current device;
 * call once per device before the first launch or stream capture. */
cudaError_t pm_prepare_kernels();

int pm_pd_block_steps();
cudaError_t pm_launch_pd_block(float4* uout, float4* pout, const float4* uin, const float4* pin, int pzero,
                               const float4* f, const float* wgt, const float* mask, float lambda, int nsteps, int W,
                               int H, cudaStream_t st);
cudaError_t pm_launch_ffma_peak(float* out, int blocks, int iters, cudaStream_t st);

/* pm_adjoint.cu */
cudaError_t pm_adjoint_upload_profile(const float* prof, cudaStream_t st);
cudaError_t pm_launch_cost_adjoint(const PmCostConsts& k, const PmView& v1, const PmView& v2, const float4* planes,
                                   int lr, const float* dcost, float* cost, float4* dplanes, float4* dI1, float4* dG1,
                                   float4* dI2, float4* dG2, cudaStream_t st);
cudaError_t pm_launch_adjoint_finish(const float4* dI, const float4* dG, int W, int H, float* out, cudaStream_t st);
cudaError_t pm_launch_gn_polish(const PmCostConsts& k, const PmView& v1, const PmView& v2, float4* planes, int lr,
                                int steps, float* cost, cudaStream_t st);

/* pm_image.cu: one image in a cvt::IFormat (validated) into RGBA float32 rows
 * of dst_pitch bytes; *msg receives the reason of a failure. */
cvtpm_status pm_image_to_rgbaf_checked(const cvtpm_image* img, const char* what, float4* dst, size_t dst_pitch,
                                       cudaStream_t st, std::string* msg);
/* The calling thread's last error message of a context-free entry point. */
const char* pm_free_error();
void pm_set_free_error(const std::string& m);

#endif
