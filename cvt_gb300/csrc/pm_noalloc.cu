/*
 * pm_noalloc.cu — cvtpm_cost_eval_noalloc: the fixed-plane cost evaluator
 * (the same computation as cvtpm_cost_eval) for callers that must not
 * allocate device memory.
 *
 * Who needs it: code that runs where cudaMalloc is forbidden or unsafe —
 * inside a host that owns every device allocation through its own pool or
 * budget (plugin hosts, real-time pipelines that pre-reserve memory at start
 * and treat any later allocation as a failure), or code that must not create
 * a context object at all.  Such a caller hands over its input and output
 * buffers and nothing else.
 *
 * How: the intermediate images the evaluator needs (colour and gradient of
 * both views, the edge-weight image and the other view's interpolation
 * records) live in one file-scope device array of PM_NOALLOC_SCRATCH_BYTES
 * (16 MiB).  That array exists on every GPU that loads the library, from load
 * until process exit.  Host code cannot use the array's name as a device
 * address, so the first call on a device (with that device current) asks the
 * runtime for the address with cudaGetSymbolAddress and keeps it; make that
 * first call before any stream capture.  This unit also keeps its own copy of
 * the spatial-profile table in constant memory and uploads it when the
 * parameters change, so it never touches the tables of the context-based
 * entry points.
 *
 * Limits: width*height must fit the scratch (about 124 bytes per pixel, so
 * roughly 135 000 pixels, e.g. 360 x 360); larger images return
 * CVTPM_ERR_SIZE before anything is launched.  All calls on a device share
 * the one array and the one table: calls that overlap on the GPU (different
 * streams, or threads without ordering) race and must be serialised by the
 * caller.  Every byte a call reads from the scratch is written earlier in
 * the same call, so nothing needs clearing between calls.
 */
#include <cstring>
#include <mutex>

#define PM_KERNELS_TU 1
#include "cvtpm.h"
#include "pm_kernels.cuh"

#define PM_NOALLOC_SCRATCH_BYTES (16u << 20)
#define PM_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[PM_NOALLOC_SCRATCH_BYTES];

namespace {

struct NoallocDevice {
    bool ready;            /* scratch address looked up */
    void* scratch;         /* device address of g_noalloc_scratch */
    bool table_ok;
    float table_cw;
    int table_prof;
};
NoallocDevice g_dev[PM_NOALLOC_MAX_DEVICES];
std::mutex g_mu;
float g_prof_host[PM_PROF_N * PM_PROF_N];

size_t up256(size_t v) { return (v + 255) / 256 * 256; }
int noalloc_rec_pitch(int W) { return (int)(((size_t)W + 2 + 3) / 4 * 4); }

/* bytes of scratch a W x H evaluation needs, and the layout */
struct Layout {
    size_t col0, col1, grad0, grad1, wgt, recA, recB, recC, recD, end;
};
Layout layout(int W, int H) {
    const size_t n = (size_t)W * H, nr = (size_t)noalloc_rec_pitch(W) * H;
    Layout L;
    size_t o = 0;
    L.col0 = o; o = up256(o + n * 16);
    L.col1 = o; o = up256(o + n * 16);
    L.grad0 = o; o = up256(o + n * 16);
    L.grad1 = o; o = up256(o + n * 16);
    L.wgt = o; o = up256(o + n * 4);
    L.recA = o; o = up256(o + nr * 16);
    L.recB = o; o = up256(o + nr * 16);
    L.recC = o; o = up256(o + nr * 16);
    L.recD = o; o = up256(o + nr * 8);
    L.end = o;
    return L;
}

/* The aggregated cost of a fixed state field, on this unit's tables. */
template <bool EXACT>
__global__ void __launch_bounds__(256) k_cost_field_noalloc(PmPassArgs a, const float4* __restrict__ states,
                                                           float* __restrict__ cost) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= a.k.W || y >= a.k.H) return;
    float4 s[1] = {states[(size_t)y * a.k.W + x]};
    bool act[1] = {true};
    float c[1];
    eval_costs<1, EXACT>(a.k, a.v1, a.v2, x, y, s, act, c);
    cost[(size_t)y * a.k.W + x] = c[0];
}

bool params_ok(const cvtpm_params* p) {
    return p->patchsize >= 1 && p->patchsize <= PM_PMAX &&
           (p->arith == CVTPM_ARITH_EXACT || p->arith == CVTPM_ARITH_FAST) &&
           (p->weight_profile == CVTPM_PROFILE_SMOOTHSTEP || p->weight_profile == CVTPM_PROFILE_CONSTANT);
}

bool image_ok(const void* ptr, int W, size_t pitch) {
    return ptr && ((uintptr_t)ptr & 15) == 0 && pitch % 16 == 0 && pitch >= (size_t)W * 16;
}

}  // namespace

extern "C" cvtpm_status cvtpm_cost_eval_noalloc(const cvtpm_params* params, const float* img1, const float* img2,
                                                int width, int height, size_t pitch, const float* states,
                                                float* cost, void* stream) {
    if (!params || !states || !cost) return CVTPM_ERR_INVALID_ARGUMENT;
    /* the kernel reads the states as float4 and writes the costs as float */
    if (((uintptr_t)states & 15) || ((uintptr_t)cost & 3)) return CVTPM_ERR_INVALID_ARGUMENT;
    if (!params_ok(params)) return CVTPM_ERR_INVALID_ARGUMENT;
    if (width < 1 || height < 1 || width > 12288 || height > 65535) return CVTPM_ERR_SIZE;
    if (!image_ok(img1, width, pitch) || !image_ok(img2, width, pitch)) return CVTPM_ERR_INVALID_ARGUMENT;
    const Layout L = layout(width, height);
    if (L.end > PM_NOALLOC_SCRATCH_BYTES) return CVTPM_ERR_SIZE;   /* image too large for the static scratch */
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CVTPM_ERR_CUDA;
    if (dev < 0 || dev >= PM_NOALLOC_MAX_DEVICES) return CVTPM_ERR_NOT_SUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    char* base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        NoallocDevice& d = g_dev[dev];
        if (!d.ready) {                          /* first call on this device: find the array */
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return CVTPM_ERR_CUDA;
            d.scratch = ptr;
            d.ready = true;
        }
        if (!d.table_ok || d.table_cw != params->color_weight || d.table_prof != params->weight_profile) {
            for (int dy = -PM_PMAX; dy <= PM_PMAX; ++dy)
                for (int dx = -PM_PMAX; dx <= PM_PMAX; ++dx)
                    g_prof_host[(dy + PM_PMAX) * PM_PROF_N + (dx + PM_PMAX)] =
                        pm_profile(dx, dy, params->color_weight, params->weight_profile);
            if (cudaMemcpyToSymbolAsync(c_prof, g_prof_host, sizeof(g_prof_host), 0, cudaMemcpyHostToDevice, st) !=
                cudaSuccess)
                return CVTPM_ERR_CUDA;
            if (cudaStreamSynchronize(st) != cudaSuccess) return CVTPM_ERR_CUDA;
            d.table_ok = true;
            d.table_cw = params->color_weight;
            d.table_prof = params->weight_profile;
        }
        base = (char*)d.scratch;
    }
    const int W = width, H = height, rp = noalloc_rec_pitch(W);
    float4* col[2] = {(float4*)(base + L.col0), (float4*)(base + L.col1)};
    float4* grad[2] = {(float4*)(base + L.grad0), (float4*)(base + L.grad1)};
    float* wgt = (float*)(base + L.wgt);
    float4* recA = (float4*)(base + L.recA);
    float4* recB = (float4*)(base + L.recB);
    float4* recC = (float4*)(base + L.recC);
    float2* recD = (float2*)(base + L.recD);
    const float* im[2] = {img1, img2};
    for (int v = 0; v < 2; ++v)
        if (pm_launch_prep((const float4*)im[v], pitch / 16, W, H, col[v], grad[v], wgt, st) != cudaSuccess)
            return CVTPM_ERR_CUDA;
    const bool exact = params->arith == CVTPM_ARITH_EXACT;
    if (!exact && pm_launch_records(col[1], grad[1], W, H, rp, recA, recB, recC, recD, st) != cudaSuccess)
        return CVTPM_ERR_CUDA;
    PmPassArgs a;
    memset(&a, 0, sizeof(a));
    a.k.W = W; a.k.H = H; a.k.P = params->patchsize;
    a.k.Wf = (float)W; a.k.Hf = (float)H;
    a.k.alpha = params->color_alpha; a.k.oma = 1.0f - params->color_alpha;
    a.k.cmax = params->color_maxdiff; a.k.gmax = params->grad_maxdiff;
    a.k.rp = rp;
    a.v1 = {col[0], grad[0], nullptr, nullptr, nullptr, nullptr};
    a.v2 = {col[1], grad[1], recA, recB, recC, recD};
    dim3 grid((W + 31) / 32, (H + 7) / 8), block(32, 8);
    if (exact) k_cost_field_noalloc<true><<<grid, block, 0, st>>>(a, (const float4*)states, cost);
    else k_cost_field_noalloc<false><<<grid, block, 0, st>>>(a, (const float4*)states, cost);
    if (cudaGetLastError() != cudaSuccess) return CVTPM_ERR_CUDA;
    return CVTPM_OK;
}
