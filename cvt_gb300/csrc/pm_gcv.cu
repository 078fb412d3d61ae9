/*
 * pm_gcv.cu — cvt::StereoGCVFilter (cvt/gfx/ifilter/StereoGCVFilter.cpp): a
 * cost-volume stereo method, the comparison baseline beside PatchMatch.  Per
 * disparity d of dmin, dmin + dt, ... (n = |dmax - dmin| / |dt| steps, d
 * accumulated in float): a point cost of colour and x-gradient
 * (stereogcv/costdepthgrad.cl), smoothed by a colour-guided filter built from
 * integral images and box filters (prefixsum/*.cl, boxfilter/*.cl,
 * guidedfilter/*.cl), folded into a running minimum (stereogcv/costmin.cl).
 * apply() runs both views and a left-right check (stereogcv/occlusioncheck.cl).
 *
 * The kernels repeat the reference's arithmetic and, for the integral images,
 * its decomposition: a 16 x 16 block scan alternating x and y steps
 * (prefixsum_pblock*.cl), sequential passes over the block-boundary columns
 * and rows (prefixsum_horiz.cl, prefixsum_vert.cl) and the in-place block
 * fix-up (prefixsum_block2.cl), so every float sum is formed in the same
 * order.  Images follow the OpenCL formats the reference allocates: RGBA
 * (float4), GRAY (CL_INTENSITY: read as (v, v, v, v), written from .x) and
 * GRAYALPHA (CL_RG: read as (r, g, 0, 1)).  Reads outside an image return 0
 * (CLK_ADDRESS_CLAMP's border colour; also for the kernels that declare
 * CLK_ADDRESS_NONE and read outside, which OpenCL leaves undefined).
 * Bilinear reads follow OpenCL 1.2 section 8.2: i0 = floor(u - 0.5),
 * a = (u - 0.5) - i0, weights (1-a)(1-b), a(1-b), (1-a)b, ab summed in that
 * order; a linear sampler at integer coordinates (costdepthconv, undefined in
 * OpenCL) reads the texel.  dot sums left to right.
 *
 * The disparities run in batches (the grid's z index is the disparity in
 * the batch): per batch one pass forms the cost and block-scans its two
 * integral images, three launches finish them, one pass forms the guided
 * filter's (a, b) from their box means and block-scans a and b, three launches
 * finish those, and one pass per pixel walks the batch's disparities in order
 * through the box means of a and b, the filter output and the running
 * minimum: 9 launches per batch, where the reference launches 24 kernels per
 * disparity.  Measured on the 1242x375 x 128 workload: the cost and (a, b)
 * passes are issue- and L1-bound (bilinear taps, divisions, block-scan
 * barriers), the block fix-up streams its read-modify-write at 3.3 TB/s, the
 * boundary-column scans are latency-bound chains.
 */
#include <math.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>

#include "cvtpm.h"
#include "pm_kernels.cuh"

namespace {

const int GCV_BATCH_MAX = 256;   /* disparities per batch, at most */

struct Img {
    float* d;
    int w, h, c;   /* channels stored: 1 GRAY, 2 GRAYALPHA, 4 RGBA */
};

__device__ __forceinline__ float4 tex(const Img& m, int x, int y) {
    if (x < 0 || y < 0 || x >= m.w || y >= m.h) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const size_t o = (size_t)y * m.w + x;
    if (m.c == 1) { const float v = m.d[o]; return make_float4(v, v, v, v); }
    if (m.c == 2) return make_float4(m.d[2 * o], m.d[2 * o + 1], 0.0f, 1.0f);
    return reinterpret_cast<const float4*>(m.d)[o];
}

__device__ __forceinline__ void put(const Img& m, int x, int y, float4 v) {
    if (x < 0 || y < 0 || x >= m.w || y >= m.h) return;
    const size_t o = (size_t)y * m.w + x;
    if (m.c == 1) m.d[o] = v.x;
    else if (m.c == 2) { m.d[2 * o] = v.x; m.d[2 * o + 1] = v.y; }
    else reinterpret_cast<float4*>(m.d)[o] = v;
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 sub4(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ float4 mul4(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 scl4(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ float dotf4(float4 a, float4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
__device__ __forceinline__ float4 shfl4(float4 v, unsigned src) {
    return make_float4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                       __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
}
__device__ __forceinline__ float4 abs4(float4 a) { return make_float4(fabsf(a.x), fabsf(a.y), fabsf(a.z), fabsf(a.w)); }

__device__ __forceinline__ float4 bilinear(const Img& m, float u, float v) {
    const float tu = u - 0.5f, tv = v - 0.5f;
    const float fu = floorf(tu), fv = floorf(tv);
    const float a = tu - fu, b = tv - fv;
    const int i0 = (int)fu, j0 = (int)fv;   /* |u|, |v| < 2^31 on every path here */
    const float4 t00 = tex(m, i0, j0), t10 = tex(m, i0 + 1, j0), t01 = tex(m, i0, j0 + 1), t11 = tex(m, i0 + 1, j0 + 1);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return add4(add4(add4(scl4(w00, t00), scl4(w10, t10)), scl4(w01, t01)), scl4(w11, t11));
}

/* ------------------------------------------------- integral images -- */
/* prefixsum_pblock / _mul2 (src * src2) / _outerrgb: 16 x 16 block scans,
 * Hillis-Steele, an x step then a y step per offset. */
enum { SCAN_PLAIN, SCAN_MUL2 };
template <int MODE>
__global__ void __launch_bounds__(256) k_scan_block(Img out, Img in, Img in2) {
    __shared__ float4 buf[256];
    const int lx = threadIdx.x, ly = threadIdx.y, lid = ly * 16 + lx;
    const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly;
    float4 t = tex(in, x, y);
    if (MODE == SCAN_MUL2) t = mul4(t, tex(in2, x, y));
    buf[lid] = t;
    for (int off = 1; off < 16; off <<= 1) {
        __syncthreads();
        if (lx >= off) t = add4(t, buf[lid - off]);
        __syncthreads();
        buf[lid] = t;
        __syncthreads();
        if (ly >= off) t = add4(t, buf[lid - 16 * off]);
        __syncthreads();
        buf[lid] = t;
    }
    put(out, x, y, t);
}

__global__ void __launch_bounds__(256) k_scan_block_outer(Img rr, Img gg, Img in) {
    __shared__ float4 lo[256], hi[256];
    const int lx = threadIdx.x, ly = threadIdx.y, lid = ly * 16 + lx;
    const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly;
    const float4 c = tex(in, x, y);
    /* (rgb.x * rgb.xyz, 0, rgb.y * rgb.yz, rgb.z * rgb.z, 0) */
    float4 a = make_float4(c.x * c.x, c.x * c.y, c.x * c.z, 0.0f), b = make_float4(c.y * c.y, c.y * c.z, c.z * c.z, 0.0f);
    lo[lid] = a;
    hi[lid] = b;
    for (int off = 1; off < 16; off <<= 1) {
        __syncthreads();
        if (lx >= off) { a = add4(a, lo[lid - off]); b = add4(b, hi[lid - off]); }
        __syncthreads();
        lo[lid] = a; hi[lid] = b;
        __syncthreads();
        if (ly >= off) { a = add4(a, lo[lid - 16 * off]); b = add4(b, hi[lid - 16 * off]); }
        __syncthreads();
        lo[lid] = a; hi[lid] = b;
    }
    put(rr, x, y, a);
    put(gg, x, y, b);
}

/* A stack of images of one shape: slice z starts at d + z * zs. */
struct Stk {
    float* d;
    int w, h, c;
    size_t zs;
    __host__ __device__ __forceinline__ Img at(int z) const { return Img{d + (size_t)z * zs, w, h, c}; }
};

/* One or two stacks scanned by one launch: blockIdx.z = slice * n + which. */
struct Stk2 {
    Stk s[2];
    int n;
    __device__ __forceinline__ Img at(int bz) const { return (bz % n) ? s[1].at(bz / n) : s[0].at(bz / n); }
};

/* prefixsum_horiz: per row, running sum over the block-boundary columns.
 * The sum runs in the reference's order; the loads of 8 boundary columns are
 * issued before their sums are stored. */
__global__ void k_scan_horiz(Stk2 p) {
    const Img m = p.at(blockIdx.z);
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= m.h) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int x0 = 15; x0 < m.w; x0 += 16 * 8) {
        float4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = tex(m, x0 + 16 * k, y);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            acc = add4(acc, v[k]);
            put(m, x0 + 16 * k, y, acc);
        }
    }
}

/* prefixsum_vert: per column, running sum over the block-boundary rows */
__global__ void k_scan_vert(Stk2 p) {
    const Img m = p.at(blockIdx.z);
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= m.w) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int y0 = 15; y0 < m.h; y0 += 16 * 8) {
        float4 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = tex(m, x, y0 + 16 * k);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            acc = add4(acc, v[k]);
            put(m, x, y0 + 16 * k, acc);
        }
    }
}

/* prefixsum_block2, in place: each work-group's window (its 16 x 16 block
 * shifted by (-1, -1)) gets the window's left column and top row added:
 * v = pre(X, Y) [+ pre(left, Y) off the left column] [+ top(X) off the top
 * row], top(X) = pre(X, top) [+ pre(left, top)], the reference's two steps
 * on its local buffer.  Here 16 lanes walk the 16 columns of a window down
 * its rows: the left column's value comes by shuffle from the window's lane
 * 0, the top row's stays in a register — no shared memory, no barriers.
 * Windows are disjoint, and the fix-ups of the image's last row and column
 * read only pixels no window covers. */
__global__ void __launch_bounds__(128) k_scan_block2(Stk2 p, int nbx, int nby) {
    const Img m = p.at(blockIdx.z);
    const int lane = threadIdx.x, lx = lane & 15;
    const int wx = blockIdx.x * 2 + (lane >> 4), wy = blockIdx.y * 4 + threadIdx.y;
    if (wy >= nby) return;                                  /* the whole warp */
    const bool live = wx < nbx;
    const int bx = wx * 16, by = wy * 16;
    const int X = bx + lx - 1;
    const unsigned src = lane & 16;                         /* the window's lane 0 */
    float4 top = tex(m, X, by - 1);
    {
        const float4 l0 = shfl4(top, src);
        if (lx) top = add4(top, l0);
    }
    for (int ly = 0; ly < 16; ++ly) {
        float4 v = top;
        if (ly) {
            v = tex(m, X, by + ly - 1);
            const float4 l = shfl4(v, src);
            if (lx) v = add4(v, l);
            v = add4(v, top);
        }
        const int x = bx + lx, y = by + ly;
        if (!live || x > m.w || y > m.h || !x || !y) continue;
        put(m, X, y - 1, v);
        if (y == m.h - 1 && lx < 15 && ly == 15 && x < m.w) put(m, x, y, add4(tex(m, x, y), tex(m, bx - 1, by + ly)));
        if (x == m.w - 1 && ly < 15 && lx == 15 && y < m.h) put(m, x, y, add4(tex(m, x, y), tex(m, bx + lx, by - 1)));
    }
}

/* boxfilter_prefixsum: the mean over the box of radius r from the integral
 * image (window clamped to the image, as the reference clamps it) */
__device__ __forceinline__ float4 box_px(const Img& in, int x, int y, int r) {
    const int x0 = max(0, x - (r + 1)), y0 = max(0, y - (r + 1));
    const int x1 = min(in.w - 1, x + r), y1 = min(in.h - 1, y + r);
    float4 v = tex(in, x0, y0);
    v = sub4(v, tex(in, x0, y1));
    v = sub4(v, tex(in, x1, y0));
    v = add4(v, tex(in, x1, y1));
    const float area = (float)((x1 - x0) * (y1 - y0));
    return make_float4(v.x / area, v.y / area, v.z / area, v.w / area);
}

__global__ void __launch_bounds__(256) k_box(Img out, Img in, int r) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= out.w || y >= out.h) return;
    put(out, x, y, box_px(in, x, y, r));
}

/* ------------------------------------------------------------ steps -- */
__global__ void __launch_bounds__(256) k_fill2(Img m, float a, float b) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x < m.w && y < m.h) put(m, x, y, make_float4(a, b, 0.0f, 0.0f));
}

/* gradx.cl: right minus left neighbour, 0 outside */
__global__ void __launch_bounds__(256) k_gradx(Img out, Img src) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= out.w || y >= out.h) return;
    put(out, x, y, sub4(tex(src, x + 1, y), tex(src, x - 1, y)));
}

/* stereogcv_costdepthgrad (point cost) at (x, y) for disparity depth:
 * img0 at the pixel, img1 at x - depth */
__device__ __forceinline__ float point_cost(const Img& img0, const Img& img1, const Img& grad0, const Img& grad1,
                                            int x, int y, float depth) {
    const int W = img0.w, H = img1.h;
    const float u = (float)x + 0.5f - depth, v = (float)y + 0.5f;
    if (u < 0.0f || u >= (float)W || v < 0.0f || v >= (float)H) return 0.008f + 0.028f;
    const float4 dm = make_float4(0.3333f, 0.3333f, 0.3333f, 0.0f);
    const float4 I0 = tex(img0, x, y), G0 = tex(grad0, x, y);
    const float4 I1 = bilinear(img1, u, v), G1 = bilinear(grad1, u, v);
    const float ci = fminf(dotf4(abs4(sub4(I1, I0)), dm), 0.028f);
    const float cg = fminf(dotf4(abs4(sub4(G1, G0)), dm), 0.008f);
    return ci + (cg - ci) * 0.10f;   /* mix(ci, cg, ALPHA) */
}

/* Disparities of one batch: slice z of every stack belongs to d[z]. */
struct Depths {
    float d[GCV_BATCH_MAX];
};

/* The cost image of disparity dl.d[z] and the 16 x 16 block scans of its two
 * integral images, the cost (GRAY) and img0 * cost (prefixsum_pblock_mul2),
 * in one pass: the same sums in the same order as the two block scans of the
 * stored cost image.  Pixels outside the image scan as 0, as the reference's
 * out-of-image reads return 0. */
__global__ void __launch_bounds__(256) k_cost_scan(Stk ig, Stk iint, Img img0, Img img1, Img grad0, Img grad1,
                                                   Depths dl) {
    __shared__ float4 b4[256];
    __shared__ float b1[256];
    const int lx = threadIdx.x, ly = threadIdx.y, lid = ly * 16 + lx;
    const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly, z = blockIdx.z;
    float c = 0.0f;
    if (x < img0.w && y < img0.h) c = point_cost(img0, img1, grad0, grad1, x, y, dl.d[z]);
    float4 t = mul4(tex(img0, x, y), make_float4(c, c, c, c));
    b4[lid] = t;
    b1[lid] = c;
    for (int off = 1; off < 16; off <<= 1) {
        __syncthreads();
        if (lx >= off) { t = add4(t, b4[lid - off]); c = c + b1[lid - off]; }
        __syncthreads();
        b4[lid] = t; b1[lid] = c;
        __syncthreads();
        if (ly >= off) { t = add4(t, b4[lid - 16 * off]); c = c + b1[lid - 16 * off]; }
        __syncthreads();
        b4[lid] = t; b1[lid] = c;
    }
    put(iint.at(z), x, y, t);
    put(ig.at(z), x, y, make_float4(c, c, c, c));
}

/* guidedfilter_calcab_outerrgb at one pixel: the 3x3 system (covariance of
 * the guide + epsilon) solved by the reference's LU steps; s is the mean
 * cost (a GRAY image, read as (s, s, s, s)). */
__device__ __forceinline__ float4 calcab_px(float4 g, float4 s, float4 sg, float4 rr, float4 gg, float eps,
                                            float* b) {
    float4 cov = sub4(sg, mul4(g, s));
    cov.w = 0.0f;
    rr.x = rr.x - g.x * g.x; rr.y = rr.y - g.x * g.y; rr.z = rr.z - g.x * g.z;
    gg.x = gg.x - g.y * g.y; gg.y = gg.y - g.y * g.z;
    gg.z = gg.z - g.z * g.z;
    float m0x = rr.x, m0y = rr.y, m0z = rr.z;
    float m1x = rr.y, m1y = gg.x, m1z = gg.y;
    float m2x = rr.z, m2y = gg.y, m2z = gg.z;
    m0x = m0x + 1.0f * eps;
    m1y = m1y + 1.0f * eps;
    m2z = m2z + 1.0f * eps;
    /* LUSolve */
    m1x = m1x / m0x;
    m2x = m2x / m0x;
    m1y = m1y - m1x * m0y; m1z = m1z - m1x * m0z;
    m2y = m2y - m2x * m0y; m2z = m2z - m2x * m0z;
    m2y = m2y / m1y;
    m2z = m2z - m2y * m1z;
    float bx = cov.x, by = cov.y, bz = cov.z;
    by = by - m1x * bx;
    bz = bz - (m2x * bx + m2y * by);
    const float xz = bz / m2z;
    const float xy = (by - m1z * xz) / m1y;
    const float xx = (bx - (m0y * xy + m0z * xz)) / m0x;
    const float4 a = make_float4(xx, xy, xz, 0.0f);
    *b = s.x - dotf4(g, a);
    return a;
}

/* Per pixel of disparity slice z: the box means of the cost and of
 * guide * cost, the guided filter's (a, b), and the 16 x 16 block scans of a
 * and b — the first steps of their integral images.  b's four channels are
 * equal (s - dot(g, a) with s a GRAY mean), so one is stored. */
__global__ void __launch_bounds__(256) k_calcab_scan(Stk iaI, Stk ibI, Stk ig, Stk iint, Img mG, Img mRR, Img mGG,
                                                     float eps, int r) {
    __shared__ float4 b4[256];
    __shared__ float b1[256];
    const int lx = threadIdx.x, ly = threadIdx.y, lid = ly * 16 + lx;
    const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly, z = blockIdx.z;
    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float b = 0.0f;
    if (x < mG.w && y < mG.h) {
        const float s = box_px(ig.at(z), x, y, r).x;
        a = calcab_px(tex(mG, x, y), make_float4(s, s, s, s), box_px(iint.at(z), x, y, r), tex(mRR, x, y),
                      tex(mGG, x, y), eps, &b);
    }
    b4[lid] = a;
    b1[lid] = b;
    for (int off = 1; off < 16; off <<= 1) {
        __syncthreads();
        if (lx >= off) { a = add4(a, b4[lid - off]); b = b + b1[lid - off]; }
        __syncthreads();
        b4[lid] = a; b1[lid] = b;
        __syncthreads();
        if (ly >= off) { a = add4(a, b4[lid - 16 * off]); b = b + b1[lid - 16 * off]; }
        __syncthreads();
        b4[lid] = a; b1[lid] = b;
    }
    put(iaI.at(z), x, y, a);
    put(ibI.at(z), x, y, make_float4(b, b, b, b));
}

/* Per pixel, the batch's disparities in order: the box means of a and b,
 * guidedfilter_applyab_gc_outer (dot(a, guide) + b) and stereogcv_costmin
 * (keep (cost, depth) of the smaller cost; ties keep the old).  A block is 32
 * pixels of a row x FM_CHUNKS consecutive runs of the batch's disparities:
 * each warp keeps its run's first strict minimum, and the runs are folded in
 * order into the pixel's (cost, depth) with the same strict comparison.  The
 * sequential rule picks the first disparity of the smallest cost below the
 * start (NaN never compares less), and so does this. */
#define FM_CHUNKS 8
/* 4 blocks per SM (64 registers): 11.44 ms per apply at 1242x375 x 128
 * disparities, against 11.95 with 77 registers and 3 blocks, 12.4 with 5 */
__global__ void __launch_bounds__(32 * FM_CHUNKS, 4) k_filter_min(Img c, Stk iaI, Stk ibI, Img guide, Depths nd, int nz,
                                                              int r) {
    __shared__ float bv[FM_CHUNKS][32];
    __shared__ int bz[FM_CHUNKS][32];
    const int lx = threadIdx.x, k = threadIdx.y;
    const int x = blockIdx.x * 32 + lx, y = blockIdx.y;
    float best = __int_as_float(0x7f800000);   /* +inf: never taken, as no cost beats the start of 1e9 with it */
    int bi = -1;
    if (x < c.w) {
        const float4 g = tex(guide, x, y);
        const int z1 = (k + 1) * nz / FM_CHUNKS;
#pragma unroll 2
        for (int z = k * nz / FM_CHUNKS; z < z1; ++z) {
            const float d = dotf4(box_px(iaI.at(z), x, y, r), g);
            const float n = d + box_px(ibI.at(z), x, y, r).x;
            if (n < best) { best = n; bi = z; }
        }
    }
    bv[k][lx] = best;
    bz[k][lx] = bi;
    __syncthreads();
    if (k || x >= c.w) return;
    float4 cc = tex(c, x, y);
    for (int j = 0; j < FM_CHUNKS; ++j)
        if (bz[j][lx] >= 0 && bv[j][lx] < cc.x) { cc.x = bv[j][lx]; cc.y = nd.d[bz[j][lx]]; }
    put(c, x, y, cc);
}

/* stereogcv_costdepthconv: depth * scale + add, 0 where it reached 1 */
__global__ void __launch_bounds__(256) k_depthconv(float* __restrict__ out, size_t opitch, Img cd, float scale, float add) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= cd.w || y >= cd.h) return;
    const float v = tex(cd, x, y).y;
    out[(size_t)y * opitch + x] = v >= 1.0f ? 0.0f : v * scale + add;
}

/* stereogcv_occlusioncheck into GRAY_UINT8: write_imagef's CL_UNORM_INT8
 * conversion, convert_uchar_sat_rte(v * 255) */
__global__ void __launch_bounds__(256) k_occlusion(uint8_t* __restrict__ out, size_t opitch, Img d0i, Img d1i, float dscale) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= d0i.w || y >= d0i.h) return;
    const float din0 = tex(d0i, x, y).x;
    const float d0 = din0 * dscale;
    const float din1 = bilinear(d1i, -d0 + (float)x + 0.5f, (float)y + 0.5f).x;
    const float d1 = din1 * dscale;
    const float diff = fabsf(-d0 + d1);
    const float v = diff <= 2.0f ? (din0 + din1) * 0.5f : 0.0f;
    const float q = rintf(v * 255.0f);
    out[(size_t)y * opitch + x] = (uint8_t)(q < 0.0f ? 0.0f : (q > 255.0f ? 255.0f : q));
}

/* ----------------------------------------------------------- host -- */
cvtpm_status fail(cvtpm_status s, const std::string& m) {
    pm_set_free_error(m);
    return s;
}

dim3 g16(int W, int H) { return dim3((W + 15) / 16, (H + 15) / 16); }
dim3 g32(int W, int H) { return dim3((W + 31) / 32, (H + 7) / 8); }


Stk2 one(Stk a) { return Stk2{{a, a}, 1}; }
Stk2 two(Stk a, Stk b) { return Stk2{{a, b}, 2}; }

/* prefixsum_horiz, prefixsum_vert and prefixsum_block2 over nz slices of
 * the stacks in p */
void scan_rest(Stk2 p, int nz, cudaStream_t st) {
    const int W = p.s[0].w, H = p.s[0].h, nb = nz * p.n;
    k_scan_horiz<<<dim3((H + 127) / 128, 1, nb), 128, 0, st>>>(p);
    k_scan_vert<<<dim3((W + 127) / 128, 1, nb), 128, 0, st>>>(p);
    const int nbx = (W + 15) / 16, nby = (H + 15) / 16;   /* the reference's work-groups */
    k_scan_block2<<<dim3((nbx + 1) / 2, (nby + 3) / 4, nb), dim3(32, 4), 0, st>>>(p, nbx, nby);
}

Stk stack(float* d, int W, int H, int c) { return Stk{d, W, H, c, (size_t)W * H * c}; }

/* Scratch: GCV_VIEW_FLOATS per pixel for a view, GCV_SLICE_FLOATS per pixel
 * and disparity of a batch (cost integral 1, guide * cost integral 4, the
 * integrals of a 4 and b 1). */
const int GCV_VIEW_FLOATS = 22, GCV_SLICE_FLOATS = 10;

std::atomic<int> g_batch{0};

size_t count_steps(float dmin, float dmax, float dt) { return (size_t)(fabsf(dmax - dmin) / fabsf(dt)); }

/* Disparities per batch: the set value, else as many as 4 GiB of slices
 * hold, at most GCV_BATCH_MAX and at most the number of steps. */
int batch_for(int W, int H, size_t steps) {
    const int set = g_batch.load();
    size_t b = set > 0 ? (size_t)set : ((size_t)4 << 30) / ((size_t)GCV_SLICE_FLOATS * 4 * W * H);
    b = b < 1 ? 1 : (b > GCV_BATCH_MAX ? GCV_BATCH_MAX : b);
    if (steps && b > steps) b = steps;
    return (int)b;
}

size_t scratch_floats(int W, int H, int batch, int extra) {
    return (size_t)W * H * (GCV_VIEW_FLOATS + (size_t)GCV_SLICE_FLOATS * batch + extra);
}

int launches_for(size_t steps, int batch) {
    const size_t nb = (steps + batch - 1) / batch;
    return (int)(3 + 5 + 6 + nb * 9 + 1);
}

/* StereoGCVFilter::depthmap (StereoGCVFilter.cpp:97-242), point cost, with
 * the disparities processed in batches: the grid's z index is the disparity
 * within the batch, and each launch covers the batch.  Every disparity's
 * values are formed by the reference's arithmetic in its order; the running
 * minimum takes the disparities in the reference's order.  The integral
 * images of the box-SAD and NCC cost variants, which the reference forms but
 * the point cost does not read, are not formed. */
void depthmap(float* dst, size_t dpitch, Img cam0, Img cam1, float dmin, float dmax, float dt, float* s, int batch,
              cudaStream_t st) {
    const int W = cam0.w, H = cam0.h;
    const size_t n = (size_t)W * H;
    auto take = [&](int c) { Img m{s, W, H, c}; s += n * (size_t)c; return m; };
    /* RGBA images and stacks first: every float4 buffer starts on a
     * multiple of 4 floats whatever W * H is */
    const Img g0 = take(4), g1 = take(4), mG = take(4), mRR = take(4), mGG = take(4);
    const Stk iint = stack(s, W, H, 4), iaI = stack(s + 4 * n * batch, W, H, 4);
    s += 8 * n * batch;
    const Img c = take(2);
    const Stk ig = stack(s, W, H, 1), ibI = stack(s + n * batch, W, H, 1);
    /* the view's set-up integrals, before the first batch: 8 floats per pixel
     * of the RGBA stacks */
    const Stk t0 = stack(iint.d, W, H, 4), t1 = stack(iint.d + 4 * n, W, H, 4);
    const int R = 9;
    k_fill2<<<g32(W, H), dim3(32, 8), 0, st>>>(c, 1e9f, 0.0f);
    k_gradx<<<g32(W, H), dim3(32, 8), 0, st>>>(g0, cam0);
    k_gradx<<<g32(W, H), dim3(32, 8), 0, st>>>(g1, cam1);
    k_scan_block<SCAN_PLAIN><<<g16(W, H), dim3(16, 16), 0, st>>>(t0.at(0), cam1, cam1);
    scan_rest(one(t0), 1, st);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mG, t0.at(0), R);
    k_scan_block_outer<<<g16(W, H), dim3(16, 16), 0, st>>>(t0.at(0), t1.at(0), cam1);
    scan_rest(two(t0, t1), 1, st);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mRR, t0.at(0), R);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mGG, t1.at(0), R);
    if (dmax < dmin && dt > 0) dt = -dt;
    size_t steps = count_steps(dmin, dmax, dt);
    float d = dmin;
    while (steps) {
        const int nz = (int)(steps < (size_t)batch ? steps : (size_t)batch);
        Depths dd, nd;
        for (int z = 0; z < nz; ++z, d += dt) {
            dd.d[z] = d;
            nd.d[z] = fabsf(d - dmin) / fabsf(dmax - dmin);
        }
        steps -= nz;
        const dim3 gz((W + 15) / 16, (H + 15) / 16, nz);
        k_cost_scan<<<gz, dim3(16, 16), 0, st>>>(ig, iint, cam1, cam0, g1, g0, dd);
        scan_rest(two(ig, iint), nz, st);
        k_calcab_scan<<<gz, dim3(16, 16), 0, st>>>(iaI, ibI, ig, iint, mG, mRR, mGG, 1e-3f, R);
        scan_rest(two(iaI, ibI), nz, st);
        k_filter_min<<<dim3((W + 31) / 32, H), dim3(32, FM_CHUNKS), 0, st>>>(c, iaI, ibI, cam1, nd, nz, R);
    }
    k_depthconv<<<g32(W, H), dim3(32, 8), 0, st>>>(dst, dpitch / 4, c, 1.0f, 0.0f);
}

cvtpm_status check_args(const float* cam0, const float* cam1, int W, int H, size_t pitch, float dmin, float dmax,
                        float dt) {
    if (!cam0 || !cam1) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: NULL image");
    if (W < 2 || H < 2) return fail(CVTPM_ERR_SIZE, "gcv: images must be at least 2 x 2");
    if (pitch != (size_t)W * 16) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: images must be tight RGBA float rows");
    if ((uintptr_t)cam0 % 16 || (uintptr_t)cam1 % 16)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: images must start on a 16-byte boundary");
    if (!isfinite(dmin) || !isfinite(dmax) || !isfinite(dt) || dt == 0.0f || dmin == dmax)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: dmin, dmax, dt must be finite, dt and dmax - dmin non-zero");
    if (fabsf(dmax - dmin) / fabsf(dt) > 65536.0f) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: more than 65536 steps");
    return CVTPM_OK;
}

/* Scratch comes from a stream-ordered pool of the library's own per device:
 * allocated on the call's stream, freed on it after the call's last kernel,
 * so concurrent calls on different streams never share bytes.  The pool
 * keeps what it has allocated (release threshold: never) for later calls. */
cudaMemPool_t scratch_pool(int dev) {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lock(mu);
    const auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = pool;
    return pool;
}

float* scratch(size_t bytes, cudaStream_t st) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    cudaMemPool_t pool = scratch_pool(dev);
    void* p = nullptr;
    if (!pool || cudaMallocFromPoolAsync(&p, bytes, pool, st) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return (float*)p;
}

}  // namespace

extern "C" {

cvtpm_status cvtpm_gcv_trim(int device, size_t keep_bytes) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return CVTPM_ERR_CUDA;
    if (device < 0 || device >= n) return CVTPM_ERR_INVALID_ARGUMENT;
    cudaMemPool_t pool = scratch_pool(device);
    if (!pool) return CVTPM_ERR_CUDA;
    /* memory of calls still in flight stays reserved: trimming only returns
     * what the pool holds unused */
    return cudaMemPoolTrimTo(pool, keep_bytes) == cudaSuccess ? CVTPM_OK : CVTPM_ERR_CUDA;
}

cvtpm_status cvtpm_gcv_set_batch(int disparities) {
    if (disparities < 0 || disparities > GCV_BATCH_MAX)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: batch must be 0 (automatic) .. " + std::to_string(GCV_BATCH_MAX));
    g_batch.store(disparities);
    return CVTPM_OK;
}

cvtpm_status cvtpm_gcv_plan(int width, int height, float dmin, float dmax, float dt, int* steps, int* batch,
                            size_t* scratch_bytes, int* launches) {
    if (width < 2 || height < 2) return fail(CVTPM_ERR_SIZE, "gcv: images must be at least 2 x 2");
    if (!isfinite(dmin) || !isfinite(dmax) || !isfinite(dt) || dt == 0.0f || dmin == dmax)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: dmin, dmax, dt must be finite, dt and dmax - dmin non-zero");
    const size_t n = count_steps(dmin, dmax, dt);
    const int b = batch_for(width, height, n);
    if (steps) *steps = (int)n;
    if (batch) *batch = b;
    if (scratch_bytes) *scratch_bytes = scratch_floats(width, height, b, 0) * sizeof(float);
    if (launches) *launches = launches_for(n, b);
    return CVTPM_OK;
}

cvtpm_status cvtpm_gcv_depthmap(float* dst, size_t dst_pitch, const float* cam0, const float* cam1, int width,
                                int height, size_t pitch, float dmin, float dmax, float dt, void* stream) {
    cvtpm_status s = check_args(cam0, cam1, width, height, pitch, dmin, dmax, dt);
    if (s != CVTPM_OK) return s;
    if (!dst || dst_pitch % 4 || dst_pitch < (size_t)width * 4) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: bad dst");
    const int b = batch_for(width, height, count_steps(dmin, dmax, dt));
    float* sc = scratch(sizeof(float) * scratch_floats(width, height, b, 0), (cudaStream_t)stream);
    if (!sc) return fail(CVTPM_ERR_ALLOC, "gcv: scratch allocation failed");
    depthmap(dst, dst_pitch, Img{(float*)cam0, width, height, 4}, Img{(float*)cam1, width, height, 4}, dmin, dmax, dt,
             sc, b, (cudaStream_t)stream);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(sc, (cudaStream_t)stream);      /* back to the pool after the call's kernels */
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("gcv: ") + cudaGetErrorString(e));
}

cvtpm_status cvtpm_gcv_apply(uint8_t* dst, size_t dst_pitch, float* d0, float* d1, size_t dpitch, const float* cam0,
                             const float* cam1, int width, int height, size_t pitch, float dmin, float dmax, float dt,
                             void* stream) {
    cvtpm_status s = check_args(cam0, cam1, width, height, pitch, dmin, dmax, dt);
    if (s != CVTPM_OK) return s;
    if (!dst || dst_pitch < (size_t)width) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: bad dst");
    if ((d0 == nullptr) != (d1 == nullptr) || (d0 && dpitch != (size_t)width * 4))
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: give both depth maps (tight rows, pitch width * 4) or neither");
    const size_t n = (size_t)width * height;
    const int b = batch_for(width, height, count_steps(dmin, dmax, dt));
    float* sc = scratch(sizeof(float) * scratch_floats(width, height, b, 2), (cudaStream_t)stream);
    if (!sc) return fail(CVTPM_ERR_ALLOC, "gcv: scratch allocation failed");
    float* own0 = sc + scratch_floats(width, height, b, 0);
    float* own1 = own0 + n;
    float* p0 = d0 ? d0 : own0;
    float* p1 = d1 ? d1 : own1;
    const size_t pp = d0 ? dpitch : (size_t)width * 4;
    cudaStream_t st = (cudaStream_t)stream;
    const Img a{(float*)cam0, width, height, 4}, c1{(float*)cam1, width, height, 4};
    depthmap(p0, pp, a, c1, dmin, dmax, dt, sc, b, st);
    depthmap(p1, pp, c1, a, -dmin, -dmax, -dt, sc, b, st);
    /* the two depth maps as GRAY images of pitch pp */
    const Img i0{p0, width, height, 1}, i1{p1, width, height, 1};
    k_occlusion<<<g32(width, height), dim3(32, 8), 0, st>>>(dst, dst_pitch, i0, i1, fabsf(dmax));
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(sc, st);                        /* back to the pool after the call's kernels */
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("gcv: ") + cudaGetErrorString(e));
}

}  // extern "C"
