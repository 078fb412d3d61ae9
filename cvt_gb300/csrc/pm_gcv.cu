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
 * Kernels are HBM-bound per-pixel passes, the scans latency-bound; a
 * disparity costs 24 launches.
 */
#include <math.h>
#include <stdint.h>

#include <string>

#include "cvtpm.h"
#include "pm_kernels.cuh"

namespace {

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

/* prefixsum_horiz: per row, running sum over the block-boundary columns */
__global__ void k_scan_horiz(Img m) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= m.h) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int x = 15; x < m.w; x += 16) {
        acc = add4(acc, tex(m, x, y));
        put(m, x, y, acc);
    }
}

/* prefixsum_vert: per column, running sum over the block-boundary rows */
__global__ void k_scan_vert(Img m) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= m.w) return;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int y = 15; y < m.h; y += 16) {
        acc = add4(acc, tex(m, x, y));
        put(m, x, y, acc);
    }
}

/* prefixsum_block2, in place: each block's window shifted by (-1, -1) gets
 * the block's boundary row and column added; windows of different blocks are
 * disjoint. */
__global__ void __launch_bounds__(256) k_scan_block2(Img m) {
    __shared__ float4 buf[16][16];
    const int lx = threadIdx.x, ly = threadIdx.y;
    const int bx = blockIdx.x * 16, by = blockIdx.y * 16;
    buf[ly][lx] = tex(m, bx + lx - 1, by + ly - 1);
    __syncthreads();
    if (lx) buf[ly][lx] = add4(buf[ly][lx], buf[ly][0]);
    __syncthreads();
    if (ly) buf[ly][lx] = add4(buf[ly][lx], buf[0][lx]);
    const int x = bx + lx, y = by + ly;
    if (x > m.w || y > m.h || !x || !y) return;
    put(m, bx + lx - 1, by + ly - 1, buf[ly][lx]);
    if (y == m.h - 1 && lx < 15 && ly == 15 && x < m.w) put(m, x, y, add4(tex(m, x, y), tex(m, bx - 1, by + ly)));
    if (x == m.w - 1 && ly < 15 && lx == 15 && y < m.h) put(m, x, y, add4(tex(m, x, y), tex(m, bx + lx, by - 1)));
}

/* boxfilter_prefixsum: the mean over the box of radius r from the integral
 * image (window clamped to the image, as the reference clamps it) */
__global__ void __launch_bounds__(256) k_box(Img out, Img in, int r) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= out.w || y >= out.h) return;
    const int x0 = max(0, x - (r + 1)), y0 = max(0, y - (r + 1));
    const int x1 = min(out.w - 1, x + r), y1 = min(out.h - 1, y + r);
    float4 v = tex(in, x0, y0);
    v = sub4(v, tex(in, x0, y1));
    v = sub4(v, tex(in, x1, y0));
    v = add4(v, tex(in, x1, y1));
    const float area = (float)((x1 - x0) * (y1 - y0));
    put(out, x, y, make_float4(v.x / area, v.y / area, v.z / area, v.w / area));
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

/* stereogcv_costdepthgrad (point cost): img0 at the pixel, img1 at x - d */
__global__ void __launch_bounds__(256) k_cost(Img cost, Img img0, Img img1, Img grad0, Img grad1, float depth) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    const int W = img0.w, H = img1.h;
    if (x >= W || y >= H) return;
    const float u = (float)x + 0.5f - depth, v = (float)y + 0.5f;
    float c;
    if (u < 0.0f || u >= (float)W || v < 0.0f || v >= (float)H) {
        c = 0.008f + 0.028f;
    } else {
        const float4 dm = make_float4(0.3333f, 0.3333f, 0.3333f, 0.0f);
        const float4 I0 = tex(img0, x, y), G0 = tex(grad0, x, y);
        const float4 I1 = bilinear(img1, u, v), G1 = bilinear(grad1, u, v);
        const float ci = fminf(dotf4(abs4(sub4(I1, I0)), dm), 0.028f);
        const float cg = fminf(dotf4(abs4(sub4(G1, G0)), dm), 0.008f);
        c = ci + (cg - ci) * 0.10f;   /* mix(ci, cg, ALPHA) */
    }
    put(cost, x, y, make_float4(c, c, c, c));
}

/* guidedfilter_calcab_outerrgb: per pixel the 3x3 system (covariance of the
 * guide + epsilon) solved by the reference's LU steps */
__global__ void __launch_bounds__(256) k_calcab(Img ia, Img ib, Img mG, Img mS, Img mSG, Img mRR, Img mGG, float eps) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= ia.w || y >= ia.h) return;
    const float4 g = tex(mG, x, y), s = tex(mS, x, y), sg = tex(mSG, x, y);
    float4 rr = tex(mRR, x, y), gg = tex(mGG, x, y);
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
    const float d = dotf4(g, a);
    put(ia, x, y, a);
    put(ib, x, y, make_float4(s.x - d, s.y - d, s.z - d, s.w - d));
}

/* guidedfilter_applyab_gc_outer: dot(a, guide) + b */
__global__ void __launch_bounds__(256) k_applyab(Img out, Img in, Img ia, Img ib) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= out.w || y >= out.h) return;
    const float d = dotf4(tex(ia, x, y), tex(in, x, y));
    const float4 b = tex(ib, x, y);
    put(out, x, y, make_float4(d + b.x, d + b.y, d + b.z, 1.0f));
}

/* stereogcv_costmin: keep (cost, depth) of the smaller cost; ties keep the old */
__global__ void __launch_bounds__(256) k_costmin(Img out, Img cnew, Img cin, float newdepth) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= out.w || y >= out.h) return;
    float4 c = tex(cin, x, y);
    const float n = tex(cnew, x, y).x;
    if (n < c.x) { c.x = n; c.y = newdepth; }
    put(out, x, y, c);
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

struct Scratch {
    float* base = nullptr;
    size_t bytes = 0;
    int device = -1;
};

void integral(Img dst, Img src, const Img* src2, cudaStream_t st) {
    if (src2) k_scan_block<SCAN_MUL2><<<g16(src.w, src.h), dim3(16, 16), 0, st>>>(dst, src, *src2);
    else k_scan_block<SCAN_PLAIN><<<g16(src.w, src.h), dim3(16, 16), 0, st>>>(dst, src, src);
    k_scan_horiz<<<(dst.h + 127) / 128, 128, 0, st>>>(dst);
    k_scan_vert<<<(dst.w + 127) / 128, 128, 0, st>>>(dst);
    k_scan_block2<<<g16(dst.w, dst.h), dim3(16, 16), 0, st>>>(dst);
}

void integral_outer(Img rr, Img gg, Img src, cudaStream_t st) {
    k_scan_block_outer<<<g16(src.w, src.h), dim3(16, 16), 0, st>>>(rr, gg, src);
    for (Img m : {rr, gg}) k_scan_horiz<<<(m.h + 127) / 128, 128, 0, st>>>(m);
    for (Img m : {rr, gg}) k_scan_vert<<<(m.w + 127) / 128, 128, 0, st>>>(m);
    for (Img m : {rr, gg}) k_scan_block2<<<g16(m.w, m.h), dim3(16, 16), 0, st>>>(m);
}

/* Scratch of one depthmap: 47 floats per pixel. */
const int GCV_FLOATS = 47;

/* StereoGCVFilter::depthmap (StereoGCVFilter.cpp:97-242), point cost.  The
 * integral images of the box-SAD and NCC cost variants, which it forms but the
 * point cost does not read, are not formed. */
void depthmap(float* dst, size_t dpitch, Img cam0, Img cam1, float dmin, float dmax, float dt, float* s,
              cudaStream_t st, int* launches) {
    const int W = cam0.w, H = cam0.h;
    const size_t n = (size_t)W * H;
    auto take = [&](int c) { Img m{s, W, H, c}; s += n * (size_t)c; return m; };
    Img g0 = take(4), g1 = take(4), ia = take(4), ib = take(4), iint = take(4), iint2 = take(4), mG = take(4);
    Img mGS = take(4), mRR = take(4), mGG = take(4), cost = take(1), costgf = take(1), mS = take(1);
    Img c[2] = {take(2), take(2)};
    int index = 0;
    const int R = 9;
    k_fill2<<<g32(W, H), dim3(32, 8), 0, st>>>(c[!index], 1e9f, 0.0f);
    k_gradx<<<g32(W, H), dim3(32, 8), 0, st>>>(g0, cam0);
    k_gradx<<<g32(W, H), dim3(32, 8), 0, st>>>(g1, cam1);
    integral(iint, cam1, nullptr, st);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mG, iint, R);
    integral_outer(iint, iint2, cam1, st);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mRR, iint, R);
    k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mGG, iint2, R);
    *launches += 3 + 4 + 1 + 7 + 2;
    if (dmax < dmin && dt > 0) dt = -dt;
    size_t steps = (size_t)(fabsf(dmax - dmin) / fabsf(dt));
    for (float d = dmin; steps--; d += dt) {
        Img g = cost;
        Img ig = iint;
        ig.c = 1;                                   /* the integral of a GRAY image is GRAY */
        k_cost<<<g32(W, H), dim3(32, 8), 0, st>>>(cost, cam1, cam0, g1, g0, d);
        integral(ig, g, nullptr, st);
        k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mS, ig, R);
        integral(iint, cam1, &cost, st);
        k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(mGS, iint, R);
        k_calcab<<<g32(W, H), dim3(32, 8), 0, st>>>(ia, ib, mG, mS, mGS, mRR, mGG, 1e-3f);
        integral(iint, ia, nullptr, st);
        k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(ia, iint, R);
        integral(iint, ib, nullptr, st);
        k_box<<<g32(W, H), dim3(32, 8), 0, st>>>(ib, iint, R);
        k_applyab<<<g32(W, H), dim3(32, 8), 0, st>>>(costgf, cam1, ia, ib);
        k_costmin<<<g32(W, H), dim3(32, 8), 0, st>>>(c[index], costgf, c[!index], fabsf(d - dmin) / fabsf(dmax - dmin));
        index = 1 - index;
        *launches += 24;
    }
    k_depthconv<<<g32(W, H), dim3(32, 8), 0, st>>>(dst, dpitch / 4, c[!index], 1.0f, 0.0f);
    *launches += 1;
}

cvtpm_status check_args(const float* cam0, const float* cam1, int W, int H, size_t pitch, float dmin, float dmax,
                        float dt) {
    if (!cam0 || !cam1) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: NULL image");
    if (W < 2 || H < 2) return fail(CVTPM_ERR_SIZE, "gcv: images must be at least 2 x 2");
    if (pitch != (size_t)W * 16) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: images must be tight RGBA float rows");
    if (!isfinite(dmin) || !isfinite(dmax) || !isfinite(dt) || dt == 0.0f || dmin == dmax)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: dmin, dmax, dt must be finite, dt and dmax - dmin non-zero");
    if (fabsf(dmax - dmin) / fabsf(dt) > 65536.0f) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: more than 65536 steps");
    return CVTPM_OK;
}

thread_local Scratch g_scratch;

/* Scratch of the calling host thread on the current device, kept between
 * calls; it grows (after a device synchronisation) when a call needs more. */
float* scratch(size_t bytes) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if (g_scratch.device == dev && g_scratch.bytes >= bytes) return g_scratch.base;
    if (g_scratch.base) {
        int cur = dev;
        cudaSetDevice(g_scratch.device);
        cudaDeviceSynchronize();
        cudaFree(g_scratch.base);
        cudaSetDevice(cur);
        g_scratch.base = nullptr;
        g_scratch.bytes = 0;
    }
    if (cudaMalloc(&g_scratch.base, bytes) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    g_scratch.bytes = bytes;
    g_scratch.device = dev;
    return g_scratch.base;
}

}  // namespace

extern "C" {

cvtpm_status cvtpm_gcv_depthmap(float* dst, size_t dst_pitch, const float* cam0, const float* cam1, int width,
                                int height, size_t pitch, float dmin, float dmax, float dt, void* stream) {
    cvtpm_status s = check_args(cam0, cam1, width, height, pitch, dmin, dmax, dt);
    if (s != CVTPM_OK) return s;
    if (!dst || dst_pitch % 4 || dst_pitch < (size_t)width * 4) return fail(CVTPM_ERR_INVALID_ARGUMENT, "gcv: bad dst");
    float* sc = scratch(sizeof(float) * GCV_FLOATS * (size_t)width * height);
    if (!sc) return fail(CVTPM_ERR_ALLOC, "gcv: scratch allocation failed");
    int launches = 0;
    depthmap(dst, dst_pitch, Img{(float*)cam0, width, height, 4}, Img{(float*)cam1, width, height, 4}, dmin, dmax, dt,
             sc, (cudaStream_t)stream, &launches);
    const cudaError_t e = cudaGetLastError();
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
    float* sc = scratch(sizeof(float) * (GCV_FLOATS + 2) * n);
    if (!sc) return fail(CVTPM_ERR_ALLOC, "gcv: scratch allocation failed");
    float* own0 = sc + GCV_FLOATS * n;
    float* own1 = own0 + n;
    float* p0 = d0 ? d0 : own0;
    float* p1 = d1 ? d1 : own1;
    const size_t pp = d0 ? dpitch : (size_t)width * 4;
    cudaStream_t st = (cudaStream_t)stream;
    int launches = 0;
    const Img a{(float*)cam0, width, height, 4}, b{(float*)cam1, width, height, 4};
    depthmap(p0, pp, a, b, dmin, dmax, dt, sc, st, &launches);
    depthmap(p1, pp, b, a, -dmin, -dmax, -dt, sc, st, &launches);
    /* the two depth maps as GRAY images of pitch pp */
    const Img i0{p0, width, height, 1}, i1{p1, width, height, 1};
    k_occlusion<<<g32(width, height), dim3(32, 8), 0, st>>>(dst, dst_pitch, i0, i1, fabsf(dmax));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("gcv: ") + cudaGetErrorString(e));
}

}  // extern "C"
