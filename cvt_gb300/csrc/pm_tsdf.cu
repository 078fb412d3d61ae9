/*
 * pm_tsdf.cu — TSDF fusion of depth maps (the consumer of the disparity maps):
 * cvt::TSDFVolume (cvt/vision/TSDFVolume.h, TSDFVolume.cpp) with the kernels
 * of cvt/cl/kernel/TSDFVolume/TSDFVolume.cl.
 *
 *   k_tsdf_clear    TSDFVolume_clear:  every voxel (1, weight)
 *   k_tsdf_add      TSDFVolume_add:    project the voxel with TG2CAM = proj *
 *                   grid-to-world, read the depth map at the nearest texel and
 *                   fold the truncated signed distance into a running mean
 *   k_tsdf_raycast  TSDFVolume_rayCastDepthmap: march each pixel's ray through
 *                   the volume (half a voxel along its dominant axis) with
 *                   trilinear reads and report the depth of the first + to -
 *                   crossing
 *   k_tsdf_slice    TSDFVolume_sliceX/Y/Z (the reference's host wrappers are
 *                   empty; the kernels' arithmetic is given here)
 *
 * The volume is W*H*D float2 (tsdf, weight), x fastest (TSDFVolume.cpp:38).
 * Matrices are row-major 4x4, as the kernels' Mat4f (cvt/cl/kernel/Matrix4.cl)
 * and cvt::Matrix4f store them.  Host matrix products follow Matrix4.h:269-288
 * (left-to-right sums) and the inverse Matrix.cpp:109-196 (cofactors; a
 * matrix with |det| < FLT_EPSILON is returned unchanged, as inverseSelf
 * leaves it).  Device arithmetic is the kernels' own, compiled without
 * contraction; OpenCL's normalize is v * (1 / sqrt(dot(v, v))) and dot is
 * summed left to right.  Clear is an HBM write stream (8 B per voxel); add
 * projects every voxel (two divisions: issue-bound) and reads and writes 16 B
 * only inside the truncation band; the ray cast is a latency-bound gather.
 *
 * The ray loop of the reference (`for (lambda = start + step; lambda <= end;
 * lambda += step)`) never ends where lambda + step rounds to lambda (a camera
 * ~2^24 voxels from the volume).  Here it stops after 2 * max(W, H, D) + 16
 * steps — more than the 2 steps per voxel along the dominant axis a ray can
 * take — and such a pixel keeps the value 0.
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "cvtpm.h"
#include "pm_kernels.cuh"

namespace {

struct Mat4 {
    float m[16];
};

/* Matrix4::operator* (Matrix4.h:269-288) */
Mat4 mat4_mul(const Mat4& a, const Mat4& b) {
    Mat4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i * 4 + j] = a.m[i * 4] * b.m[j] + a.m[i * 4 + 1] * b.m[4 + j] + a.m[i * 4 + 2] * b.m[8 + j] +
                             a.m[i * 4 + 3] * b.m[12 + j];
    return r;
}

/* Matrix4::inverseSelf (Matrix.cpp:109-196): 2x2 and 3x3 minors of the
 * Laplace expansion, in the reference's order; |det| < FLT_EPSILON leaves the
 * matrix as it is. */
Mat4 mat4_inverse(const Mat4& in) {
    const float* a = in.m;
#define M(i, j) a[(i) * 4 + (j)]
    const float d23_01 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1), d23_02 = M(2, 0) * M(3, 2) - M(3, 0) * M(2, 2);
    const float d23_03 = M(2, 0) * M(3, 3) - M(3, 0) * M(2, 3), d23_12 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    const float d23_13 = M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3), d23_23 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    const float c123_123 = M(1, 1) * d23_23 - M(1, 2) * d23_13 + M(1, 3) * d23_12;
    const float c123_023 = M(1, 0) * d23_23 - M(1, 2) * d23_03 + M(1, 3) * d23_02;
    const float c123_013 = M(1, 0) * d23_13 - M(1, 1) * d23_03 + M(1, 3) * d23_01;
    const float c123_012 = M(1, 0) * d23_12 - M(1, 1) * d23_02 + M(1, 2) * d23_01;
    const float det = M(0, 0) * c123_123 - M(0, 1) * c123_023 + M(0, 2) * c123_013 - M(0, 3) * c123_012;
    if (fabsf(det) < FLT_EPSILON) return in;
    const float inv = 1.0f / det;
    const float c023_123 = M(0, 1) * d23_23 - M(0, 2) * d23_13 + M(0, 3) * d23_12;
    const float c023_023 = M(0, 0) * d23_23 - M(0, 2) * d23_03 + M(0, 3) * d23_02;
    const float c023_013 = M(0, 0) * d23_13 - M(0, 1) * d23_03 + M(0, 3) * d23_01;
    const float c023_012 = M(0, 0) * d23_12 - M(0, 1) * d23_02 + M(0, 2) * d23_01;
    const float d13_01 = M(1, 0) * M(3, 1) - M(3, 0) * M(1, 1), d13_02 = M(1, 0) * M(3, 2) - M(3, 0) * M(1, 2);
    const float d13_03 = M(1, 0) * M(3, 3) - M(3, 0) * M(1, 3), d13_12 = M(1, 1) * M(3, 2) - M(3, 1) * M(1, 2);
    const float d13_13 = M(1, 1) * M(3, 3) - M(3, 1) * M(1, 3), d13_23 = M(1, 2) * M(3, 3) - M(3, 2) * M(1, 3);
    const float c013_123 = M(0, 1) * d13_23 - M(0, 2) * d13_13 + M(0, 3) * d13_12;
    const float c013_023 = M(0, 0) * d13_23 - M(0, 2) * d13_03 + M(0, 3) * d13_02;
    const float c013_013 = M(0, 0) * d13_13 - M(0, 1) * d13_03 + M(0, 3) * d13_01;
    const float c013_012 = M(0, 0) * d13_12 - M(0, 1) * d13_02 + M(0, 2) * d13_01;
    const float d12_01 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1), d12_02 = M(1, 0) * M(2, 2) - M(2, 0) * M(1, 2);
    const float d12_03 = M(1, 0) * M(2, 3) - M(2, 0) * M(1, 3), d12_12 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    const float d12_13 = M(1, 1) * M(2, 3) - M(2, 1) * M(1, 3), d12_23 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    const float c012_123 = M(0, 1) * d12_23 - M(0, 2) * d12_13 + M(0, 3) * d12_12;
    const float c012_023 = M(0, 0) * d12_23 - M(0, 2) * d12_03 + M(0, 3) * d12_02;
    const float c012_013 = M(0, 0) * d12_13 - M(0, 1) * d12_03 + M(0, 3) * d12_01;
    const float c012_012 = M(0, 0) * d12_12 - M(0, 1) * d12_02 + M(0, 2) * d12_01;
#undef M
    const Mat4 r = {{c123_123 * inv, -c023_123 * inv, c013_123 * inv, -c012_123 * inv,
                     -c123_023 * inv, c023_023 * inv, -c013_023 * inv, c012_023 * inv,
                     c123_013 * inv, -c023_013 * inv, c013_013 * inv, -c012_013 * inv,
                     -c123_012 * inv, c023_012 * inv, -c013_012 * inv, c012_012 * inv}};
    return r;
}

/* ------------------------------------------------------------ device -- */
struct DMat4 {
    float4 r[4];
};

DMat4 to_dev(const Mat4& a) {
    DMat4 d;
    for (int i = 0; i < 4; ++i) d.r[i] = make_float4(a.m[i * 4], a.m[i * 4 + 1], a.m[i * 4 + 2], a.m[i * 4 + 3]);
    return d;
}

/* dot4 (pm_device.cuh) sums left to right, as OpenCL's dot is emulated */
__device__ __forceinline__ float4 xform(const DMat4& m, float4 v) {   /* mat4f_transform (Matrix4.cl) */
    return make_float4(dot4(m.r[0], v), dot4(m.r[1], v), dot4(m.r[2], v), dot4(m.r[3], v));
}
__device__ __forceinline__ float mixf(float a, float b, float t) { return a + (b - a) * t; }

/* clear: two voxels per 16-byte store over the linear volume (512^3: 0.141 ms
 * = 7.6 TB/s, against 0.267 ms with one 8-byte store per voxel).  add:
 * TSDF_ZPT z-planes per thread (512^3, 640x480 map: 1 plane 0.310 ms, 2 0.306,
 * 4 0.249, 8 0.220). */
#define TSDF_CLEAR_VEC 1
#define TSDF_ZPT 8
__global__ void __launch_bounds__(256) k_tsdf_clear(float2* __restrict__ cv, int W, int H, int D, float init) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= W || y >= H || z >= D) return;
    cv[((size_t)z * H + y) * W + x] = make_float2(1.0f, init);
}

/* The same over the volume as n voxels: thread i writes voxels 2i and 2i+1
 * with one 16-byte store (the allocation is 256-byte aligned). */
__global__ void __launch_bounds__(256) k_tsdf_clear_vec(float4* __restrict__ cv4, size_t n, float init) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * i + 1 < n) cv4[i] = make_float4(1.0f, init, 1.0f, init);
    else if (2 * i < n) ((float2*)cv4)[2 * i] = make_float2(1.0f, init);
}

__device__ __forceinline__ void tsdf_add_voxel(float2* __restrict__ cv, int W, int H, int x, int y, int z,
                                               const float* __restrict__ dmap, size_t dpitch4, int iw, int ih,
                                               float dscale, const DMat4& tg2cam, float trunc) {
    const float4 g = xform(tg2cam, make_float4((float)x, (float)y, (float)z, 1.0f));
    /* Voxels the update would skip anyway, found without the two divisions:
     * it needs g.z > 0 (the depth read before that test has no effect), and
     * for g.z > 0 a numerator beyond -2 g.z or (size + 2) g.z makes the
     * rounded quotient < 0 or > size (the product rounds by at most one part
     * in 2^24).  NaN and infinite values fall through to the full test. */
    if (!(g.z > 0.0f)) return;
    const float lo = -2.0f * g.z;
    if (g.x < lo || g.y < lo || g.x > ((float)iw + 2.0f) * g.z || g.y > ((float)ih + 2.0f) * g.z) return;
    const float ix = g.x / g.z, iy = g.y / g.z;
    if (ix < (float)iw && iy < (float)ih && ix >= 0.0f && iy >= 0.0f) {
        const float d = dmap[(size_t)(int)floorf(iy) * dpitch4 + (int)floorf(ix)] * dscale;   /* nearest texel */
        if (d > 0.0f && g.z > 0.0f) {
            const float sdf = d - g.z, w = 1.0f;
            const float tsdf = sdf / trunc;
            if (fabsf(sdf) <= trunc) {
                float2* p = cv + ((size_t)z * H + y) * W + x;
                const float2 o = *p;
                *p = make_float2((o.x * o.y + tsdf * w) / (o.y + w), o.y + w);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_tsdf_add(float2* __restrict__ cv, int W, int H, int D,
                                                  const float* __restrict__ dmap, size_t dpitch4, int iw, int ih,
                                                  float dscale, DMat4 tg2cam, float trunc) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= W || y >= H) return;
#pragma unroll 1
    for (int z = blockIdx.z * TSDF_ZPT; z < min(D, (int)(blockIdx.z + 1) * TSDF_ZPT); ++z)
        tsdf_add_voxel(cv, W, H, x, y, z, dmap, dpitch4, iw, ih, dscale, tg2cam, trunc);
}

/* TSDFVolume_trilinearValue: 1e10 if a corner has weight < 1 */
__device__ __forceinline__ float trilinear(const float2* __restrict__ cv, int W, int H, int D, float px, float py,
                                           float pz) {
    px = fminf(fmaxf(0.0f, px), (float)(W - 2));
    py = fminf(fmaxf(0.0f, py), (float)(H - 2));
    pz = fminf(fmaxf(0.0f, pz), (float)(D - 2));
    const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
    const float ax = px - bx, ay = py - by, az = pz - bz;
    const int ix = (int)bx, iy = (int)by, iz = (int)bz;
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {   /* s0..s7: x fastest, then y, then z */
        const float2 t = cv[((size_t)(iz + (k >> 2)) * H + (iy + ((k >> 1) & 1))) * W + (ix + (k & 1))];
        if (t.y < 1.0f) return 1e10f;
        v[k] = t.x;
    }
    const float z0 = mixf(v[0], v[4], az), z1 = mixf(v[1], v[5], az), z2 = mixf(v[2], v[6], az), z3 = mixf(v[3], v[7], az);
    const float y0 = mixf(z0, z2, ay), y1 = mixf(z1, z3, ay);
    return mixf(y0, y1, ax);
}

__device__ __forceinline__ float ray_bound(float o, float d, int extent, bool start) {
    return (((d > 0.0f) == start ? 0.0f : (float)extent) - o) / d;
}

__global__ void __launch_bounds__(256) k_tsdf_raycast(float* __restrict__ out, size_t opitch4, int iw, int ih,
                                                      const float2* __restrict__ cv, int W, int H, int D,
                                                      DMat4 tcam2g, DMat4 tg2cam, float scale, int max_steps) {
    const int gx = blockIdx.x * 32 + threadIdx.x, gy = blockIdx.y * 8 + threadIdx.y;
    if (gx >= iw || gy >= ih) return;
    const float4 o4 = xform(tcam2g, make_float4(0.0f, 0.0f, 0.0f, 1.0f));
    const float4 t4 = xform(tcam2g, make_float4((float)gx, (float)gy, 1.0f, 1.0f));
    float dx = t4.x - o4.x, dy = t4.y - o4.y, dz = t4.z - o4.z;
    const float rn = 1.0f / sqrtf((dx * dx + dy * dy) + dz * dz);   /* normalize */
    dx = dx * rn; dy = dy * rn; dz = dz * rn;
    const float rs = fmaxf(fmaxf(ray_bound(o4.x, dx, W, true), ray_bound(o4.y, dy, H, true)), ray_bound(o4.z, dz, D, true));
    const float re = fminf(fminf(ray_bound(o4.x, dx, W, false), ray_bound(o4.y, dy, H, false)), ray_bound(o4.z, dz, D, false));
    float ret = 0.0f;
    if (rs < re && isfinite(rs) && isfinite(re) && isfinite(dx) && isfinite(dy) && isfinite(dz)) {
        const float vx = fabsf(dx * (re - rs)), vy = fabsf(dy * (re - rs)), vz = fabsf(dz * (re - rs));
        const float step = 0.5f * sqrtf((vx * vx + vy * vy) + vz * vz) / fmaxf(vx, fmaxf(vy, vz));
        float ppx = o4.x + dx * rs, ppy = o4.y + dy * rs, ppz = o4.z + dz * rs;
        float vp = trilinear(cv, W, H, D, ppx, ppy, ppz);
        int n = 0;
        for (float lambda = rs + step; lambda <= re && n < max_steps; lambda += step, ++n) {
            const float px = o4.x + dx * lambda, py = o4.y + dy * lambda, pz = o4.z + dz * lambda;
            const float v = trilinear(cv, W, H, D, px, py, pz);
            if (vp < 0.0f && v > 0.0f) break;
            if (vp > 0.0f && v < 0.0f) {
                const float alpha = -v / (vp - v);
                const float g = mixf(pz, ppz, alpha);   /* the reference mixes z only and uses it for x, y, z */
                ret = fmaxf(-(dot4(tg2cam.r[2], make_float4(g, g, g, 1.0f))) * scale, 0.0f);
                break;
            }
            vp = v;
            ppx = px; ppy = py; ppz = pz;
        }
    }
    out[(size_t)gy * opitch4 + gx] = ret;
}

/* TSDFVolume_sliceX/Y/Z: RGBA (clamp(tsdf + 0.5, 0, 1) x3, 1) at plane v */
__global__ void __launch_bounds__(256) k_tsdf_slice(float4* __restrict__ out, size_t opitch4, int axis, int v,
                                                    const float2* __restrict__ cv, int W, int H, int D, int ow, int oh) {
    const int a = blockIdx.x * 32 + threadIdx.x, b = blockIdx.y * 8 + threadIdx.y;
    if (a >= ow || b >= oh) return;
    const int x = axis == 0 ? v : a, y = axis == 0 ? a : (axis == 1 ? v : b), z = axis == 2 ? v : b;
    const float t = fminf(fmaxf(cv[((size_t)z * H + y) * W + x].x + 0.5f, 0.0f), 1.0f);
    out[(size_t)b * opitch4 + a] = make_float4(t, t, t, 1.0f);
}

cvtpm_status fail(cvtpm_status s, const std::string& m) {
    pm_set_free_error(m);
    return s;
}

bool finite16(const float* m) {
    for (int i = 0; i < 16; ++i)
        if (!isfinite(m[i])) return false;
    return true;
}

}  // namespace

struct cvtpm_tsdf {
    int device;
    int W, H, D;
    float trunc;
    Mat4 g2w;
    float2* vol;
};

/* Vision::disparityToDepthmap (cvt/vision/Vision.cpp:147-168): the depth
 * (focallength * baseline) / (disparity * dispscale) where the scaled
 * disparity exceeds dispthres, else 0.  8 bytes per pixel: HBM-bound. */
__global__ void __launch_bounds__(256) k_disparity_to_depth(float* __restrict__ depth, size_t dp,
                                                            const float* __restrict__ disp, size_t sp, int W, int H,
                                                            float dispscale, float fb, float thres) {
    const int x = blockIdx.x * 64 + threadIdx.x, y = blockIdx.y * 4 + threadIdx.y;
    if (x >= W || y >= H) return;
    const float d = disp[(size_t)y * sp + x] * dispscale;
    depth[(size_t)y * dp + x] = d > thres ? fb / d : 0.0f;
}

extern "C" {

cvtpm_status cvtpm_tsdf_projection(const float* intrinsics, const float* extrinsics, float* proj) {
    if (!intrinsics || !extrinsics || !proj) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf projection: NULL argument");
    Mat4 K = {{intrinsics[0], intrinsics[1], intrinsics[2], 0.0f, intrinsics[3], intrinsics[4], intrinsics[5], 0.0f,
               intrinsics[6], intrinsics[7], intrinsics[8], 0.0f, 0.0f, 0.0f, 0.0f, 1.0f}};   /* Matrix3::toMatrix4 */
    Mat4 E;
    memcpy(E.m, extrinsics, sizeof E.m);
    const Mat4 P = mat4_mul(K, E);   /* proj = K.toMatrix4(); proj *= extrinsics (TSDFVolume.cpp:79-84) */
    memcpy(proj, P.m, sizeof P.m);
    return CVTPM_OK;
}

cvtpm_status cvtpm_tsdf_create(cvtpm_tsdf** out, int device, const float* grid_to_world, int width, int height,
                               int depth, float truncation) {
    if (!out || !grid_to_world) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf create: NULL argument");
    *out = nullptr;
    if (width < 2 || height < 2 || depth < 2 || width > 4096 || height > 4096 || depth > 4096)
        return fail(CVTPM_ERR_SIZE, "tsdf create: each dimension must be 2..4096");
    if (!finite16(grid_to_world) || !(truncation > 0.0f)) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf create: bad grid-to-world or truncation");
    if (cudaSetDevice(device) != cudaSuccess) return fail(CVTPM_ERR_CUDA, "tsdf create: cudaSetDevice");
    cvtpm_tsdf* v = new cvtpm_tsdf();
    v->device = device;
    v->W = width; v->H = height; v->D = depth;
    v->trunc = truncation;
    memcpy(v->g2w.m, grid_to_world, sizeof v->g2w.m);
    if (cudaMalloc(&v->vol, sizeof(float2) * (size_t)width * height * depth) != cudaSuccess) {
        cudaGetLastError();
        delete v;
        return fail(CVTPM_ERR_ALLOC, "tsdf create: volume allocation failed");
    }
    *out = v;
    return CVTPM_OK;
}

cvtpm_status cvtpm_tsdf_destroy(cvtpm_tsdf* v) {
    if (!v) return CVTPM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(v->device);
    cudaFree(v->vol);
    delete v;
    return CVTPM_OK;
}

cvtpm_status cvtpm_tsdf_info(const cvtpm_tsdf* v, int* width, int* height, int* depth, void** data) {
    if (!v) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf info: NULL volume");
    if (width) *width = v->W;
    if (height) *height = v->H;
    if (depth) *depth = v->D;
    if (data) *data = v->vol;
    return CVTPM_OK;
}

cvtpm_status cvtpm_tsdf_clear(cvtpm_tsdf* v, float weight, void* stream) {
    if (!v) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf clear: NULL volume");
    cudaSetDevice(v->device);
    if (TSDF_CLEAR_VEC) {
        const size_t n = (size_t)v->W * v->H * v->D, th = (n + 1) / 2;
        k_tsdf_clear_vec<<<(unsigned)((th + 255) / 256), 256, 0, (cudaStream_t)stream>>>((float4*)v->vol, n, weight);
    } else {
        k_tsdf_clear<<<dim3((v->W + 31) / 32, (v->H + 7) / 8, v->D), dim3(32, 8), 0, (cudaStream_t)stream>>>(
            v->vol, v->W, v->H, v->D, weight);
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("tsdf clear: ") + cudaGetErrorString(e));
}

cvtpm_status cvtpm_tsdf_add_depthmap(cvtpm_tsdf* v, const float* proj, const float* depthmap, int dwidth, int dheight,
                                     size_t dpitch, float scale, void* stream) {
    if (!v || !proj || !depthmap) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf add: NULL argument");
    if (dwidth < 1 || dheight < 1) return fail(CVTPM_ERR_SIZE, "tsdf add: empty depth map");
    if (dpitch % 4 || dpitch < (size_t)dwidth * 4) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf add: bad depth map pitch");
    if (!finite16(proj)) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf add: non-finite projection");
    Mat4 P;
    memcpy(P.m, proj, sizeof P.m);
    const DMat4 T = to_dev(mat4_mul(P, v->g2w));   /* projall = proj * g2w (TSDFVolume.cpp:64) */
    cudaSetDevice(v->device);
    k_tsdf_add<<<dim3((v->W + 31) / 32, (v->H + 7) / 8, (v->D + TSDF_ZPT - 1) / TSDF_ZPT), dim3(32, 8), 0,
                 (cudaStream_t)stream>>>(
        v->vol, v->W, v->H, v->D, depthmap, dpitch / 4, dwidth, dheight, scale, T, v->trunc);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("tsdf add: ") + cudaGetErrorString(e));
}

cvtpm_status cvtpm_tsdf_raycast(cvtpm_tsdf* v, const float* proj, float* depthmap, int dwidth, int dheight,
                                size_t dpitch, float scale, void* stream) {
    if (!v || !proj || !depthmap) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf raycast: NULL argument");
    if (dwidth < 1 || dheight < 1) return fail(CVTPM_ERR_SIZE, "tsdf raycast: empty depth map");
    if (dpitch % 4 || dpitch < (size_t)dwidth * 4) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf raycast: bad depth map pitch");
    if (!finite16(proj)) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf raycast: non-finite projection");
    Mat4 P;
    memcpy(P.m, proj, sizeof P.m);
    const Mat4 all = mat4_mul(P, v->g2w);
    const DMat4 T = to_dev(all), Ti = to_dev(mat4_inverse(all));
    const int max_steps = 2 * (v->W > v->H ? (v->W > v->D ? v->W : v->D) : (v->H > v->D ? v->H : v->D)) + 16;
    cudaSetDevice(v->device);
    k_tsdf_raycast<<<dim3((dwidth + 31) / 32, (dheight + 7) / 8), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        depthmap, dpitch / 4, dwidth, dheight, v->vol, v->W, v->H, v->D, Ti, T, scale, max_steps);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("tsdf raycast: ") + cudaGetErrorString(e));
}

cvtpm_status cvtpm_tsdf_slice(cvtpm_tsdf* v, int axis, int index, float* rgba, size_t pitch, void* stream) {
    if (!v || !rgba) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf slice: NULL argument");
    if (axis < 0 || axis > 2) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf slice: axis must be 0 (x), 1 (y) or 2 (z)");
    const int ext = axis == 0 ? v->W : (axis == 1 ? v->H : v->D);
    if (index < 0 || index >= ext) return fail(CVTPM_ERR_SIZE, "tsdf slice: index outside the volume");
    const int ow = axis == 0 ? v->H : v->W, oh = axis == 2 ? v->H : v->D;
    if (pitch % 16 || pitch < (size_t)ow * 16) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf slice: bad pitch");
    cudaSetDevice(v->device);
    k_tsdf_slice<<<dim3((ow + 31) / 32, (oh + 7) / 8), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        (float4*)rgba, pitch / 16, axis, index, v->vol, v->W, v->H, v->D, ow, oh);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("tsdf slice: ") + cudaGetErrorString(e));
}

cvtpm_status cvtpm_tsdf_save_raw(cvtpm_tsdf* v, const char* path, int weighted) {
    if (!v || !path) return fail(CVTPM_ERR_INVALID_ARGUMENT, "tsdf save: NULL argument");
    const size_t n = (size_t)v->W * v->H * v->D;
    std::vector<float> host(2 * n);
    cudaSetDevice(v->device);
    if (cudaMemcpy(host.data(), v->vol, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(CVTPM_ERR_CUDA, "tsdf save: copy failed");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(CVTPM_ERR_IO, std::string("tsdf save: cannot open ") + path);
    bool ok;
    if (weighted) {   /* (tsdf, weight) pairs; else the tsdf values alone (TSDFVolume.cpp:130-152) */
        ok = fwrite(host.data(), sizeof(float), 2 * n, f) == 2 * n;
    } else {
        for (size_t i = 0; i < n; ++i) host[i] = host[2 * i];
        ok = fwrite(host.data(), sizeof(float), n, f) == n;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? CVTPM_OK : fail(CVTPM_ERR_IO, std::string("tsdf save: write failed for ") + path);
}

}  // extern "C"

extern "C" cvtpm_status cvtpm_disparity_to_depth(float* depth, size_t depth_pitch, const float* disparity,
                                                 size_t disp_pitch, int width, int height, float dispscale,
                                                 float focallength, float baseline, float dispthres, void* stream) {
    if (!depth || !disparity) return fail(CVTPM_ERR_INVALID_ARGUMENT, "disparity to depth: NULL argument");
    if (width < 1 || height < 1) return fail(CVTPM_ERR_SIZE, "disparity to depth: empty image");
    if (depth_pitch % 4 || disp_pitch % 4 || depth_pitch < (size_t)width * 4 || disp_pitch < (size_t)width * 4)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "disparity to depth: bad pitch");
    const float fb = focallength * baseline;   /* Vision.cpp:153, in float */
    k_disparity_to_depth<<<dim3((width + 63) / 64, (height + 3) / 4), dim3(64, 4), 0, (cudaStream_t)stream>>>(
        depth, depth_pitch / 4, disparity, disp_pitch / 4, width, height, dispscale, fb, dispthres);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CVTPM_OK : fail(CVTPM_ERR_CUDA, std::string("disparity to depth: ") + cudaGetErrorString(e));
}
