/*
 * pm_rectify.cu — stereo rectification for real pairs: the rectified
 * calibration (host), the undistort-rectify warp maps and the bilinear
 * resampling through them (device).
 *
 *   host   StereoCameraCalibration::rectificationMatrices / undistortRectify
 *          (cvt/vision/StereoCameraCalibration.h:166-277), with the
 *          Matrix3 / Quaternion / Vector3 operations they use
 *          (cvt/math/Matrix3.h:257-286,508-553; Quaternion.h:128-164,517-523;
 *          Vector3.h:120-126,176-199,275-282,332-356)
 *   device UndistortRectifyWarp::operator() (StereoCameraCalibration.h:79-92)
 *          evaluated per output pixel, as IWarp::warpGeneric does
 *          (cvt/gfx/ifilter/IWarp.h:80-99)
 *   device IWarp::apply (cvt/gfx/ifilter/IWarp.cpp:49-66,254-376) with the
 *          bilinear samplers SIMD::warpBilinear1f / 4f / 1u8 / 4u8
 *          (cvt/util/SIMD.cpp:4497-4710) and their helpers _floor (:732-739)
 *          and _mix4U8 (:702-717)
 *
 * The host part is float arithmetic in the reference's operation order with
 * the C library's sqrtf / sinf / cosf / acosf (the reference's Math:: wrappers
 * call the same functions); compiled without contraction.  The kernels use no
 * transcendental function: -fmad=false and IEEE division make them bit-exact
 * against the same arithmetic on the CPU.  Both kernels are HBM-bound gathers
 * (maps: 8 bytes written per pixel; resampling: 8 bytes of map + 4 texels
 * read, one pixel written).
 */
#include <math.h>
#include <string.h>

#include <string>

#include "cvtpm.h"
#include "pm_kernels.cuh"

namespace {

/* ----------------------------------------------------------- host math -- */
struct M3 {
    float m[3][3];
};
struct V3 {
    float x, y, z;
};

M3 m3_mul(const M3& a, const M3& b) {   /* Matrix3.h:275-286 */
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}

V3 m3_mul(const M3& a, const V3& v) {   /* Matrix3.h:257-262 */
    return V3{a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
              a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z};
}

M3 m3_transpose(const M3& a) {
    M3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[j][i];
    return r;
}

float v3_dot(const V3& self, const V3& v) { return v.x * self.x + v.y * self.y + v.z * self.z; }   /* Vector3.h:176-179 */

V3 v3_cross(const V3& a, const V3& v) {   /* Vector3.h:188-191 */
    return V3{a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x};
}

void v3_normalize(V3& v) {   /* Vector3.h:344-352: multiply by 1/sqrt(length^2) */
    const float lenSqr = v.x * v.x + v.y * v.y + v.z * v.z;
    const float inv = 1.0f / sqrtf(lenSqr);
    v.x *= inv;
    v.y *= inv;
    v.z *= inv;
}

float v3_length(const V3& v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }   /* Vector3.h:332-335 */

/* Matrix3::setRotation (Matrix3.h:508-553): the rotation matrix of the
 * normalized axis and angle, through the half-angle quaternion. */
M3 rotation(V3 axis, float rad) {
    v3_normalize(axis);
    const float c = cosf(rad * 0.5f), s = sinf(rad * 0.5f);
    const float x = axis.x * s, y = axis.y * s, z = axis.z * s;
    const float x2 = x + x, y2 = y + y, z2 = z + z;
    const float xx = x * x2, xy = x * y2, xz = x * z2;
    const float yy = y * y2, yz = y * z2, zz = z * z2;
    const float wx = c * x2, wy = c * y2, wz = c * z2;
    M3 r;
    r.m[0][0] = 1.0f - (yy + zz);
    r.m[0][1] = xy - wz;
    r.m[0][2] = xz + wy;
    r.m[1][0] = xy + wz;
    r.m[1][1] = 1.0f - (xx + zz);
    r.m[1][2] = yz - wx;
    r.m[2][0] = xz - wy;
    r.m[2][1] = yz + wx;
    r.m[2][2] = 1.0f - (xx + yy);
    return r;
}

/* Matrix3::toAxisAngle through Quaternion(Matrix3) (Shoemake; Quaternion.h:
 * 128-164) and Quaternion::toAxisAngle (:517-523). */
void axis_angle(const M3& R, V3* axis, float* angle) {
    float q[3], w;
    const float tr = R.m[0][0] + R.m[1][1] + R.m[2][2];
    if (tr > 0.0f) {
        float root = sqrtf(tr + 1.0f);
        w = 0.5f * root;
        root = 0.5f / root;
        q[0] = (R.m[2][1] - R.m[1][2]) * root;
        q[1] = (R.m[0][2] - R.m[2][0]) * root;
        q[2] = (R.m[1][0] - R.m[0][1]) * root;
    } else {
        int i = 0;
        if (R.m[1][1] > R.m[0][0]) i = 1;
        if (R.m[2][2] > R.m[i][i]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        float root = sqrtf(R.m[i][i] - R.m[j][j] - R.m[k][k] + 1.0f);
        q[i] = 0.5f * root;
        root = 0.5f / root;
        w = (R.m[k][j] - R.m[j][k]) * root;
        q[j] = (R.m[j][i] + R.m[i][j]) * root;
        q[k] = (R.m[k][i] + R.m[i][k]) * root;
    }
    *angle = acosf(w) * 2.0f;
    const float s = sinf(*angle * 0.5f);
    V3 a{q[0] / s, q[1] / s, q[2] / s};   /* Vector3::operator/= divides */
    v3_normalize(a);
    *axis = a;
}

/* Vector3f(Matrix4::col(3)): the homogeneous point, 1/w formed in double
 * (Vector3.h:120-126). */
V3 translation(const float* E) {
    const float invw = (float)(1.0 / (double)E[15]);
    return V3{invw * E[3], invw * E[7], invw * E[11]};
}

/* StereoCameraCalibration::rectificationMatrices with verticalstereo = false
 * (StereoCameraCalibration.h:166-197). */
void rect_matrices(const float* E, M3* Rl, M3* Rr) {
    M3 R;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R.m[i][j] = E[i * 4 + j];
    V3 axis;
    float angle;
    axis_angle(R, &axis, &angle);
    *Rl = rotation(axis, 0.5f * angle);
    *Rr = rotation(axis, -0.5f * angle);
    const V3 t = m3_mul(*Rr, translation(E));
    V3 u{1.0f, 0.0f, 0.0f};
    if (v3_dot(u, t) < 0.0f) u = V3{-u.x, -u.y, -u.z};
    V3 ax = v3_cross(t, u);
    v3_normalize(ax);
    const float ang = acosf(fabsf(v3_dot(t, u)) / v3_length(t));
    const M3 R2 = rotation(ax, ang);
    *Rr = m3_mul(R2, *Rr);
    *Rl = m3_mul(R2, *Rl);
}

/* UndistortRectifyWarp's constants (StereoCameraCalibration.h:66-101). */
struct RectOp {
    float fnx, fny, cnx, cny;
    float rot[9];
    float k0, k1, k2, t0, t1;
    float fox, foy, cox, coy;
};

RectOp make_op(float fnew, float cx, float cy, const M3& Rt, const cvtpm_camera& cam) {
    RectOp o;
    o.fnx = o.fny = fnew;
    o.cnx = cx;
    o.cny = cy;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o.rot[i * 3 + j] = Rt.m[i][j];
    o.k0 = cam.radial[0];
    o.k1 = cam.radial[1];
    o.k2 = cam.radial[2];
    o.t0 = cam.tangential[0];
    o.t1 = cam.tangential[1];
    o.fox = cam.intrinsics[0];
    o.foy = cam.intrinsics[4];
    o.cox = cam.intrinsics[2];
    o.coy = cam.intrinsics[5];
    return o;
}

/* ------------------------------------------------------------ kernels -- */
/* UndistortRectifyWarp::operator() at pixel (x, y) (:79-92). */
__global__ void __launch_bounds__(256) k_rectify_map(RectOp o, int W, int H, float2* __restrict__ map, size_t pitch2) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= W || y >= H) return;
    const float dx = ((float)x - o.cnx) / o.fnx, dy = ((float)y - o.cny) / o.fny;
    const float hz = o.rot[6] * dx + o.rot[7] * dy + o.rot[8];
    const float px = (o.rot[0] * dx + o.rot[1] * dy + o.rot[2]) / hz;   /* Matrix3 * Vector2: homogeneous */
    const float py = (o.rot[3] * dx + o.rot[4] * dy + o.rot[5]) / hz;
    const float r2 = px * px + py * py;
    const float r4 = r2 * r2;
    const float r6 = r2 * r4;
    const float poly = 1.0f + o.k0 * r2 + o.k1 * r4 + o.k2 * r6;
    const float xy2 = 2.0f * px * py;
    const float mx = o.fox * (px * poly + xy2 * o.t0 + o.t1 * (r2 + 2.0f * px * px)) + o.cox;
    const float my = o.foy * (py * poly + xy2 * o.t1 + o.t0 * (r2 + 2.0f * py * py)) + o.coy;
    map[(size_t)y * pitch2 + x] = make_float2(mx, my);
}

enum { WARP_F1, WARP_F4, WARP_U8C1, WARP_U8C4 };

/* SIMD.cpp:732-739: truncation minus the sign bit (one below the floor for
 * negative integers and -0). */
__device__ __forceinline__ int ref_floor(float v) { return (int)v - (int)(__float_as_uint(v) >> 31); }

__device__ __forceinline__ float mixf(float a, float b, float t) { return a + (b - a) * t; }   /* Math.h:77 */

__device__ __forceinline__ uint32_t mix4u8(uint32_t s1, uint32_t s2, uint32_t a) {   /* SIMD.cpp:702-717 */
    uint32_t t = ((s2 >> 8) & 0xff00ffu) - ((s1 >> 8) & 0xff00ffu);
    t *= a;
    t += s1 & 0xff00ff00u;
    t &= 0xff00ff00u;
    uint32_t t2 = (s2 & 0xff00ffu) - (s1 & 0xff00ffu);
    t2 *= a;
    t2 = t2 >> 8;
    t2 += s1 & 0xff00ffu;
    t2 &= 0xff00ffu;
    return t + t2;
}

/* One output pixel of IWarp::apply: source coordinates c, output row `out`. */
template <int KIND>
__device__ __forceinline__ void warp_px(const unsigned char* __restrict__ src, size_t sstride, int sw, int sh,
                                        float2 c, unsigned char* __restrict__ out, int x) {
    if (KIND == WARP_F1 || KIND == WARP_F4) {
        constexpr int C = KIND == WARP_F1 ? 1 : 4;
        const float fill[4] = {0.0f, 0.0f, 0.0f, C == 1 ? 0.0f : 1.0f};
        float* o = (float*)out + (size_t)x * C;
        const bool ok = fabsf(c.x) < 2147483520.0f && fabsf(c.y) < 2147483520.0f;   /* finite, int-convertible */
        const int lx = ok ? ref_floor(c.x) : -2, ly = ok ? ref_floor(c.y) : -2;
        if (!(lx >= -1 && lx < sw && ly >= -1 && ly < sh)) {
#pragma unroll
            for (int k = 0; k < C; ++k) o[k] = fill[k];
            return;
        }
        const float a1 = c.x - (float)lx, a2 = c.y - (float)ly;
        const bool inner = lx >= 0 && lx < sw - 1 && ly >= 0 && ly < sh - 1;
#pragma unroll
        for (int k = 0; k < C; ++k) {
            float v00, v10, v01, v11;
            if (inner) {
                const float* r0 = (const float*)(src + (size_t)ly * sstride) + (size_t)lx * C + k;
                const float* r1 = (const float*)(src + (size_t)(ly + 1) * sstride) + (size_t)lx * C + k;
                v00 = r0[0]; v10 = r0[C]; v01 = r1[0]; v11 = r1[C];
            } else {
                auto val = [&](int px, int py) {
                    return (px >= 0 && px < sw && py >= 0 && py < sh)
                               ? ((const float*)(src + (size_t)py * sstride))[(size_t)px * C + k] : fill[k];
                };
                v00 = val(lx, ly); v10 = val(lx + 1, ly); v01 = val(lx, ly + 1); v11 = val(lx + 1, ly + 1);
            }
            o[k] = mixf(mixf(v00, v10, a1), mixf(v01, v11, a1), a2);
        }
    } else if (KIND == WARP_U8C1) {
        if (!(fabsf(c.x) < 32768.0f && fabsf(c.y) < 32768.0f)) { out[x] = 0; return; }
        const int fx = (int)(c.x * 65536.0f), fy = (int)(c.y * 65536.0f);
        const int lx = fx >> 16, ly = fy >> 16;
        const int ax = fx & 0xffff, ay = fy & 0xffff;
        if ((unsigned)lx < (unsigned)(sw - 1) && (unsigned)ly < (unsigned)(sh - 1)) {
            const unsigned char* p = src + (size_t)ly * sstride + lx;
            const int g0 = p[0], g1 = p[1], g2 = p[sstride], g3 = p[sstride + 1];
            const int v1 = g0 + (((g1 - g0) * ax) >> 16);
            const int v2 = g2 + (((g3 - g2) * ax) >> 16);
            out[x] = (unsigned char)(v1 + (((v2 - v1) * ay) >> 16));
        } else if (lx >= -1 && lx < sw && ly >= -1 && ly < sh) {
            auto val = [&](int px, int py) {
                return (px >= 0 && px < sw && py >= 0 && py < sh) ? (int)src[(size_t)py * sstride + px] : 0;
            };
            int a = val(lx, ly), b = val(lx + 1, ly);
            const int v1 = a + (((b - a) * ax) >> 16);
            a = val(lx, ly + 1);
            b = val(lx + 1, ly + 1);
            const int v2 = a + (((b - a) * ax) >> 16);
            out[x] = (unsigned char)(v1 + (((v2 - v1) * ay) >> 16));
        } else {
            out[x] = 0;
        }
    } else {
        const uint32_t fill = 0xff000000u;
        uint32_t* o = (uint32_t*)out + x;
        if (!(fabsf(c.x) < 8388608.0f && fabsf(c.y) < 8388608.0f)) { *o = fill; return; }
        const int fx = (int)(c.x * 256.0f), fy = (int)(c.y * 256.0f);
        const int lx = fx >> 8, ly = fy >> 8;
        const uint32_t a1 = (uint32_t)fx & 0xffu, a2 = (uint32_t)fy & 0xffu;
        auto px_at = [&](int px, int py) { return *(const uint32_t*)(src + (size_t)py * sstride + (size_t)px * 4); };
        if (lx >= 0 && lx < sw - 1 && ly >= 0 && ly < sh - 1) {
            const uint32_t v1 = mix4u8(px_at(lx, ly), px_at(lx + 1, ly), a1);
            const uint32_t v2 = mix4u8(px_at(lx, ly + 1), px_at(lx + 1, ly + 1), a1);
            *o = mix4u8(v1, v2, a2);
        } else if (lx >= -1 && lx < sw && ly >= -1 && ly < sh) {
            auto val = [&](int px, int py) { return (px >= 0 && px < sw && py >= 0 && py < sh) ? px_at(px, py) : fill; };
            const uint32_t v1 = mix4u8(val(lx, ly), val(lx + 1, ly), a1);
            const uint32_t v2 = mix4u8(val(lx, ly + 1), val(lx + 1, ly + 1), a1);
            *o = mix4u8(v1, v2, a2);
        } else {
            *o = fill;
        }
    }
}

/* WARP_PX output pixels per thread, 32 apart (a warp covers WARP_PX runs of 32
 * consecutive pixels): the map loads of all of them are in flight before the
 * dependent texel reads.  3840x2160 RGBA8 pair: 1 px 0.095 ms, 2 px 0.075 ms,
 * 4 px 0.071 ms per step (GB300). */
#define WARP_PX 4
template <int KIND>
__global__ void __launch_bounds__(256) k_warp_apply(const unsigned char* __restrict__ src, size_t sstride, int sw, int sh,
                                                    const float2* __restrict__ map, size_t mpitch2, int W, int H,
                                                    unsigned char* __restrict__ dst, size_t dstride) {
    const int y = blockIdx.y * 8 + threadIdx.y;
    if (y >= H) return;
    const int x0 = blockIdx.x * (32 * WARP_PX) + threadIdx.x;
    float2 c[WARP_PX];
#pragma unroll
    for (int k = 0; k < WARP_PX; ++k)   /* the map loads first, then the dependent texel reads */
        if (x0 + 32 * k < W) c[k] = map[(size_t)y * mpitch2 + x0 + 32 * k];
#pragma unroll
    for (int k = 0; k < WARP_PX; ++k)
        if (x0 + 32 * k < W) warp_px<KIND>(src, sstride, sw, sh, c[k], dst + (size_t)y * dstride, x0 + 32 * k);
}

cvtpm_status fail(cvtpm_status s, const std::string& m) {
    pm_set_free_error(m);
    return s;
}

bool finite_all(const float* v, int n) {
    for (int i = 0; i < n; ++i)
        if (!isfinite(v[i])) return false;
    return true;
}

}  // namespace

extern "C" {

cvtpm_status cvtpm_stereo_rectify(const cvtpm_camera* first, const cvtpm_camera* second, const float* extrinsics,
                                  int vertical, cvtpm_rectification* out, int width, int height, float* warp_first,
                                  float* warp_second, size_t warp_pitch, void* stream) {
    if (!first || !second || !extrinsics || !out) return fail(CVTPM_ERR_INVALID_ARGUMENT, "rectify: NULL argument");
    if (!finite_all(first->intrinsics, 9) || !finite_all(second->intrinsics, 9) || !finite_all(extrinsics, 16))
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "rectify: non-finite calibration");
    const bool maps = warp_first || warp_second;
    if (maps) {
        if (!warp_first || !warp_second) return fail(CVTPM_ERR_INVALID_ARGUMENT, "rectify: give both warp maps or neither");
        if (width < 1 || height < 1) return fail(CVTPM_ERR_SIZE, "rectify: empty warp maps");
        if (warp_pitch % 8 || warp_pitch < (size_t)width * 8)
            return fail(CVTPM_ERR_INVALID_ARGUMENT, "rectify: warp pitch not a multiple of 8 of at least width * 8");
    }
    /* StereoCameraCalibration::undistortRectify (:199-277) */
    M3 Rl, Rr;
    rect_matrices(extrinsics, &Rl, &Rr);
    const V3 t = m3_mul(Rr, translation(extrinsics));
    const V3 u = m3_mul(Rr, t);
    memset(out, 0, sizeof(*out));
    for (int i = 0; i < 4; ++i) out->extrinsics[i * 5] = 1.0f;
    out->extrinsics[3] = u.x;
    out->extrinsics[7] = u.y;
    out->extrinsics[11] = u.z;
    const float fleft = first->intrinsics[4], fright = second->intrinsics[4];
    const float fnew = fleft < fright ? fleft : fright;   /* Math::min */
    float clx = first->intrinsics[2], cly = first->intrinsics[5];
    float crx = second->intrinsics[2], cry = second->intrinsics[5];
    if (vertical) {
        clx = crx = (clx + crx) * 0.5f;
    } else {
        const float newy = (cly + cry) * 0.5f;
        cly = newy;
        cry = newy;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            out->rot_first[i * 3 + j] = Rl.m[i][j];
            out->rot_second[i * 3 + j] = Rr.m[i][j];
        }
    const float K0[9] = {fnew, 0.0f, clx, 0.0f, fnew, cly, 0.0f, 0.0f, 1.0f};
    const float K1[9] = {fnew, 0.0f, crx, 0.0f, fnew, cry, 0.0f, 0.0f, 1.0f};
    memcpy(out->first.intrinsics, K0, sizeof K0);
    memcpy(out->second.intrinsics, K1, sizeof K1);
    if (!maps) return CVTPM_OK;
    const RectOp ol = make_op(fnew, clx, cly, m3_transpose(Rl), *first);
    const RectOp orr = make_op(fnew, crx, cry, m3_transpose(Rr), *second);
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 grid((width + 31) / 32, (height + 7) / 8);
    k_rectify_map<<<grid, dim3(32, 8), 0, st>>>(ol, width, height, (float2*)warp_first, warp_pitch / 8);
    k_rectify_map<<<grid, dim3(32, 8), 0, st>>>(orr, width, height, (float2*)warp_second, warp_pitch / 8);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CVTPM_ERR_CUDA, std::string("rectify maps: ") + cudaGetErrorString(e));
    return CVTPM_OK;
}

cvtpm_status cvtpm_warp_apply(const cvtpm_image* dst, const cvtpm_image* src, const float* warp, size_t warp_pitch,
                              void* stream) {
    if (!dst || !src || !warp || !dst->data || !src->data) return fail(CVTPM_ERR_INVALID_ARGUMENT, "warp: NULL argument");
    int kind;
    size_t bpp, align;
    switch (src->format) {
        case CVTPM_IFORMAT_GRAY_FLOAT: kind = WARP_F1; bpp = 4; align = 4; break;
        case CVTPM_IFORMAT_RGBA_FLOAT:
        case CVTPM_IFORMAT_BGRA_FLOAT: kind = WARP_F4; bpp = 16; align = 4; break;
        case CVTPM_IFORMAT_GRAY_UINT8: kind = WARP_U8C1; bpp = 1; align = 1; break;
        case CVTPM_IFORMAT_RGBA_UINT8:
        case CVTPM_IFORMAT_BGRA_UINT8: kind = WARP_U8C4; bpp = 4; align = 4; break;
        default: return fail(CVTPM_ERR_NOT_SUPPORTED, "warp: unsupported image format");   /* IWarp.cpp:63 */
    }
    if (dst->format != src->format) return fail(CVTPM_ERR_INVALID_ARGUMENT, "warp: dst must have src's format");
    if (src->width < 1 || src->height < 1 || dst->width < 1 || dst->height < 1)
        return fail(CVTPM_ERR_SIZE, "warp: empty image");
    if (src->stride < (size_t)src->width * bpp || dst->stride < (size_t)dst->width * bpp || src->stride % align ||
        dst->stride % align || (uintptr_t)src->data % align || (uintptr_t)dst->data % align)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "warp: bad stride or alignment");
    if (warp_pitch % 8 || warp_pitch < (size_t)dst->width * 8 || (uintptr_t)warp % 8)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "warp: bad warp pitch or alignment");
    const dim3 grid((dst->width + 32 * WARP_PX - 1) / (32 * WARP_PX), (dst->height + 7) / 8);
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned char* s = (const unsigned char*)src->data;
    unsigned char* d = (unsigned char*)dst->data;
    const float2* m = (const float2*)warp;
    const size_t mp = warp_pitch / 8;
    switch (kind) {
        case WARP_F1: k_warp_apply<WARP_F1><<<grid, dim3(32, 8), 0, st>>>(s, src->stride, src->width, src->height, m, mp, dst->width, dst->height, d, dst->stride); break;
        case WARP_F4: k_warp_apply<WARP_F4><<<grid, dim3(32, 8), 0, st>>>(s, src->stride, src->width, src->height, m, mp, dst->width, dst->height, d, dst->stride); break;
        case WARP_U8C1: k_warp_apply<WARP_U8C1><<<grid, dim3(32, 8), 0, st>>>(s, src->stride, src->width, src->height, m, mp, dst->width, dst->height, d, dst->stride); break;
        default: k_warp_apply<WARP_U8C4><<<grid, dim3(32, 8), 0, st>>>(s, src->stride, src->width, src->height, m, mp, dst->width, dst->height, d, dst->stride); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CVTPM_ERR_CUDA, std::string("warp: ") + cudaGetErrorString(e));
    return CVTPM_OK;
}

}  // extern "C"
