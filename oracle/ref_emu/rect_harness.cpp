/*
 * TEST INFRASTRUCTURE — C entry points into the reference's own stereo
 * rectification and resampling code, compiled from its sources where they
 * lie (recipe: build_ref.py, build_rect):
 *
 *   cvt/vision/StereoCameraCalibration.h   StereoCameraCalibration(first,
 *       second, extrinsics), rectificationMatrices, undistortRectify and its
 *       UndistortRectifyWarp functor, with cvt/math (Matrix3, Matrix4,
 *       Quaternion, Vector2/3/4) underneath
 *   cvt/util/SIMD.cpp                      SIMD::warpBilinear1f / 4f / 1u8 /
 *       4u8, called row by row as IWarp::applyFC1 / FC4 / U8C1 / U8C4 do
 *       (cvt/gfx/ifilter/IWarp.cpp:254-376; IWarp.cpp itself pulls in the
 *       plugin system, so its four row loops are repeated here)
 *
 * Stubs in rect_shim/: empty Eigen/Core and Eigen/LU (cvt/math/Math.h
 * includes them and uses nothing), a host-memory Image for the warp maps and
 * IWarp::warpGeneric's per-pixel loop.  rect_stubs.cpp supplies the two XML
 * parsers that CameraCalibration's deserialize references (their source,
 * cvt/math/Matrix.cpp, needs Eigen's SVD).
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <list>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

/* UndistortRectifyWarp is a private member type; the harness constructs
 * nothing through it, it only runs undistortRectify, which uses it. */
#define private public
#include <cvt/vision/StereoCameraCalibration.h>
#undef private
#include <cvt/util/SIMD.h>

#define EXPORT extern "C" __attribute__((visibility("default")))

using namespace cvt;

namespace {
struct GenericSIMD : SIMD {
    GenericSIMD() {}
};

CameraCalibration camera(const float* K, const float* rad, const float* tan) {
    CameraCalibration c;
    c.setIntrinsics(Matrix3f(K[0], K[1], K[2], K[3], K[4], K[5], K[6], K[7], K[8]));
    c.setDistortion(Vector3f(rad[0], rad[1], rad[2]), Vector2f(tan[0], tan[1]));
    return c;
}

void put3(const Matrix3f& m, float* o) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o[i * 3 + j] = m[i][j];
}
}  // namespace

/* StereoCameraCalibration(first, second, extrinsics).undistortRectify on
 * W x H maps; the rectified calibration and rectificationMatrices' result. */
EXPORT int ref_rectify(const float* K0, const float* rad0, const float* tan0, const float* K1, const float* rad1,
                       const float* tan1, const float* E, int vertical, int W, int H, float* map0, float* map1,
                       float* K0new, float* K1new, float* Enew, float* Rl, float* Rr) {
    try {
        Matrix4f ext(E[0], E[1], E[2], E[3], E[4], E[5], E[6], E[7], E[8], E[9], E[10], E[11], E[12], E[13], E[14],
                     E[15]);
        StereoCameraCalibration sc(camera(K0, rad0, tan0), camera(K1, rad1, tan1), ext);
        StereoCameraCalibration out;
        Image wl((size_t)W, (size_t)H), wr((size_t)W, (size_t)H);
        sc.undistortRectify(out, wl, wr, (size_t)W, (size_t)H, vertical != 0);
        memcpy(map0, wl.data(), sizeof(float) * 2 * W * H);
        memcpy(map1, wr.data(), sizeof(float) * 2 * W * H);
        put3(out.firstCamera().intrinsics(), K0new);
        put3(out.secondCamera().intrinsics(), K1new);
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) Enew[i * 4 + j] = out.extrinsics()[i][j];
        Matrix3f a, b;
        sc.rectificationMatrices(a, b);
        put3(a, Rl);
        put3(b, Rr);
    } catch (const std::exception& e) {
        fprintf(stderr, "ref_rectify: %s\n", e.what());
        return 1;
    }
    return 0;
}

/* IWarp::apply's row loops (IWarp.cpp:254-376): kind 0 GRAY_FLOAT (fill 0),
 * 1 RGBA/BGRA_FLOAT (fill 0,0,0,1), 2 GRAY_UINT8 (fill 0), 3 RGBA/BGRA_UINT8
 * (fill 0xff000000).  The map has W x H (x, y) pairs, rows of mstride bytes. */
EXPORT int ref_warp(int kind, const void* src, size_t sstride, int sw, int sh, const float* map, size_t mstride,
                    int W, int H, void* dst, size_t dstride) {
    GenericSIMD simd;
    const float black[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    for (int y = 0; y < H; ++y) {
        const float* m = (const float*)((const uint8_t*)map + (size_t)y * mstride);
        uint8_t* d = (uint8_t*)dst + (size_t)y * dstride;
        switch (kind) {
            case 0: simd.warpBilinear1f((float*)d, m, (const float*)src, sstride, sw, sh, 0.0f, W); break;
            case 1: simd.warpBilinear4f((float*)d, m, (const float*)src, sstride, sw, sh, black, W); break;
            case 2: simd.warpBilinear1u8(d, m, (const uint8_t*)src, sstride, sw, sh, 0, W); break;
            case 3: simd.warpBilinear4u8(d, m, (const uint8_t*)src, sstride, sw, sh, 0xff000000u, W); break;
            default: return 1;
        }
    }
    return 0;
}

/* The float-to-8-bit conversions Image::convert applies before the PNG
 * saver writes a float image (cvt/gfx/IConvert.cpp: GRAY_FLOAT ->
 * Conv_GRAYf_to_GRAYu8, GRAYALPHA_FLOAT -> Conv_f_to_u8, RGBA/BGRA_FLOAT ->
 * Conv_XXXAf_to_XXXAu8): kind 0, 1, 2; n floats (kind 2: n / 4 pixels). */
EXPORT int ref_conv_f_u8(int kind, const float* src, uint8_t* dst, size_t n) {
    GenericSIMD simd;
    switch (kind) {
        case 0: simd.Conv_GRAYf_to_GRAYu8(dst, src, n); break;
        case 1: simd.Conv_f_to_u8(dst, src, n); break;
        case 2: simd.Conv_XXXAf_to_XXXAu8(dst, src, n / 4); break;
        default: return 1;
    }
    return 0;
}

/* cvt::Matrix4f operator* (cvt/math/Matrix4.h:269-288), row-major in and out;
 * the product TSDFVolume::addDepthMap forms (proj * grid-to-world). */
EXPORT int ref_mat4_mul(const float* a, const float* b, float* out) {
    Matrix4f A(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15]);
    Matrix4f B(b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8], b[9], b[10], b[11], b[12], b[13], b[14], b[15]);
    const Matrix4f C = A * B;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) out[i * 4 + j] = C[i][j];
    return 0;
}
