/*
 * cvt/PMHuberStereo.hpp — header-only C++ facade over the C ABI (cvtpm.h)
 * that keeps the reference's call shape:
 *
 *   cvt::PMHuberStereo stereo;                              // PMHuberStereo.h:37
 *   stereo.depthMap(dmap, left, right, patchsize, depthmax,
 *                   iterations, viewsamples, dscale, &normalmap);   // :40
 *
 * cvt::Image here is a minimal device image: RGBA_FLOAT (4 floats per pixel)
 * or GRAY_FLOAT (1 float), rows padded to 16 bytes, memory from cudaMalloc
 * (the reference's IALLOCATOR_CL images, cvt/gfx/ImageAllocatorCL.cpp:40-54,
 * become device buffers).  depthMap reallocates dmap as GRAY_FLOAT and
 * normalmap as RGBA_FLOAT, as the reference does (PMHuberStereo.cpp:278,286),
 * and throws cvt::CVTException on inconsistent inputs (:66-68) or any other
 * failure.  Link with libcvtpm.so and the CUDA runtime.
 */
#ifndef CVT_GB300_PMHUBERSTEREO_HPP
#define CVT_GB300_PMHUBERSTEREO_HPP

#include <cuda_runtime_api.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>

#include "../cvtpm.h"

namespace cvt {

class CVTException : public std::runtime_error {
  public:
    explicit CVTException(const std::string& m) : std::runtime_error(m) {}
};

enum class IFormat { RGBA_FLOAT, GRAY_FLOAT };

class Image {
  public:
    Image() = default;
    Image(size_t w, size_t h, IFormat f = IFormat::RGBA_FLOAT) { reallocate(w, h, f); }
    Image(const Image&) = delete;
    Image& operator=(const Image&) = delete;
    Image(Image&& o) noexcept { swap(o); }
    Image& operator=(Image&& o) noexcept { swap(o); return *this; }
    ~Image() { release(); }

    void reallocate(size_t w, size_t h, IFormat f) {
        if (w == _w && h == _h && f == _f && _data) return;
        release();
        _w = w; _h = h; _f = f;
        size_t row = w * channels() * sizeof(float);
        _pitch = (row + 15) / 16 * 16;
        if (w && h && cudaMalloc(&_data, _pitch * h) != cudaSuccess) {
            _data = nullptr;
            throw CVTException("cvt::Image: device allocation failed");
        }
    }
    /* host <-> device copies of tightly packed rows */
    void upload(const float* host) {
        size_t row = _w * channels() * sizeof(float);
        if (cudaMemcpy2D(_data, _pitch, host, row, row, _h, cudaMemcpyHostToDevice) != cudaSuccess)
            throw CVTException("cvt::Image: upload failed");
    }
    void download(float* host) const {
        size_t row = _w * channels() * sizeof(float);
        if (cudaMemcpy2D(host, row, _data, _pitch, row, _h, cudaMemcpyDeviceToHost) != cudaSuccess)
            throw CVTException("cvt::Image: download failed");
    }
    size_t width() const { return _w; }
    size_t height() const { return _h; }
    size_t channels() const { return _f == IFormat::RGBA_FLOAT ? 4 : 1; }
    size_t pitch() const { return _pitch; }
    IFormat format() const { return _f; }
    float* data() { return static_cast<float*>(_data); }
    const float* data() const { return static_cast<const float*>(_data); }

  private:
    void release() { if (_data) cudaFree(_data); _data = nullptr; }
    void swap(Image& o) {
        std::swap(_w, o._w); std::swap(_h, o._h); std::swap(_f, o._f);
        std::swap(_pitch, o._pitch); std::swap(_data, o._data);
    }
    size_t _w = 0, _h = 0, _pitch = 0;
    IFormat _f = IFormat::RGBA_FLOAT;
    void* _data = nullptr;
};

class PMHuberStereo {
  public:
    explicit PMHuberStereo(int device = 0, int preset = CVTPM_PRESET_REFERENCE) {
        if (cvtpm_create(&_ctx, device) != CVTPM_OK) throw CVTException("PMHuberStereo: no CUDA device");
        cvtpm_params p;
        cvtpm_params_default(&p, preset);
        check(cvtpm_set_params(_ctx, &p));
    }
    ~PMHuberStereo() { if (_ctx) cvtpm_destroy(_ctx); }
    PMHuberStereo(const PMHuberStereo&) = delete;
    PMHuberStereo& operator=(const PMHuberStereo&) = delete;

    void setParams(const cvtpm_params& p) { check(cvtpm_set_params(_ctx, &p)); }
    cvtpm_params params() const { cvtpm_params p; cvtpm_get_params(_ctx, &p); return p; }

    /* PMHuberStereo::depthMap (cvt/vision/PMHuberStereo.h:40).  Runs on
     * `stream` (default stream if omitted) and synchronizes it. */
    void depthMap(Image& dmap, const Image& left, const Image& right, size_t patchsize, float depthmax,
                  size_t iterations, size_t viewsamples, float dscale = -1.0f, Image* normalmap = NULL,
                  cudaStream_t stream = 0) {
        if (left.width() != right.width() || left.height() != right.height() ||
            left.format() != IFormat::RGBA_FLOAT || right.format() != IFormat::RGBA_FLOAT ||
            left.pitch() != right.pitch())
            throw CVTException("Left/Right stereo images inconsistent or incompatible memory type");
        dmap.reallocate(left.width(), left.height(), IFormat::GRAY_FLOAT);
        if (normalmap) normalmap->reallocate(left.width(), left.height(), IFormat::RGBA_FLOAT);
        check(cvtpm_depthmap(_ctx, dmap.data(), dmap.pitch(), left.data(), right.data(), (int)left.width(),
                             (int)left.height(), left.pitch(), (int)patchsize, depthmax, (int)iterations,
                             (int)viewsamples, dscale, normalmap ? normalmap->data() : NULL,
                             normalmap ? normalmap->pitch() : 0, NULL, stream));
        check(cvtpm_synchronize(_ctx, stream));
    }

    /* PMHuberStereo::depthMapInpaint (PMHuberStereo.h:41): disparity in pixels. */
    void depthMapInpaint(Image& dmap, const Image& left, const Image& right, size_t patchsize, float depthmax,
                         size_t iterations, size_t viewsamples, cudaStream_t stream = 0) {
        if (left.width() != right.width() || left.height() != right.height() ||
            left.format() != IFormat::RGBA_FLOAT || right.format() != IFormat::RGBA_FLOAT ||
            left.pitch() != right.pitch())
            throw CVTException("Left/Right stereo images inconsistent or incompatible memory type");
        dmap.reallocate(left.width(), left.height(), IFormat::GRAY_FLOAT);
        check(cvtpm_depthmap_inpaint(_ctx, dmap.data(), dmap.pitch(), left.data(), right.data(), (int)left.width(),
                                     (int)left.height(), left.pitch(), (int)patchsize, depthmax, (int)iterations,
                                     (int)viewsamples, NULL, stream));
        check(cvtpm_synchronize(_ctx, stream));
    }

  private:
    void check(cvtpm_status s) {
        if (s != CVTPM_OK) throw CVTException(std::string(cvtpm_status_string(s)) + ": " + cvtpm_last_error(_ctx));
    }
    cvtpm_ctx* _ctx = nullptr;
};

}  // namespace cvt
#endif
