/*
 * cvt/PMHuberStereo.hpp — header-only C++ facade over the C ABI (cvtpm.h)
 * that keeps the reference's call shape:
 *
 *   cvt::PMHuberStereo stereo;                              // PMHuberStereo.h:37
 *   stereo.depthMap(dmap, left, right, patchsize, depthmax,
 *                   iterations, viewsamples, dscale, &normalmap);   // :40
 *
 * cvt::Image here is a minimal device image in any cvt::IFormat, rows padded
 * to 16 bytes, memory from cudaMalloc (the reference's IALLOCATOR_CL images,
 * cvt/gfx/ImageAllocatorCL.cpp:40-54, become device buffers).  depthMap reads
 * left and right as the reference's kernels read them (read_imagef).  depthMap reallocates dmap as GRAY_FLOAT and
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
#include <vector>

#include "../cvtpm.h"

namespace cvt {

class CVTException : public std::runtime_error {
  public:
    explicit CVTException(const std::string& m) : std::runtime_error(m) {}
};

/* cvt::IFormatID (cvt/gfx/IFormat.h:36-63), same values. */
enum class IFormat : int {
    GRAY_UINT8 = CVTPM_IFORMAT_GRAY_UINT8, GRAY_UINT16, GRAY_INT16, GRAY_FLOAT,
    GRAYALPHA_UINT8, GRAYALPHA_UINT16, GRAYALPHA_INT16, GRAYALPHA_FLOAT,
    RGBA_UINT8, RGBA_UINT16, RGBA_INT16, RGBA_FLOAT,
    BGRA_UINT8, BGRA_UINT16, BGRA_INT16, BGRA_FLOAT,
    BAYER_RGGB_UINT8, BAYER_GRBG_UINT8, BAYER_GBRG_UINT8,
    YUYV_UINT8, UYVY_UINT8
};

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
        const size_t bpp = cvtpm_iformat_bpp((int)f);
        if (!bpp) throw CVTException("cvt::Image: unknown format");
        release();
        _w = w; _h = h; _f = f;
        _pitch = (w * bpp + 15) / 16 * 16;
        if (w && h && cudaMalloc(&_data, _pitch * h) != cudaSuccess) {
            _data = nullptr;
            throw CVTException("cvt::Image: device allocation failed");
        }
    }
    /* host <-> device copies of tightly packed rows (width * bpp() bytes) */
    void upload(const void* host) {
        if (cudaMemcpy2D(_data, _pitch, host, row(), row(), _h, cudaMemcpyHostToDevice) != cudaSuccess)
            throw CVTException("cvt::Image: upload failed");
    }
    void download(void* host) const {
        if (cudaMemcpy2D(host, row(), _data, _pitch, row(), _h, cudaMemcpyDeviceToHost) != cudaSuccess)
            throw CVTException("cvt::Image: download failed");
    }
    /* Image::load / Image::save by file extension (the reference picks its
     * loader / saver plugin the same way): .raw is CVTRaw, .png is PNG, .ppm
     * and .pgm are read as RGBA_UINT8 / GRAY_UINT8, .pfm is written from
     * float formats. */
    void load(const std::string& path) {
        cvtpm_image d{};
        const bool raw = ends_with(path, ".raw"), png = ends_with(path, ".png") || ends_with(path, ".PNG");
        if (!raw && !png && !ends_with(path, ".ppm") && !ends_with(path, ".pgm") && !ends_with(path, ".PPM") &&
            !ends_with(path, ".PGM"))
            throw CVTException("cvt::Image::load: no loader for " + path);
        auto rd = raw ? cvtpm_raw_read : (png ? cvtpm_png_read : cvtpm_ppm_read);
        if (rd(path.c_str(), &d) != CVTPM_OK) throw CVTException(cvtpm_last_error(NULL));
        std::vector<unsigned char> host(d.stride * (size_t)d.height);
        d.data = host.data();
        if (rd(path.c_str(), &d) != CVTPM_OK) throw CVTException(cvtpm_last_error(NULL));
        reallocate((size_t)d.width, (size_t)d.height, (IFormat)d.format);
        upload(host.data());
    }
    void save(const std::string& path) const {
        std::vector<unsigned char> host(row() * _h);
        download(host.data());
        cvtpm_image d{(int)_f, (int)_w, (int)_h, row(), host.data()};
        cvtpm_status s;
        if (ends_with(path, ".raw")) s = cvtpm_raw_write(path.c_str(), &d);
        else if (ends_with(path, ".pfm")) s = cvtpm_pfm_write(path.c_str(), &d);
        else if (ends_with(path, ".png") || ends_with(path, ".PNG")) s = cvtpm_png_write(path.c_str(), &d);
        else throw CVTException("cvt::Image::save: no saver for " + path);
        if (s != CVTPM_OK) throw CVTException(cvtpm_last_error(NULL));
    }
    size_t width() const { return _w; }
    size_t height() const { return _h; }
    size_t bpp() const { return cvtpm_iformat_bpp((int)_f); }
    size_t channels() const {
        switch (_f) {
            case IFormat::RGBA_UINT8: case IFormat::RGBA_UINT16: case IFormat::RGBA_INT16: case IFormat::RGBA_FLOAT:
            case IFormat::BGRA_UINT8: case IFormat::BGRA_UINT16: case IFormat::BGRA_INT16: case IFormat::BGRA_FLOAT:
                return 4;
            case IFormat::GRAYALPHA_UINT8: case IFormat::GRAYALPHA_UINT16: case IFormat::GRAYALPHA_INT16:
            case IFormat::GRAYALPHA_FLOAT: case IFormat::YUYV_UINT8: case IFormat::UYVY_UINT8:
                return 2;
            default:
                return 1;
        }
    }
    size_t pitch() const { return _pitch; }
    IFormat format() const { return _f; }
    void* ptr() { return _data; }
    const void* ptr() const { return _data; }
    float* data() { return static_cast<float*>(_data); }
    const float* data() const { return static_cast<const float*>(_data); }
    cvtpm_image desc() const { return cvtpm_image{(int)_f, (int)_w, (int)_h, _pitch, _data}; }

  private:
    size_t row() const { return _w * bpp(); }
    static bool ends_with(const std::string& s, const char* e) {
        const std::string x(e);
        return s.size() >= x.size() && s.compare(s.size() - x.size(), x.size(), x) == 0;
    }
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
        if (left.width() != right.width() || left.height() != right.height())
            throw CVTException("Left/Right stereo images inconsistent or incompatible memory type");
        dmap.reallocate(left.width(), left.height(), IFormat::GRAY_FLOAT);
        if (normalmap) normalmap->reallocate(left.width(), left.height(), IFormat::RGBA_FLOAT);
        if (left.format() == IFormat::RGBA_FLOAT && right.format() == IFormat::RGBA_FLOAT &&
            left.pitch() == right.pitch()) {
            check(cvtpm_depthmap(_ctx, dmap.data(), dmap.pitch(), left.data(), right.data(), (int)left.width(),
                                 (int)left.height(), left.pitch(), (int)patchsize, depthmax, (int)iterations,
                                 (int)viewsamples, dscale, normalmap ? normalmap->data() : NULL,
                                 normalmap ? normalmap->pitch() : 0, NULL, stream));
        } else {   /* any other formats: read as the reference's read_imagef reads them */
            const cvtpm_image l = left.desc(), r = right.desc();
            check(cvtpm_depthmap_image(_ctx, dmap.data(), dmap.pitch(), &l, &r, (int)patchsize, depthmax,
                                       (int)iterations, (int)viewsamples, dscale,
                                       normalmap ? normalmap->data() : NULL, normalmap ? normalmap->pitch() : 0,
                                       NULL, stream));
        }
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
