/*
 * TEST INFRASTRUCTURE — stand-in for cvt/gfx/Image.h so that the reference's
 * cvt/vision/PMHuberStereo.cpp and cvt/gfx/PDROF.h compile against the
 * OpenCL-C emulation.  An Image is a host float buffer: RGBA_FLOAT (4 floats
 * per pixel, CL_RGBA) or GRAY_FLOAT (1 float, CL_INTENSITY), as
 * cvt/gfx/IFormat.h:293-312 maps them.  save() writes nothing.
 */
#ifndef CVT_SHIM_IMAGE_H
#define CVT_SHIM_IMAGE_H

#include <cstddef>
#include <cstring>
#include <vector>

#include "clemu_api.h"

namespace cvt {

enum IAllocatorType { IALLOCATOR_MEM = 0, IALLOCATOR_GL, IALLOCATOR_CL };

struct IFormat {
    int channels;
    int id;
    static const IFormat RGBA_FLOAT;
    static const IFormat GRAY_FLOAT;
    bool operator==(const IFormat& o) const { return id == o.id; }
    bool operator!=(const IFormat& o) const { return id != o.id; }
};
inline const IFormat IFormat::RGBA_FLOAT = {4, 1};
inline const IFormat IFormat::GRAY_FLOAT = {1, 2};

class Image {
  public:
    Image() : _fmt(IFormat::RGBA_FLOAT), _mem(IALLOCATOR_CL) { sync(0, 0); }
    Image(size_t w, size_t h, const IFormat& f = IFormat::RGBA_FLOAT, IAllocatorType t = IALLOCATOR_MEM)
        : _fmt(f), _mem(t) { sync(w, h); }
    Image(const Image& o, IAllocatorType t = IALLOCATOR_MEM) : _fmt(o._fmt), _mem(t), _buf(o._buf) { sync(o._img.w, o._img.h); }
    Image& operator=(const Image& o) { _fmt = o._fmt; _buf = o._buf; sync(o._img.w, o._img.h); return *this; }

    size_t width() const { return (size_t)_img.w; }
    size_t height() const { return (size_t)_img.h; }
    IAllocatorType memType() const { return _mem; }
    size_t channels() const { return (size_t)_fmt.channels; }
    const IFormat& format() const { return _fmt; }
    void reallocate(size_t w, size_t h, const IFormat& f, IAllocatorType t) {
        if ((size_t)_img.w == w && (size_t)_img.h == h && f == _fmt && t == _mem) return;
        _fmt = f; _mem = t; _buf.clear(); sync(w, h);
    }
    void save(const char*) const {}
    clemu::Img* cl() const { return const_cast<clemu::Img*>(&_img); }
    float* data() { return _buf.data(); }
    const float* data() const { return _buf.data(); }

  private:
    void sync(size_t w, size_t h) {
        _buf.resize(w * h * (size_t)_fmt.channels, 0.0f);
        _img.w = (int)w; _img.h = (int)h; _img.channels = _fmt.channels; _img.data = _buf.data();
    }
    IFormat _fmt;
    IAllocatorType _mem;
    std::vector<float> _buf;
    clemu::Img _img;
};

/* cvt/math/Math.h:79-103 (that header needs Eigen, absent here): clamp,
 * smoothstep and pad, the helpers PMHuberStereo.cpp and PDROF.h call. */
namespace Math {
template <typename T> static inline T clamp(T v, T min, T max) { return (v < min) ? min : (v > max) ? max : v; }
template <typename T> static inline T smoothstep(T x) {
    T t = clamp<T>(x, 0, 1);
    return t * t * (((T)3) - ((T)2) * t);
}
static inline size_t pad(size_t v, size_t multiple) {
    size_t r = v % multiple;
    if (!r) return v;
    return v + multiple - r;
}
}  // namespace Math

}  // namespace cvt
#endif
