/* TEST INFRASTRUCTURE — the part of cvt::Image that the rectification
 * harness needs: a GRAYALPHA_FLOAT warp map held in host memory.  Replaces
 * cvt/gfx/Image.h (which pulls in OpenGL and OpenCL) when the reference's
 * StereoCameraCalibration.h is compiled for the oracle. */
#ifndef CVT_IMAGE_H
#define CVT_IMAGE_H
#include <cstddef>
#include <vector>
namespace cvt {
class Image {
  public:
    Image(size_t w = 0, size_t h = 0) : _w(w), _h(h), _buf(2 * w * h) {}
    size_t width() const { return _w; }
    size_t height() const { return _h; }
    float* line(size_t y) { return _buf.data() + 2 * _w * y; }
    const float* data() const { return _buf.data(); }
  private:
    size_t _w, _h;
    std::vector<float> _buf;
};
}
#endif
