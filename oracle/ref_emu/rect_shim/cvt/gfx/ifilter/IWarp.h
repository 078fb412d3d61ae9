/* TEST INFRASTRUCTURE — IWarp::warpGeneric for the rectification harness:
 * the per-pixel loop of cvt/gfx/ifilter/IWarp.h:80-99 (op evaluated at
 * Vector2f(x, y), x and y the integer pixel position, result stored as the
 * pixel's (x, y) pair) over the shim Image.  The reference's IWarp.h pulls in
 * the plugin system (a generated header). */
#ifndef CVT_IWARP_H
#define CVT_IWARP_H
#include <cvt/gfx/Image.h>
#include <cvt/math/Vector.h>
namespace cvt {
struct IWarp {
    template <typename TFUNC>
    static void warpGeneric(Image& idst, TFUNC op) {
        for (size_t y = 0; y < idst.height(); y++) {
            float* dst = idst.line(y);
            for (size_t x = 0; x < idst.width(); x++) {
                Vector2f p = op(Vector2f(x, y));
                *dst++ = p.x;
                *dst++ = p.y;
            }
        }
    }
};
}
#endif
