/* Drop-in check for C++ callers: reads two RGBA float32 images (raw, W*H*4),
 * runs cvt::PMHuberStereo::depthMap through include/cvt/PMHuberStereo.hpp and
 * writes the disparity map (raw, W*H floats).
 * usage: facade_main W H patchsize depthmax iterations left.raw right.raw out.raw
 *    or: facade_main --files patchsize depthmax iterations left right out.{pfm,png,raw}
 * The second form loads the pair with cvt::Image::load (CVTRaw, PNG or PPM
 * files in any format), runs depthMap and saves the disparity map by the
 * output's extension (PFM, PNG or CVTRaw). */
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cvt/PMHuberStereo.hpp"

static bool read_all(const char* path, std::vector<float>& v) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    size_t n = fread(v.data(), sizeof(float), v.size(), f);
    fclose(f);
    return n == v.size();
}

static int files(char** argv) {
    try {
        cvt::Image left, right, dmap;
        left.load(argv[5]);
        right.load(argv[6]);
        cvt::PMHuberStereo stereo;                         /* REFERENCE preset */
        stereo.depthMap(dmap, left, right, (size_t)atoi(argv[2]), (float)atof(argv[3]), (size_t)atoi(argv[4]), 4);
        dmap.save(argv[7]);
    } catch (const std::exception& e) {
        fprintf(stderr, "error: %s\n", e.what());
        return 4;
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 8 && std::string(argv[1]) == "--files") return files(argv);
    if (argc != 9) { fprintf(stderr, "usage\n"); return 2; }
    size_t W = (size_t)atoi(argv[1]), H = (size_t)atoi(argv[2]);
    size_t patch = (size_t)atoi(argv[3]);
    float dmax = (float)atof(argv[4]);
    size_t iters = (size_t)atoi(argv[5]);
    std::vector<float> l(W * H * 4), r(W * H * 4), d(W * H);
    if (!read_all(argv[6], l) || !read_all(argv[7], r)) { fprintf(stderr, "read failed\n"); return 3; }
    try {
        cvt::Image left(W, H), right(W, H), dmap;
        left.upload(l.data());
        right.upload(r.data());
        cvt::PMHuberStereo stereo;                         /* REFERENCE preset */
        stereo.depthMap(dmap, left, right, patch, dmax, iters, 4);
        dmap.download(d.data());
        try {
            cvt::Image other(W + 1, H);
            stereo.depthMap(dmap, left, other, patch, dmax, iters, 4);
            fprintf(stderr, "expected CVTException\n");
            return 5;
        } catch (const cvt::CVTException&) {
        }
    } catch (const std::exception& e) {
        fprintf(stderr, "error: %s\n", e.what());
        return 4;
    }
    FILE* f = fopen(argv[8], "wb");
    if (!f) return 6;
    fwrite(d.data(), sizeof(float), d.size(), f);
    fclose(f);
    return 0;
}
