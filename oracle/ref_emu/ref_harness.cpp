/*
 * ref_harness.cpp — TEST INFRASTRUCTURE.  C entry points around the
 * reference's own code compiled for the OpenCL-C emulation:
 * cvt::PMHuberStereo::depthMap (cvt/vision/PMHuberStereo.cpp:64-291) and
 * depthMapInpaint (:293-506), cvt::PDROF::apply (cvt/gfx/PDROF.h:50-96),
 * cvt::PDROFInpaint::apply (cvt/gfx/PDROFInpaint.h:50-98) and single kernels of
 * cvt/cl/kernel/pmhstereo.cl.  It produces the golden fixtures under
 * tests/golden/ (tests/golden/make_golden.py) and never ships.
 */
#include <cstring>
#include <string>
#include <vector>

#include <cvt/vision/PMHuberStereo.h>
#include "clemu_api.h"

using cvt::Image;
using cvt::IFormat;
using cvt::IALLOCATOR_CL;

namespace {

Image rgba(const float* src, int W, int H) {
    Image im((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL);
    memcpy(im.data(), src, sizeof(float) * 4 * (size_t)W * H);
    return im;
}

size_t pad16(size_t v) { return cvt::Math::pad(v, 16); }

void launch2d(const char* name, const std::vector<clemu::Arg>& args, int W, int H) {
    clemu::launch(name, args, pad16(W), pad16(H), 16, 16);
}

clemu::Arg img_arg(Image& im) { clemu::Arg a; a.kind = clemu::Arg::IMAGE; a.img = im.cl(); return a; }
clemu::Arg int_arg(int v) { clemu::Arg a; a.kind = clemu::Arg::INT; a.i = v; return a; }
clemu::Arg float_arg(float v) { clemu::Arg a; a.kind = clemu::Arg::FLOAT; a.f = v; return a; }

}  // namespace

extern "C" {

/* PMHuberStereo::depthMap.  states (optional, 2*W*H*4): the outputs of the
 * last left and right pmhstereo_propagate_view launches. */
int ref_depthmap(const float* left, const float* right, int W, int H, int patchsize, float depthmax,
                 int iterations, float dscale, float* dmap, float* normalmap, float* states) {
    Image L = rgba(left, W, H), R = rgba(right, W, H);
    std::vector<float> last[2];
    clemu::on_launch = [&](const std::string& name, const std::vector<clemu::Arg>& args) {
        if (name == "pmhstereo_propagate_view") {
            const clemu::Img* out = args[0].img;
            int lr = args[10].i;
            last[lr ? 0 : 1].assign(out->data, out->data + (size_t)out->w * out->h * 4);
        }
    };
    Image dm, nm;
    try {
        cvt::PMHuberStereo st;
        st.depthMap(dm, L, R, (size_t)patchsize, depthmax, (size_t)iterations, 4, dscale, normalmap ? &nm : NULL);
    } catch (...) {
        clemu::on_launch = nullptr;
        return 1;
    }
    clemu::on_launch = nullptr;
    memcpy(dmap, dm.data(), sizeof(float) * (size_t)W * H);
    if (normalmap) memcpy(normalmap, nm.data(), sizeof(float) * 4 * (size_t)W * H);
    if (states) {
        size_t n = (size_t)W * H * 4;
        if (last[0].size() != n || last[1].size() != n) return 2;
        memcpy(states, last[0].data(), n * sizeof(float));
        memcpy(states + n, last[1].data(), n * sizeof(float));
    }
    return 0;
}

/* pmhstereo_gradxy / pmhstereo_weight on one RGBA image. */
int ref_gradxy(const float* img, int W, int H, float* out) {
    Image src = rgba(img, W, H), dst((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL);
    launch2d("pmhstereo_gradxy", {img_arg(dst), img_arg(src)}, W, H);
    memcpy(out, dst.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}
int ref_weight(const float* img, int W, int H, float* out) {
    Image src = rgba(img, W, H), dst((size_t)W, (size_t)H, IFormat::GRAY_FLOAT, IALLOCATOR_CL);
    launch2d("pmhstereo_weight", {img_arg(dst), img_arg(src)}, W, H);
    memcpy(out, dst.data(), sizeof(float) * (size_t)W * H);
    return 0;
}

/* patch_eval_color_grad_weighted for a fixed state field. */
int ref_cost_field(const float* img1, const float* img2, int W, int H, const float* states, int patchsize,
                   float* cost) {
    Image c1 = rgba(img1, W, H), c2 = rgba(img2, W, H);
    Image g1((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL), g2 = g1;
    launch2d("pmhstereo_gradxy", {img_arg(g1), img_arg(c1)}, W, H);
    launch2d("pmhstereo_gradxy", {img_arg(g2), img_arg(c2)}, W, H);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            cost[(size_t)y * W + x] = clemu::pmh_patch_eval(c1.cl(), g1.cl(), c2.cl(), g2.cl(), (float)x, (float)y,
                                                            states + ((size_t)y * W + x) * 4, patchsize, 1);
    return 0;
}

/* pmhstereo_init for view lr (img1 is that view). */
int ref_init(const float* img1, const float* img2, int W, int H, int patchsize, float depthmax, int lr, float* out) {
    Image c1 = rgba(img1, W, H), c2 = rgba(img2, W, H);
    Image g1((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL), g2 = g1, o = g1;
    launch2d("pmhstereo_gradxy", {img_arg(g1), img_arg(c1)}, W, H);
    launch2d("pmhstereo_gradxy", {img_arg(g2), img_arg(c2)}, W, H);
    launch2d("pmhstereo_init", {img_arg(o), img_arg(c1), img_arg(c2), img_arg(g1), img_arg(g2), int_arg(patchsize),
                                float_arg(depthmax), int_arg(lr)}, W, H);
    memcpy(out, o.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}

/* cvt::PDROF::apply: `output` is read as the warm start and overwritten. */
int ref_pdrof(float* output, const float* input, const float* weight, int W, int H, float lambda, int iters) {
    Image out = rgba(output, W, H), in = rgba(input, W, H);
    Image w((size_t)W, (size_t)H, IFormat::GRAY_FLOAT, IALLOCATOR_CL);
    memcpy(w.data(), weight, sizeof(float) * (size_t)W * H);
    cvt::PDROF pd;
    pd.apply(out, in, w, lambda, iters);
    memcpy(output, out.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}

/* One pmhstereo_propagate_view launch.  viewin: W*H records of
 * {int n; float4 value[4]} (80 bytes each, the reference's VIEWPROP_t) or NULL
 * for none; viewout receives the scatter (same layout) when not NULL. */
int ref_propagate(const float* img1, const float* img2, int W, int H, const float* old, const float* smooth,
                  float theta, int patchsize, float depthmax, int lr, int iter, const void* viewin, void* viewout,
                  float* out) {
    Image c1 = rgba(img1, W, H), c2 = rgba(img2, W, H), o = rgba(old, W, H), sm = rgba(smooth, W, H);
    Image g1((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL), g2 = g1, res = g1;
    launch2d("pmhstereo_gradxy", {img_arg(g1), img_arg(c1)}, W, H);
    launch2d("pmhstereo_gradxy", {img_arg(g2), img_arg(c2)}, W, H);
    cvt::CLBuffer vin(80 * (size_t)W * H), vout(80 * (size_t)W * H);
    if (viewin) memcpy(vin.ptr(), viewin, 80 * (size_t)W * H);
    clemu::Arg bi, bo;
    bi.kind = bo.kind = clemu::Arg::BUFFER;
    bi.ptr = vin.ptr(); bo.ptr = vout.ptr();
    launch2d("pmhstereo_propagate_view", {img_arg(res), img_arg(o), img_arg(c1), img_arg(c2), img_arg(g1), img_arg(g2),
                                          img_arg(sm), float_arg(theta), int_arg(patchsize), float_arg(depthmax),
                                          int_arg(lr), int_arg(iter), bi, bo}, W, H);
    memcpy(out, res.data(), sizeof(float) * 4 * (size_t)W * H);
    if (viewout) memcpy(viewout, vout.ptr(), 80 * (size_t)W * H);
    return 0;
}

/* PMHuberStereo::depthMapInpaint (PMHuberStereo.cpp:293-506).  states
 * (optional, 2*W*H*4): the outputs of the last left and right
 * pmhstereo_propagate_view launches. */
int ref_depthmap_inpaint(const float* left, const float* right, int W, int H, int patchsize, float depthmax,
                         int iterations, float* dmap, float* states) {
    Image L = rgba(left, W, H), R = rgba(right, W, H);
    std::vector<float> last[2];
    clemu::on_launch = [&](const std::string& name, const std::vector<clemu::Arg>& args) {
        if (name == "pmhstereo_propagate_view") {
            const clemu::Img* out = args[0].img;
            int lr = args[10].i;
            last[lr ? 0 : 1].assign(out->data, out->data + (size_t)out->w * out->h * 4);
        }
    };
    Image dm;
    try {
        cvt::PMHuberStereo st;
        st.depthMapInpaint(dm, L, R, (size_t)patchsize, depthmax, (size_t)iterations, 4);
    } catch (...) {
        clemu::on_launch = nullptr;
        return 1;
    }
    clemu::on_launch = nullptr;
    memcpy(dmap, dm.data(), sizeof(float) * (size_t)W * H);
    if (states) {
        size_t n = (size_t)W * H * 4;
        if (last[0].size() != n || last[1].size() != n) return 2;
        memcpy(states, last[0].data(), n * sizeof(float));
        memcpy(states + n, last[1].data(), n * sizeof(float));
    }
    return 0;
}

/* pmhstereo_occmap (pmhstereo.cl:682-712) of state images a (view lr) and b. */
int ref_occmap(const float* a, const float* b, int W, int H, float maxdiff, int lr, float* out) {
    Image ia = rgba(a, W, H), ib = rgba(b, W, H), o((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL);
    launch2d("pmhstereo_occmap", {img_arg(o), img_arg(ia), img_arg(ib), float_arg(maxdiff), int_arg(lr)}, W, H);
    memcpy(out, o.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}

/* pmhstereo_normal_depth (pmhstereo.cl:663-680). */
int ref_normal_depth(const float* states, int W, int H, float depthmax, int lr, float* out) {
    Image in = rgba(states, W, H), o((size_t)W, (size_t)H, IFormat::RGBA_FLOAT, IALLOCATOR_CL);
    launch2d("pmhstereo_normal_depth", {img_arg(o), img_arg(in), float_arg(depthmax), int_arg(lr)}, W, H);
    memcpy(out, o.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}

/* cvt::PDROFInpaint::apply (PDROFInpaint.h:50-98); mask RGBA (x used). */
int ref_pdrof_inpaint(float* output, const float* input, const float* weight, const float* mask, int W, int H,
                      float lambda, int iters) {
    Image out = rgba(output, W, H), in = rgba(input, W, H), m = rgba(mask, W, H);
    Image w((size_t)W, (size_t)H, IFormat::GRAY_FLOAT, IALLOCATOR_CL);
    memcpy(w.data(), weight, sizeof(float) * (size_t)W * H);
    cvt::PDROFInpaint pd;
    pd.apply(out, in, w, m, lambda, iters);
    memcpy(output, out.data(), sizeof(float) * 4 * (size_t)W * H);
    return 0;
}

/* TSDFVolume (cvt/vision/TSDFVolume.cpp:47-104, kernels
 * cvt/cl/kernel/TSDFVolume/TSDFVolume.cl).  The volume is W*H*D float2
 * (tsdf, weight); matrices row-major 4x4 as the kernels' Mat4f; NDRanges as
 * the host code sets them (pad16 in x and y, 16 x 16 groups). */
static clemu::Arg buf_arg(void* p) { clemu::Arg a; a.kind = clemu::Arg::BUFFER; a.ptr = p; return a; }
static clemu::Arg mat_arg(const float* m) {
    clemu::Arg a;
    a.kind = clemu::Arg::BYTES;
    a.bytes.assign((const unsigned char*)m, (const unsigned char*)m + 16 * sizeof(float));
    return a;
}

int ref_tsdf_clear(float* vol, int W, int H, int D, float weight) {
    clemu::launch3("TSDFVolume_clear", {buf_arg(vol), int_arg(W), int_arg(H), int_arg(D), float_arg(weight)}, pad16(W),
                   pad16(H), (size_t)D, 16, 16);
    return 0;
}

/* TSDFVolume::addDepthMap(proj, depthmap, scale) with TG2CAM = proj * g2w;
 * the depth map is a GRAY_FLOAT image (read .x). */
int ref_tsdf_add(float* vol, int W, int H, int D, const float* dmap, int iw, int ih, float dscale, const float* tg2cam,
                 float trunc) {
    Image dm((size_t)iw, (size_t)ih, IFormat::GRAY_FLOAT, IALLOCATOR_CL);
    memcpy(dm.data(), dmap, sizeof(float) * (size_t)iw * ih);
    clemu::launch3("TSDFVolume_add", {buf_arg(vol), int_arg(W), int_arg(H), int_arg(D), img_arg(dm), float_arg(dscale),
                                      mat_arg(tg2cam), float_arg(trunc)}, pad16(W), pad16(H), (size_t)D, 16, 16);
    return 0;
}

/* TSDFVolume::rayCastDepthMap(depthmap, proj, scale): TCAM2G = (proj * g2w)^-1. */
int ref_tsdf_raycast(float* out, int iw, int ih, float* vol, int W, int H, int D, const float* tcam2g,
                     const float* tg2cam, float scale) {
    Image o((size_t)iw, (size_t)ih, IFormat::GRAY_FLOAT, IALLOCATOR_CL);
    clemu::launch("TSDFVolume_rayCastDepthmap", {img_arg(o), buf_arg(vol), int_arg(W), int_arg(H), int_arg(D),
                                                 mat_arg(tcam2g), mat_arg(tg2cam), float_arg(scale)},
                  pad16(iw), pad16(ih), 16, 16);
    memcpy(out, o.data(), sizeof(float) * (size_t)iw * ih);
    return 0;
}

/* TSDFVolume_sliceX/Y/Z (TSDFVolume.cl) at plane v into an RGBA image of
 * the slice's size (the NDRange as large as the image). */
int ref_tsdf_slice(float* rgba, int axis, int v, float* vol, int W, int H, int D) {
    const int ow = axis == 0 ? H : W, oh = axis == 2 ? H : D;
    Image o((size_t)ow, (size_t)oh, IFormat::RGBA_FLOAT, IALLOCATOR_CL);
    const char* k = axis == 0 ? "TSDFVolume_sliceX" : (axis == 1 ? "TSDFVolume_sliceY" : "TSDFVolume_sliceZ");
    clemu::launch(k, {img_arg(o), int_arg(v), buf_arg(vol), int_arg(W), int_arg(H), int_arg(D)}, pad16(ow), pad16(oh),
                  16, 16);
    memcpy(rgba, o.data(), sizeof(float) * 4 * (size_t)ow * oh);
    return 0;
}

}  // extern "C"
