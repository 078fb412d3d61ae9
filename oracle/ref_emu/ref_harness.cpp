/*
 * ref_harness.cpp — TEST INFRASTRUCTURE.  C entry points around the
 * reference's own code compiled for the OpenCL-C emulation:
 * cvt::PMHuberStereo::depthMap (cvt/vision/PMHuberStereo.cpp:64-291) and
 * depthMapInpaint (:293-506), cvt::PDROF::apply (cvt/gfx/PDROF.h:50-96),
 * cvt::PDROFInpaint::apply (cvt/gfx/PDROFInpaint.h:50-98) and single kernels of
 * cvt/cl/kernel/pmhstereo.cl.  It produces the golden fixtures under
 * tests/golden/ (tests/golden/make_golden.py) and never ships.
 */
#include <cmath>
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

/* ---- cvt::StereoGCVFilter (cvt/gfx/ifilter/StereoGCVFilter.cpp:75-242) ----
 * The kernels are the reference's; the launch sequence below repeats
 * StereoGCVFilter::depthmap / apply, IntegralFilter::apply / applyOuterRGB
 * (cvt/gfx/ifilter/IntegralFilter.cpp:68-170, block size 16) and
 * BoxFilter::apply (cvt/gfx/ifilter/BoxFilter.cpp:48-62) with their NDRanges.
 * The integral images of the box-SAD and NCC cost variants (imeanG1, G0, G12,
 * G02), which the point-SAD cost the reference compiles does not read, are not
 * formed.  The occlusion result is written to a GRAY_UINT8 image: the float
 * kernel output is converted as write_imagef does for CL_UNORM_INT8
 * (convert_uchar_sat_rte(v * 255)). */
namespace gcv {
struct Im {
    clemu::Img img;
    std::vector<float> d;
    Im(int w, int h, int ch) : d((size_t)w * h * ch, 0.0f) { img.w = w; img.h = h; img.channels = ch; img.data = d.data(); }
    void set(int ch) { d.assign((size_t)img.w * img.h * ch, 0.0f); img.channels = ch; img.data = d.data(); }
};
clemu::Arg I(Im& m) { clemu::Arg a; a.kind = clemu::Arg::IMAGE; a.img = &m.img; return a; }
clemu::Arg L(size_t bytes) { clemu::Arg a; a.kind = clemu::Arg::LOCAL; a.local_size = bytes; return a; }
clemu::Arg F4(const float* v) { clemu::Arg a; a.kind = clemu::Arg::FLOAT4; for (int k = 0; k < 4; ++k) a.f4[k] = v[k]; return a; }
const int BS = 16;

/* IntegralFilter::apply(dst, src, src2): dst takes src's channel count */
void integral(Im& dst, Im& src, Im* src2) {
    const int W = src.img.w, H = src.img.h;
    dst.set(src.img.channels);
    if (src2) {   /* (the squared variant, src2 == &src, serves only the unused NCC cost) */
        clemu::launch("prefixsum_pblock_mul2", {I(dst), I(src), I(*src2), L(16 * BS * BS)}, pad16(W), pad16(H), BS, BS);
    } else {
        clemu::launch("prefixsum_pblock", {I(dst), I(src), L(16 * BS * BS)}, pad16(W), pad16(H), BS, BS);
    }
    clemu::launch("prefixsum_horiz", {I(dst), I(dst), int_arg(BS)}, pad16(H), 1, BS, 1);
    clemu::launch("prefixsum_vert", {I(dst), I(dst), int_arg(BS)}, pad16(W), 1, BS, 1);
    clemu::launch("prefixsum_block2", {I(dst), I(dst)}, pad16(W), pad16(H), BS, BS);
}

void integral_outer(Im& rr, Im& gg, Im& src) {
    const int W = src.img.w, H = src.img.h;
    rr.set(4);
    gg.set(4);
    clemu::launch("prefixsum_pblock_outerrgb", {I(rr), I(gg), I(src), L(32 * BS * BS)}, pad16(W), pad16(H), BS, BS);
    for (Im* m : {&rr, &gg}) clemu::launch("prefixsum_horiz", {I(*m), I(*m), int_arg(BS)}, pad16(H), 1, BS, 1);
    for (Im* m : {&rr, &gg}) clemu::launch("prefixsum_vert", {I(*m), I(*m), int_arg(BS)}, pad16(W), 1, BS, 1);
    for (Im* m : {&rr, &gg}) clemu::launch("prefixsum_block2", {I(*m), I(*m)}, pad16(W), pad16(H), BS, BS);
}

void box(Im& dst, Im& src, int r) {   /* dst keeps its channel count */
    clemu::launch("boxfilter_prefixsum", {I(dst), I(src), int_arg(r)}, pad16(src.img.w), pad16(src.img.h), 16, 16);
}

/* StereoGCVFilter::depthmap (:75-242) with the point-SAD cost */
void depthmap(Im& dst, Im& cam0, Im& cam1, float dmin, float dmax, float dt) {
    const int W = cam0.img.w, H = cam0.img.h;
    const int RADIUS = 9;
    const float EPSILON = 1e-3f;
    Im cost(W, H, 1), costgf(W, H, 1), c0(W, H, 2), c1(W, H, 2), g0(W, H, 4), g1(W, H, 4);
    Im ia(W, H, 4), ib(W, H, 4), iint(W, H, 4), iint2(W, H, 4), imeanG(W, H, 4), imeanS(W, H, 1), imeanGS(W, H, 4);
    Im mRR(W, H, 4), mGG(W, H, 4);
    Im* c[2] = {&c0, &c1};
    int index = 0;
    const float fill[4] = {1e9f, 0.0f, 0.0f, 0.0f};
    clemu::launch("fill", {I(*c[!index]), F4(fill)}, pad16(W), pad16(H), 16, 16);
    clemu::launch("gradx", {I(g0), I(cam0), L(16 * 18 * 16)}, pad16(W), pad16(H), 16, 16);
    clemu::launch("gradx", {I(g1), I(cam1), L(16 * 18 * 16)}, pad16(W), pad16(H), 16, 16);
    integral(iint, cam1, nullptr);
    box(imeanG, iint, RADIUS);
    integral_outer(iint, iint2, cam1);
    box(mRR, iint, RADIUS);
    box(mGG, iint2, RADIUS);
    if (dmax < dmin && dt > 0) dt = -dt;
    size_t n = (size_t)(std::fabs(dmax - dmin) / std::fabs(dt));
    for (float d = dmin; n--; d += dt) {
        clemu::launch("stereogcv_costdepthgrad", {I(cost), I(cam1), I(cam0), I(g1), I(g0), float_arg(d)},
                      pad16(W), pad16(H), 16, 16);
        integral(iint, cost, nullptr);
        box(imeanS, iint, RADIUS);
        integral(iint, cam1, &cost);
        box(imeanGS, iint, RADIUS);
        clemu::launch("guidedfilter_calcab_outerrgb", {I(ia), I(ib), I(imeanG), I(imeanS), I(imeanGS), I(mRR), I(mGG),
                                                       float_arg(EPSILON)}, pad16(W), pad16(H), 16, 16);
        integral(iint, ia, nullptr);
        box(ia, iint, RADIUS);
        integral(iint, ib, nullptr);
        box(ib, iint, RADIUS);
        clemu::launch("guidedfilter_applyab_gc_outer", {I(costgf), I(cam1), I(ia), I(ib)}, pad16(W), pad16(H), 16, 16);
        clemu::launch("stereogcv_costmin", {I(*c[index]), I(costgf), I(*c[!index]),
                                            float_arg(std::fabs(d - dmin) / (std::fabs(dmax - dmin)))},
                      pad16(W), pad16(H), 16, 16);
        index = 1 - index;
    }
    clemu::launch("stereogcv_costdepthconv", {I(dst), I(*c[!index]), float_arg(1.0f), float_arg(0.0f)},
                  pad16(W), pad16(H), 16, 16);
}
}  // namespace gcv

/* StereoGCVFilter::depthmap on RGBA float images: dst W*H normalized depth. */
int ref_gcv_depthmap(float* out, const float* cam0, const float* cam1, int W, int H, float dmin, float dmax, float dt) {
    gcv::Im a(W, H, 4), b(W, H, 4), d(W, H, 1);
    memcpy(a.d.data(), cam0, sizeof(float) * 4 * (size_t)W * H);
    memcpy(b.d.data(), cam1, sizeof(float) * 4 * (size_t)W * H);
    gcv::depthmap(d, a, b, dmin, dmax, dt);
    memcpy(out, d.d.data(), sizeof(float) * (size_t)W * H);
    return 0;
}

/* StereoGCVFilter::apply (:75-95): both depth maps and the occlusion check
 * into GRAY_UINT8 (d0, d1 returned too; the reference also saves them as PNG
 * files, which is not done here). */
int ref_gcv_apply(uint8_t* out, float* d0out, float* d1out, const float* cam0, const float* cam1, int W, int H,
                  float dmin, float dmax, float dt) {
    gcv::Im a(W, H, 4), b(W, H, 4), d0(W, H, 1), d1(W, H, 1), o(W, H, 1);
    memcpy(a.d.data(), cam0, sizeof(float) * 4 * (size_t)W * H);
    memcpy(b.d.data(), cam1, sizeof(float) * 4 * (size_t)W * H);
    gcv::depthmap(d0, a, b, dmin, dmax, dt);
    gcv::depthmap(d1, b, a, -dmin, -dmax, -dt);
    clemu::launch("stereogcv_occlusioncheck", {gcv::I(o), gcv::I(d0), gcv::I(d1), float_arg(std::fabs(dmax))},
                  pad16(W), pad16(H), 16, 16);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        const float v = std::nearbyint(o.d[i] * 255.0f);   /* round to nearest even (default mode), saturate */
        out[i] = (uint8_t)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
    }
    memcpy(d0out, d0.d.data(), sizeof(float) * (size_t)W * H);
    memcpy(d1out, d1.d.data(), sizeof(float) * (size_t)W * H);
    return 0;
}

}  // extern "C"
