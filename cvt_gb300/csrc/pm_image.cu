/*
 * pm_image.cu — the reference's image formats as its kernels read them.
 *
 * cvt::PMHuberStereo reads its left/right cvt::Image objects through OpenCL
 * images: IFormat::toCLImageFormat (cvt/gfx/IFormat.h:293-328) gives each
 * cvt::IFormatID an OpenCL channel order and type, and read_imagef returns
 * RGBA floats from them (OpenCL 1.2, 6.12.14 and 8.3.1.1).  k_image_to_rgbaf
 * performs that read once per pixel into the RGBA float32 layout the rest of
 * the library works on.  One thread per pixel; the format switch is uniform
 * over the grid.  HBM-bound: bpp bytes read and 16 written per pixel.
 */
#include <string>

#include "cvtpm.h"
#include "pm_kernels.cuh"

namespace {

enum Order { ORD_INTENSITY, ORD_RG, ORD_RA, ORD_RGBA, ORD_BGRA };
enum Type { TY_UNORM8, TY_UNORM16, TY_SNORM16, TY_FLOAT };

struct FormatDesc {
    int channels;   /* stored per pixel */
    int order;
    int type;
};

/* cvt/gfx/IFormat.h:299-322, indexed by IFormatID */
bool describe(int f, FormatDesc* d) {
    static const FormatDesc tab[] = {
        {0, 0, 0},
        {1, ORD_INTENSITY, TY_UNORM8}, {1, ORD_INTENSITY, TY_UNORM16}, {1, ORD_INTENSITY, TY_SNORM16},
        {1, ORD_INTENSITY, TY_FLOAT},
        {2, ORD_RG, TY_UNORM8}, {2, ORD_RG, TY_UNORM16}, {2, ORD_RG, TY_SNORM16}, {2, ORD_RG, TY_FLOAT},
        {4, ORD_RGBA, TY_UNORM8}, {4, ORD_RGBA, TY_UNORM16}, {4, ORD_RGBA, TY_SNORM16}, {4, ORD_RGBA, TY_FLOAT},
        {4, ORD_BGRA, TY_UNORM8}, {4, ORD_BGRA, TY_UNORM16}, {4, ORD_BGRA, TY_SNORM16}, {4, ORD_BGRA, TY_FLOAT},
        {1, ORD_INTENSITY, TY_UNORM8}, {1, ORD_INTENSITY, TY_UNORM8}, {1, ORD_INTENSITY, TY_UNORM8},
        {2, ORD_RA, TY_UNORM8}, {2, ORD_RA, TY_UNORM8},
    };
    if (f < CVTPM_IFORMAT_GRAY_UINT8 || f > CVTPM_IFORMAT_UYVY_UINT8) return false;
    *d = tab[f];
    return true;
}

size_t type_bytes(int t) { return t == TY_UNORM8 ? 1 : (t == TY_FLOAT ? 4 : 2); }

thread_local std::string g_err;

cvtpm_status fail(cvtpm_status s, const std::string& m) {
    g_err = m;
    return s;
}

/* OpenCL 1.2, 8.3.1.1: normalized integer to float. */
__device__ __forceinline__ float conv(const unsigned char* p, int type) {
    switch (type) {
    case TY_UNORM8: return (float)p[0] / 255.0f;
    case TY_UNORM16: return (float)*(const unsigned short*)p / 65535.0f;
    case TY_SNORM16: return fmaxf(-1.0f, (float)*(const short*)p / 32767.0f);
    default: return *(const float*)p;
    }
}

__global__ void __launch_bounds__(256) k_image_to_rgbaf(const unsigned char* __restrict__ src, size_t stride,
                                                        int W, int H, FormatDesc d, float4* __restrict__ dst,
                                                        size_t dpitch4) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= W || y >= H) return;
    const int tb = d.type == TY_UNORM8 ? 1 : (d.type == TY_FLOAT ? 4 : 2);
    const unsigned char* p = src + (size_t)y * stride + (size_t)x * d.channels * tb;
    float4 o;
    switch (d.order) {
    case ORD_INTENSITY: {
        const float v = conv(p, d.type);
        o = make_float4(v, v, v, v);
        break;
    }
    case ORD_RG: o = make_float4(conv(p, d.type), conv(p + tb, d.type), 0.0f, 1.0f); break;
    case ORD_RA: o = make_float4(conv(p, d.type), 0.0f, 0.0f, conv(p + tb, d.type)); break;
    case ORD_RGBA:
        o = make_float4(conv(p, d.type), conv(p + tb, d.type), conv(p + 2 * tb, d.type), conv(p + 3 * tb, d.type));
        break;
    default:   /* stored B, G, R, A */
        o = make_float4(conv(p + 2 * tb, d.type), conv(p + tb, d.type), conv(p, d.type), conv(p + 3 * tb, d.type));
        break;
    }
    dst[(size_t)y * dpitch4 + x] = o;
}

/* Validates an image descriptor; on success *d describes its format. */
cvtpm_status check_image(const cvtpm_image* img, const char* what, FormatDesc* d, std::string* msg) {
    const std::string w(what);
    if (!img) { *msg = w + ": descriptor is NULL"; return CVTPM_ERR_INVALID_ARGUMENT; }
    if (!describe(img->format, d)) { *msg = w + ": unknown image format " + std::to_string(img->format); return CVTPM_ERR_INVALID_ARGUMENT; }
    if (img->width < 1 || img->height < 1) { *msg = w + ": empty image"; return CVTPM_ERR_SIZE; }
    const size_t tb = type_bytes(d->type);
    if (!img->data) { *msg = w + ": data is NULL"; return CVTPM_ERR_INVALID_ARGUMENT; }
    if (img->stride < (size_t)img->width * d->channels * tb) { *msg = w + ": stride below width * bytes per pixel"; return CVTPM_ERR_INVALID_ARGUMENT; }
    if ((uintptr_t)img->data % tb || img->stride % tb) { *msg = w + ": data or stride not aligned to the channel size"; return CVTPM_ERR_INVALID_ARGUMENT; }
    return CVTPM_OK;
}

cudaError_t launch_image_to_rgbaf(const cvtpm_image* img, float4* dst, size_t dst_pitch, cudaStream_t st) {
    FormatDesc d;
    describe(img->format, &d);
    const dim3 grid((img->width + 31) / 32, (img->height + 7) / 8);
    k_image_to_rgbaf<<<grid, dim3(32, 8), 0, st>>>((const unsigned char*)img->data, img->stride, img->width,
                                                    img->height, d, dst, dst_pitch / 16);
    return cudaGetLastError();
}

}  // namespace

/* The conversion of one image for cvtpm_depthmap_image (context scratch). */
cvtpm_status pm_image_to_rgbaf_checked(const cvtpm_image* img, const char* what, float4* dst, size_t dst_pitch,
                                       cudaStream_t st, std::string* msg) {
    FormatDesc d;
    cvtpm_status s = check_image(img, what, &d, msg);
    if (s != CVTPM_OK) return s;
    cudaError_t e = launch_image_to_rgbaf(img, dst, dst_pitch, st);
    if (e != cudaSuccess) { *msg = std::string(what) + ": " + cudaGetErrorString(e); return CVTPM_ERR_CUDA; }
    return CVTPM_OK;
}

const char* pm_free_error() { return g_err.c_str(); }
void pm_set_free_error(const std::string& m) { g_err = m; }

extern "C" {

size_t cvtpm_iformat_bpp(int format) {
    FormatDesc d;
    if (!describe(format, &d)) return 0;
    return (size_t)d.channels * type_bytes(d.type);
}

cvtpm_status cvtpm_image_to_rgbaf(const cvtpm_image* src, float* dst, size_t dst_pitch, void* stream) {
    std::string msg;
    FormatDesc d;
    cvtpm_status s = check_image(src, "src", &d, &msg);
    if (s != CVTPM_OK) return fail(s, msg);
    if (!dst || dst_pitch % 16 || dst_pitch < (size_t)src->width * 16)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "dst is NULL or its pitch is not a multiple of 16 of at least width * 16");
    cudaError_t e = launch_image_to_rgbaf(src, (float4*)dst, dst_pitch, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(CVTPM_ERR_CUDA, std::string("image conversion: ") + cudaGetErrorString(e));
    return CVTPM_OK;
}

}  // extern "C"
