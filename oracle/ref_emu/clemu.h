/*
 * clemu.h — TEST INFRASTRUCTURE.  A small OpenCL C 1.x emulation that lets the
 * reference's own kernel sources (cvt/cl/kernel/pmhstereo.cl, RNG.cl,
 * PDHuberWeighted.cl, fill.cl), after the mechanical rewrite done by
 * translate.py, compile as C++ and run on the CPU.  Its outputs are the golden
 * fixtures that pin the oracle.
 *
 * What it fixes where OpenCL leaves a choice:
 *  - native_exp -> pm_wexp, exp -> pm_exp, pow -> pm_pow, acospi -> pm_acospi
 *    (cvt_gb300/csrc/pm_math.h); native_sqrt/sqrt -> IEEE sqrt,
 *    native_rsqrt -> 1/sqrt; dot/length/smoothstep evaluated left to right
 *    without contraction (the build uses -ffp-contract=off);
 *  - samplers follow the OpenCL 1.2 specification formulas (section 8.2) at
 *    full FP32 precision; the CLK_ADDRESS_CLAMP border colour is 0 for both
 *    CL_RGBA and CL_INTENSITY images; CL_INTENSITY reads return (I,I,I,I);
 *  - a float converted to int: NaN -> 0, out of range saturates;
 *  - vector literals evaluate their components left to right (brace
 *    initialisation);
 *  - work-groups run one after another in row-major order; inside a group
 *    the work-items run in raster order between barriers (fibers), so
 *    atomic_inc orders follow that sequence.
 */
#ifndef CLEMU_H
#define CLEMU_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <type_traits>
#include <utility>
#include <string>
#include <vector>

#include "clemu_api.h"
#include "pm_math.h"

#undef isfinite
#undef isnan
#undef isinf

namespace clemu {

typedef unsigned int uint;
typedef unsigned long ulong;
typedef unsigned char uchar;
typedef int sampler_t;

enum {
    CLK_NORMALIZED_COORDS_FALSE = 0,
    CLK_NORMALIZED_COORDS_TRUE = 1,
    CLK_ADDRESS_NONE = 0,
    CLK_ADDRESS_CLAMP_TO_EDGE = 2,
    CLK_ADDRESS_CLAMP = 4,
    CLK_ADDRESS_MASK = 6,
    CLK_FILTER_NEAREST = 0,
    CLK_FILTER_LINEAR = 16,
    CLK_LOCAL_MEM_FENCE = 1,
    CLK_GLOBAL_MEM_FENCE = 2
};

inline int cvt_i(float v) {
    if (v != v) return 0;
    if (v >= 2147483647.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}
template <class T> inline int to_int(T v) { return static_cast<int>(v); }
inline int to_int(float v) { return cvt_i(v); }
inline int to_int(double v) { return cvt_i((float)v); }
template <class T> inline uint to_uint(T v) { return static_cast<uint>(v); }
template <class T> inline float to_float(T v) { return static_cast<float>(v); }

struct float3;
struct float2 {
    float x, y;
    float2() : x(0), y(0) {}
    float2(float s) : x(s), y(s) {}
    template <class A, class B> float2(A a, B b) : x(to_float(a)), y(to_float(b)) {}
    float& s0() { return x; }
    float& s1() { return y; }
    float s0() const { return x; }
    float s1() const { return y; }
};
struct float3 {
    float x, y, z;
    float3() : x(0), y(0), z(0) {}
    float3(float s) : x(s), y(s), z(s) {}
    template <class A, class B, class C> float3(A a, B b, C c) : x(to_float(a)), y(to_float(b)), z(to_float(c)) {}
};
struct int2 {
    int x, y;
    int2() : x(0), y(0) {}
    int2(int s) : x(s), y(s) {}
    template <class A, class B> int2(A a, B b) : x(to_int(a)), y(to_int(b)) {}
};
struct int3 {
    int x, y, z;
    int3() : x(0), y(0), z(0) {}
    template <class A, class B, class C> int3(A a, B b, C c) : x(to_int(a)), y(to_int(b)), z(to_int(c)) {}
};
struct int4 { int x, y, z, w; };
struct uint2 {
    uint x, y;
    uint2() : x(0), y(0) {}
    template <class A, class B> uint2(A a, B b) : x(to_uint(a)), y(to_uint(b)) {}
};

/* swizzle proxies: .xy / .xyz of a float4 (translate.py rewrites them to calls) */
struct Swz2 {
    float* p[2];
    operator float2() const { return float2(*p[0], *p[1]); }
    Swz2& operator=(const float2& v) { *p[0] = v.x; *p[1] = v.y; return *this; }
    Swz2& operator=(float s) { *p[0] = s; *p[1] = s; return *this; }
    Swz2& operator-=(const float2& v) { *p[0] = *p[0] - v.x; *p[1] = *p[1] - v.y; return *this; }
    Swz2& operator+=(const float2& v) { *p[0] = *p[0] + v.x; *p[1] = *p[1] + v.y; return *this; }
};
struct Swz3 {
    float* p[3];
    operator float3() const { return float3(*p[0], *p[1], *p[2]); }
    Swz3& operator=(const float3& v) { *p[0] = v.x; *p[1] = v.y; *p[2] = v.z; return *this; }
    Swz3& operator=(float s) { *p[0] = s; *p[1] = s; *p[2] = s; return *this; }
    Swz3& operator*=(float s) { *p[0] = *p[0] * s; *p[1] = *p[1] * s; *p[2] = *p[2] * s; return *this; }
    Swz3& operator-=(const float3& v) { *p[0] = *p[0] - v.x; *p[1] = *p[1] - v.y; *p[2] = *p[2] - v.z; return *this; }
    Swz3& operator+=(const float3& v) { *p[0] = *p[0] + v.x; *p[1] = *p[1] + v.y; *p[2] = *p[2] + v.z; return *this; }
};

struct alignas(16) float4 {
    float x, y, z, w;
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float s) : x(s), y(s), z(s), w(s) {}
    template <class A, class B, class C, class D>
    float4(A a, B b, C c, D d) : x(to_float(a)), y(to_float(b)), z(to_float(c)), w(to_float(d)) {}
    float4(const float3& v, float w);   /* (float4)(v, w) */
    float4(float a, const float2& v, float d) : x(a), y(v.x), z(v.y), w(d) {}   /* (float4)(a, v, d) */
    Swz2 xy() const { float* q = const_cast<float*>(&x); return Swz2{{q, q + 1}}; }
    Swz3 xyz() const { float* q = const_cast<float*>(&x); return Swz3{{q, q + 1, q + 2}}; }
    float2 s01() const { return float2(x, y); }
    float2 s23() const { return float2(z, w); }
    Swz2 yz() const { float* q = const_cast<float*>(&x); return Swz2{{q + 1, q + 2}}; }
    Swz2 zw() const { float* q = const_cast<float*>(&x); return Swz2{{q + 2, q + 3}}; }
    float4& operator+=(const float4& o);
    float4& operator-=(const float4& o) { x = x - o.x; y = y - o.y; z = z - o.z; w = w - o.w; return *this; }
    float4& operator*=(const float4& o) { x = x * o.x; y = y * o.y; z = z * o.z; w = w * o.w; return *this; }
    float4& operator/=(const float4& o) { x = x / o.x; y = y / o.y; z = z / o.z; w = w / o.w; return *this; }
};
inline float4::float4(const float3& v, float w_) : x(v.x), y(v.y), z(v.z), w(w_) {}
struct alignas(32) float8 {
    float4 l, h;
    float8() {}
    float8(float s) : l(s), h(s) {}
    float8(const float4& a, const float4& b) : l(a), h(b) {}
    /* (float8)(float3, float, float2, float, float) */
    float8(const float3& a, float b, const float2& c, float d, float e) : l(a, b), h(c.x, c.y, d, e) {}
    float8& operator+=(const float8& o) { l += o.l; h += o.h; return *this; }
    float& s0() { return l.x; }
    float& s1() { return l.y; }
    float& s2() { return l.z; }
    float& s3() { return l.w; }
    float& s4() { return h.x; }
    float& s5() { return h.y; }
    float& s6() { return h.z; }
    float& s7() { return h.w; }
    float4 s0123() const { return l; }
    float4 s4567() const { return h; }
    float4& lo() { return l; }
    float4& hi() { return h; }
    const float4& lo() const { return l; }
    const float4& hi() const { return h; }
};

/* ----- arithmetic (componentwise, no contraction) ----- */
#define CLEMU_V2(op) \
    inline float2 operator op(const float2& a, const float2& b) { return float2(a.x op b.x, a.y op b.y); } \
    inline float2 operator op(const float2& a, float s) { return float2(a.x op s, a.y op s); } \
    inline float2 operator op(float s, const float2& a) { return float2(s op a.x, s op a.y); }
#define CLEMU_V3(op) \
    inline float3 operator op(const float3& a, const float3& b) { return float3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline float3 operator op(const float3& a, float s) { return float3(a.x op s, a.y op s, a.z op s); } \
    inline float3 operator op(float s, const float3& a) { return float3(s op a.x, s op a.y, s op a.z); }
#define CLEMU_V4(op) \
    inline float4 operator op(const float4& a, const float4& b) { return float4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); } \
    inline float4 operator op(const float4& a, float s) { return float4(a.x op s, a.y op s, a.z op s, a.w op s); } \
    inline float4 operator op(float s, const float4& a) { return float4(s op a.x, s op a.y, s op a.z, s op a.w); }
CLEMU_V2(+) CLEMU_V2(-) CLEMU_V2(*) CLEMU_V2(/)
CLEMU_V3(+) CLEMU_V3(-) CLEMU_V3(*) CLEMU_V3(/)
CLEMU_V4(+) CLEMU_V4(-) CLEMU_V4(*) CLEMU_V4(/)
inline float3 operator-(const Swz3& a, const Swz3& b) { return float3(a) - float3(b); }
inline float2 operator/(const Swz2& a, float s) { return float2(a) / s; }
inline float2 operator*(const Swz2& a, float s) { return float2(a) * s; }
inline float3 operator*(const Swz3& a, float s) { return float3(a) * s; }
inline float3 operator*(float s, const Swz3& a) { return s * float3(a); }
inline float2 operator*(float s, const Swz2& a) { return s * float2(a); }
inline int2 operator-(const int2& a, const int2& b) { return int2(a.x - b.x, a.y - b.y); }
inline int2 min(const int2& a, const int2& b) { return int2(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y); }
inline int2 max(const int2& a, const int2& b) { return int2(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y); }
inline int mul24(int a, int b) { return a * b; }   /* exact for the 24-bit operands of these kernels */
inline float4 operator-(const float4& a) { return float4(-a.x, -a.y, -a.z, -a.w); }
inline float4& float4::operator+=(const float4& o) { x = x + o.x; y = y + o.y; z = z + o.z; w = w + o.w; return *this; }
inline float8 operator/(const float8& a, const float8& b) { return float8(a.l / b.l, a.h / b.h); }
inline int2 operator+(const int2& a, const int2& b) { return int2(a.x + b.x, a.y + b.y); }
inline float2 operator+(const int2& a, const float2& b) { return float2((float)a.x + b.x, (float)a.y + b.y); }

/* ----- built-in functions ----- */
inline float fabs(float v) { return std::fabs(v); }
inline float3 fabs(const float3& v) { return float3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float4 fabs(const float4& v) { return float4(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z), std::fabs(v.w)); }
inline float fmin(float a, float b) { return std::fmin(a, b); }
inline float fmax(float a, float b) { return std::fmax(a, b); }
inline float3 fmin(const float3& a, float s) { return float3(std::fmin(a.x, s), std::fmin(a.y, s), std::fmin(a.z, s)); }
inline float4 fmin(const float4& a, float s) { return float4(std::fmin(a.x, s), std::fmin(a.y, s), std::fmin(a.z, s), std::fmin(a.w, s)); }
inline float4 fmax(const float4& a, const float4& b) { return float4(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z), std::fmax(a.w, b.w)); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
/* OpenCL min/max of floats: y < x ? y : x and x < y ? y : x (6.12.4) */
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float4 cross(const float4& a, const float4& b) {   /* OpenCL 6.12.5: w = 0 */
    return float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
inline float clamp(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }
inline float sqrt(float v) { return std::sqrt(v); }
inline float4 sqrt(const float4& v) { return float4(std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z), std::sqrt(v.w)); }
inline float native_sqrt(float v) { return std::sqrt(v); }
inline float native_rsqrt(float v) { return 1.0f / std::sqrt(v); }
inline float native_exp(float v) { return pm_wexp(v); }
inline float exp(float v) { return pm_exp(v); }
inline float pow(float a, float b) { return pm_pow(a, b); }
inline float acospi(float v) { return pm_acospi(v); }
inline float round(float v) { return std::round(v); }
inline float floor(float v) { return std::floor(v); }
inline float3 floor(const float3& v) { return float3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline float3 fmin(const float3& a, const float3& b) {
    return float3(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z));
}
inline float3 fmax(const float3& a, const float3& b) {
    return float3(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z));
}
/* mix(x, y, a) = x + (y - x) * a (OpenCL 1.2, 6.12.4), per component */
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline float2 mix(const float2& a, const float2& b, float t) { return float2(mix(a.x, b.x, t), mix(a.y, b.y, t)); }
inline float4 mix(const float4& a, const float4& b, float t) {
    return float4(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t), mix(a.w, b.w, t));
}
/* sincos(float3, float3*) appears in helpers of Matrix4.cl (mat4f_rotation)
 * that no emulated kernel calls; it is not emulated. */
inline float3 sincos(const float3&, float3*) {
    std::fprintf(stderr, "clemu: sincos(float3) is not emulated\n");
    std::abort();
}
/* normalize: OpenCL leaves its rounding to the implementation; here
 * v * (1 / sqrt(dot(v, v))), the native_rsqrt convention above */
inline float3 normalize(const float3& v) {
    const float r = 1.0f / std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
    return float3(v.x * r, v.y * r, v.z * r);
}
inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const float3& a, const float3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const float4& a, const float4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float length(const float2& a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline float length(const float3& a) { return std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }
inline float length(const float4& a) { return std::sqrt(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w); }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline int isfinite(float v) { return std::isfinite(v) ? 1 : 0; }
inline int3 isfinite(const float3& v) {
    return int3{std::isfinite(v.x) ? -1 : 0, std::isfinite(v.y) ? -1 : 0, std::isfinite(v.z) ? -1 : 0};
}
inline int all(const int3& v) { return (v.x < 0) && (v.y < 0) && (v.z < 0); }
inline int all(int v) { return v < 0; }
inline float select(float a, float b, int c) { return c ? b : a; }
inline int mad24(int a, int b, int c) { return a * b + c; }
inline uint mad_hi(uint a, uint b, uint c) { return (uint)(((unsigned long long)a * b) >> 32) + c; }
inline int atomic_inc(int* p) { int o = *p; *p = o + 1; return o; }

/* ----- images ----- */
typedef Img* image2d_t;

inline int get_image_width(image2d_t i) { return i->w; }
inline int get_image_height(image2d_t i) { return i->h; }

inline float4 texel(image2d_t img, int x, int y, int addr) {
    if (addr == CLK_ADDRESS_CLAMP_TO_EDGE) {
        x = x < 0 ? 0 : (x >= img->w ? img->w - 1 : x);
        y = y < 0 ? 0 : (y >= img->h ? img->h - 1 : y);
    } else if (x < 0 || y < 0 || x >= img->w || y >= img->h) {
        return float4(0.0f);    /* CLK_ADDRESS_CLAMP border colour */
    }
    if (img->channels == 1) return float4(img->data[(size_t)y * img->w + x]);   /* CL_INTENSITY: (I, I, I, I) */
    if (img->channels == 2) {                                                    /* CL_RG: (R, G, 0, 1) */
        const float* q = img->data + ((size_t)y * img->w + x) * 2;
        return float4(q[0], q[1], 0.0f, 1.0f);
    }
    const float* p = img->data + ((size_t)y * img->w + x) * 4;
    return float4(p[0], p[1], p[2], p[3]);
}

inline float4 read_imagef(image2d_t img, sampler_t s, int2 c) { return texel(img, c.x, c.y, s & CLK_ADDRESS_MASK); }

inline float4 read_imagef(image2d_t img, sampler_t s, float2 c) {
    const int addr = s & CLK_ADDRESS_MASK;
    if ((s & CLK_FILTER_LINEAR) == 0)
        return texel(img, cvt_i(std::floor(c.x)), cvt_i(std::floor(c.y)), addr);
    /* OpenCL 1.2 section 8.2: i0 = floor(u - 0.5), a = frac(u - 0.5); result
     * (1-a)(1-b)T_i0j0 + a(1-b)T_i1j0 + (1-a)b T_i0j1 + ab T_i1j1 */
    float tu = c.x - 0.5f, tv = c.y - 0.5f;
    float fu = std::floor(tu), fv = std::floor(tv);
    float a = tu - fu, b = tv - fv;
    int i0 = cvt_i(fu), j0 = cvt_i(fv);
    float4 t00 = texel(img, i0, j0, addr), t10 = texel(img, i0 + 1, j0, addr);
    float4 t01 = texel(img, i0, j0 + 1, addr), t11 = texel(img, i0 + 1, j0 + 1, addr);
    return ((1.0f - a) * (1.0f - b)) * t00 + (a * (1.0f - b)) * t10 + ((1.0f - a) * b) * t01 + (a * b) * t11;
}

inline void write_imagef(image2d_t img, int2 c, float4 v) {
    if (c.x < 0 || c.y < 0 || c.x >= img->w || c.y >= img->h) return;
    if (img->channels == 1) { img->data[(size_t)c.y * img->w + c.x] = v.x; return; }
    if (img->channels == 2) { float* q = img->data + ((size_t)c.y * img->w + c.x) * 2; q[0] = v.x; q[1] = v.y; return; }
    float* p = img->data + ((size_t)c.y * img->w + c.x) * 4;
    p[0] = v.x; p[1] = v.y; p[2] = v.z; p[3] = v.w;
}

/* ----- work-item context (clemu_rt.cpp) ----- */
struct WorkItem { size_t gid[3], lid[3], grp[3], lsz[3]; };
extern thread_local WorkItem* t_item;
inline size_t get_global_id(int d) { return t_item->gid[d]; }
inline size_t get_local_id(int d) { return t_item->lid[d]; }
inline size_t get_group_id(int d) { return t_item->grp[d]; }
inline size_t get_local_size(int d) { return t_item->lsz[d]; }
void barrier(int flags);

/* kernel registration (clemu_rt.cpp) */
typedef std::function<void(const std::vector<Arg>&)> ItemFn;   /* runs one work-item */
void reg(const std::string& name, bool uses_barrier, ItemFn fn);
void* local_arena(int index, size_t bytes);

/* any other argument type: a struct passed by value (Arg::BYTES) */
template <class T> struct ArgConv {
    static T get(const Arg& a, int) {
        T t;
        std::memcpy((void*)&t, a.bytes.data(), sizeof(T));
        return t;
    }
};
template <> struct ArgConv<image2d_t> { static image2d_t get(const Arg& a, int) { return a.img; } };
template <> struct ArgConv<int> { static int get(const Arg& a, int) { return a.kind == Arg::FLOAT ? (int)a.f : a.i; } };
template <> struct ArgConv<float> { static float get(const Arg& a, int) { return a.kind == Arg::INT ? (float)a.i : a.f; } };
template <> struct ArgConv<float4> { static float4 get(const Arg& a, int) { return float4(a.f4[0], a.f4[1], a.f4[2], a.f4[3]); } };
template <class P> struct ArgConv<P*> {
    static P* get(const Arg& a, int idx) { return (P*)(a.kind == Arg::LOCAL ? local_arena(idx, a.local_size) : a.ptr); }
};
template <class... A, size_t... I>
inline void call_kernel(void (*fn)(A...), const std::vector<Arg>& args, std::index_sequence<I...>) {
    fn(ArgConv<typename std::decay<A>::type>::get(args[I], (int)I)...);
}
template <class... A>
inline void reg_kernel(const char* name, bool uses_barrier, void (*fn)(A...)) {
    reg(name, uses_barrier, [fn](const std::vector<Arg>& args) { call_kernel(fn, args, std::index_sequence_for<A...>{}); });
}

}  // namespace clemu

#define kernel
#define __kernel
#define global
#define __global
#define __local
#define __constant
#define read_only
#define write_only
#define __read_only
#define __write_only

#endif
