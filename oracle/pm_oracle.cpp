/*
 * pm_oracle.cpp — TEST INFRASTRUCTURE: the CPU oracle of the slanted-plane
 * PatchMatch stereo path.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm load it, and only as a checker or as the timed
 * CPU baseline.  The product (cvt_gb300/, libcvtpm.so) never links it.
 *
 * It restates, in plain C++17 FP32 (no contraction, IEEE division and sqrt, no
 * flush-to-zero), the reference's OpenCL path:
 *   cvt/cl/kernel/pmhstereo.cl      kernels and plane algebra
 *   cvt/cl/kernel/RNG.cl            MWC64X generator
 *   cvt/cl/kernel/PDHuberWeighted.cl + cvt/gfx/PDROF.h   Huber-TV smoother
 *   cvt/vision/PMHuberStereo.cpp:64-291                 the depthMap schedule
 * Each function names the lines it follows.
 *
 * Choices where the reference is not deterministic or not defined:
 *  - native_exp / exp / pow / acospi use the project's functions
 *    (cvt_gb300/csrc/pm_math.h); native_sqrt / native_rsqrt are IEEE sqrt and
 *    1/sqrt.  OpenCL leaves their accuracy to the implementation.
 *  - The view-candidate scatter (pmhstereo.cl:394-400) races on atomic_inc;
 *    here the up-to-4 survivors of a target pixel are the sources with the
 *    smallest x, in increasing x — the order a sequential execution of the
 *    reference's 16x16 work-groups (row-major groups, raster order inside a
 *    group) produces, because only sources of the same row compete.
 *  - Vector literals evaluate their components left to right (the random
 *    neighbour offsets draw x before y, pmhstereo.cl:356).
 *  - Non-finite sample positions are treated as outside the image, and a NaN
 *    converted to int is 0 (the NVIDIA conversion).  These only arise for
 *    non-finite plane states.
 * The bilinear sampler is the OpenCL specification's formula at full FP32
 * precision (no 8-bit fraction quantisation as texture hardware has).
 *
 * ARITH_FAST selects the tap arithmetic of the CUDA fast kernel instead
 * (FMA forms, (value, forward-difference) records of the other view,
 * separate colour/gradient accumulators); it is the bit-exact CPU mirror of
 * that kernel.
 */
#include <cfloat>
#include "cvtpm.h"
#include "pm_math.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct F4 { float x, y, z, w; };
static inline F4 f4(float x, float y, float z, float w) { F4 r = {x, y, z, w}; return r; }
static inline F4 f4s(float s) { return f4(s, s, s, s); }
static inline F4 operator+(F4 a, F4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline F4 operator-(F4 a, F4 b) { return f4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline F4 operator*(F4 a, F4 b) { return f4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
static inline F4 operator/(F4 a, F4 b) { return f4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
static inline F4 operator*(float s, F4 a) { return f4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline bool finite3(F4 s) { return std::isfinite(s.x) && std::isfinite(s.y) && std::isfinite(s.z); }
static inline float len4(F4 a) { return sqrtf(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w); }
static inline float len3(F4 a) { return sqrtf((a.x * a.x + a.y * a.y) + a.z * a.z); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int f2i_nan0(float v) { return (v != v) ? 0 : (int)v; }

/* ------------------------------------------------------------------ RNG -- */
/* MWC64X, RNG.cl:35-156.  MulMod64 is evaluated with a 128-bit product; it
 * returns the same residue as the bit-serial loop of RNG.cl:49-59
 * (orc_mwc_mulmod_serial keeps that loop for the known-answer test). */
const uint32_t MWC_A = 4294883355u;
const uint64_t MWC_M = 18446383549859758079ull;
const uint64_t MWC_BASEID = 4077358422479273989ull;

static inline uint64_t mwc_addmod(uint64_t a, uint64_t b, uint64_t M) {  /* RNG.cl:35-41 */
    uint64_t v = a + b;
    if ((v >= M) || (v < a)) v = v - M;
    return v;
}
static uint64_t mwc_mulmod_serial(uint64_t a, uint64_t b, uint64_t M) { /* RNG.cl:49-59 */
    uint64_t r = 0;
    while (a != 0) {
        if (a & 1) r = mwc_addmod(r, b, M);
        b = mwc_addmod(b, b, M);
        a = a >> 1;
    }
    return r;
}
static inline uint64_t mwc_mulmod(uint64_t a, uint64_t b, uint64_t M) {
    return (uint64_t)(((unsigned __int128)a * b) % M);
}
static uint64_t mwc_powmod(uint64_t a, uint64_t e, uint64_t M) {       /* RNG.cl:66-76 */
    uint64_t sqr = a, acc = 1;
    while (e != 0) {
        if (e & 1) acc = mwc_mulmod(acc, sqr, M);
        sqr = mwc_mulmod(sqr, sqr, M);
        e = e >> 1;
    }
    return acc;
}

struct Rng {
    int kind;
    uint32_t x, c;                  /* MWC64X */
    uint32_t ctr[4], key[2], buf[4];/* Philox */
    uint32_t n;
};

/* RNG_init(rng, linpos, numdraws) = SeedStreams(0, 0) then Skip(linpos*numdraws),
 * RNG.cl:151-154 with RNG.cl:78-100,120-132. */
static void mwc_init(Rng& r, uint64_t distance) {
    uint64_t m0 = mwc_powmod(MWC_A, 0, MWC_M);           /* dist = 0 + gid*1*0 */
    uint64_t x = mwc_mulmod(MWC_BASEID, m0, MWC_M);
    uint32_t sx = (uint32_t)(x / MWC_A), sc = (uint32_t)(x % MWC_A);
    uint64_t m = mwc_powmod(MWC_A, distance, MWC_M);
    uint64_t v = (uint64_t)sx * (uint64_t)MWC_A + sc;
    v = mwc_mulmod(v, m, MWC_M);
    r.kind = CVTPM_RNG_MWC64X;
    r.x = (uint32_t)(v / MWC_A);
    r.c = (uint32_t)(v % MWC_A);
}
static inline float mwc_float(Rng& r) {                                /* RNG.cl:108-118,142-147 */
    uint32_t res = r.x ^ r.c;
    uint32_t X = r.x, C = r.c;
    uint32_t Xn = MWC_A * X + C;
    uint32_t carry = (uint32_t)(Xn < C);
    uint32_t Cn = (uint32_t)(((uint64_t)MWC_A * X) >> 32) + carry;    /* mad_hi */
    r.x = Xn; r.c = Cn;
    return 2.3283064365386962890625e-10f * (float)res;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter (pixel, tag,
 * view, block), key = seed.  Draw k is word k%4 of block k/4. */
static inline void philox10(const uint32_t in[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
const uint32_t PHILOX_TAG_INIT = 0xFFFFFFFFu;
static void philox_init(Rng& r, uint64_t seed, uint32_t pixel, uint32_t tag, uint32_t view) {
    r.kind = CVTPM_RNG_PHILOX;
    r.ctr[0] = pixel; r.ctr[1] = tag; r.ctr[2] = view; r.ctr[3] = 0;
    r.key[0] = (uint32_t)seed; r.key[1] = (uint32_t)(seed >> 32);
    r.n = 0;
}
static inline float philox_float(Rng& r) {
    if ((r.n & 3u) == 0) { r.ctr[3] = r.n >> 2; philox10(r.ctr, r.key, r.buf); }
    uint32_t u = r.buf[r.n & 3u];
    r.n++;
    return 2.3283064365386962890625e-10f * (float)u;
}
static inline float rng_float(Rng& r) { return r.kind == CVTPM_RNG_PHILOX ? philox_float(r) : mwc_float(r); }

/* ------------------------------------------------------- plane algebra -- */
static inline F4 viewprop(F4 n) {                                      /* pmhstereo.cl:119-124 */
    return f4(1.0f / n.x, -n.y / n.x, -n.z / n.x, 0.0f);
}
static inline float transform_x(F4 s, float cx, float cy) {            /* :126-129 */
    return s.x * cx + s.y * cy + s.z;
}
static F4 state_init(Rng& rng, float cx, float cy, int lr, float normmul, float depthmax) {  /* :50-68 */
    float z = rng_float(rng) * depthmax;
    float nx = (rng_float(rng) - 0.5f) * normmul * 0.95f;
    float ny = (rng_float(rng) - 0.5f) * normmul * 0.95f;
    nx = pm_clamp(nx, -0.95f, 0.95f);
    ny = pm_clamp(ny, -0.95f, 0.95f);
    float nfactor = fmaxf(sqrtf(nx * nx + ny * ny) + 0.001f, 1.0f);
    nx = nx / nfactor; ny = ny / nfactor;
    float nz = sqrtf(1.0f - nx * nx - ny * ny);
    F4 ret = f4(1.0f - (-nx / nz), 0.0f - (-ny / nz), 0.0f - ((nx * cx + ny * cy) / nz + z), 0.0f - 0.0f);
    if (!lr) ret = viewprop(ret);
    return ret;
}
static F4 to_ref_normal_depth(F4 state, float cx, float cy, int lr) {  /* :70-86 */
    F4 s = lr ? state : viewprop(state);
    s = f4(1.0f - s.x, 0.0f - s.y, 0.0f - s.z, 0.0f - s.w);
    F4 ret;
    ret.w = s.x * cx + s.y * cy + s.z;
    ret.z = pm_rsqrt(s.x * s.x + s.y * s.y + 1.0f);
    ret.x = -s.x * ret.z;
    ret.y = -s.y * ret.z;
    if (!finite3(ret)) return f4(0.0f, 0.0f, 1.0f, 0.0f);
    return ret;
}
static F4 state_refine(Rng& rng, F4 in, float cx, float cy, float depthmax, int lr) {  /* :88-117 */
    F4 state = lr ? in : viewprop(in);
    state = f4(1.0f - state.x, 0.0f - state.y, 0.0f - state.z, 0.0f - state.w);
    float z = state.x * cx + state.y * cy + state.z;
    float nz = pm_rsqrt(state.x * state.x + state.y * state.y + 1.0f);
    float nx = -state.x * nz;
    float ny = -state.y * nz;
    z += (rng_float(rng) - 0.5f) * 2.0f;
    z = pm_clamp(z, 0.0f, depthmax);
    nx += (rng_float(rng) - 0.5f) * 0.1f;
    ny += (rng_float(rng) - 0.5f) * 0.1f;
    nx = pm_clamp(nx, -0.95f, 0.95f);
    ny = pm_clamp(ny, -0.95f, 0.95f);
    float nfactor = fmaxf(sqrtf(nx * nx + ny * ny) + 0.001f, 1.0f);
    nx = nx / nfactor; ny = ny / nfactor;
    nz = sqrtf(1.0f - nx * nx - ny * ny);
    F4 ret = f4(-nx / nz, -ny / nz, (nx * cx + ny * cy) / nz + z, 0.0f);
    ret = f4(1.0f - ret.x, 0.0f - ret.y, 0.0f - ret.z, 0.0f - ret.w);
    if (!lr) return viewprop(state);   /* the reference returns the unperturbed state here (:114-115) */
    return ret;
}
static inline void to_normal(F4 st, float n[3]) {                     /* :144-153 */
    F4 s = f4(1.0f - st.x, 0.0f - st.y, 0.0f - st.z, 0.0f - st.w);
    n[2] = pm_rsqrt(s.x * s.x + s.y * s.y + 1.0f);
    n[0] = -s.x * n[2];
    n[1] = -s.y * n[2];
}
static inline float dot4(F4 a, F4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
static void smooth_distance(F4 sa, F4 sb, F4 smooth, float cx, float cy, float depthmax, int lr,
                            float* dA, float* dB) {                  /* :266-283 */
    F4 a = to_ref_normal_depth(sa, cx, cy, lr);
    F4 b = to_ref_normal_depth(sb, cx, cy, lr);
    F4 diag = f4(1.0f, 1.0f, 0.0f, 1.0f / (depthmax * depthmax));
    if (!finite3(sa) || !finite3(sb)) { *dA = 0.0f; *dB = 0.0f; return; }
    F4 da = a - smooth;
    *dA = dot4(da, diag * da);
    F4 db = b - smooth;
    *dB = dot4(db, diag * db);
}

/* -------------------------------------------------------- view images -- */
struct View {
    int W, H;
    const F4* col;    /* RGBA input                       */
    const F4* grad;   /* (dx, dy, dxy, dyx), :785-831      */
    std::vector<float> rec; /* FAST: 14 floats per pixel: T(x) then T(x+1)-T(x) */
};

static void build_records(View& v) {
    int W = v.W, H = v.H;
    v.rec.assign((size_t)W * H * 14, 0.0f);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const F4& c0 = v.col[(size_t)y * W + x];
            const F4& g0 = v.grad[(size_t)y * W + x];
            int x1 = std::min(x + 1, W - 1);
            const F4& c1 = v.col[(size_t)y * W + x1];
            const F4& g1 = v.grad[(size_t)y * W + x1];
            float T0[7] = {c0.x, c0.y, c0.z, g0.x, g0.y, g0.z, g0.w};
            float T1[7] = {c1.x, c1.y, c1.z, g1.x, g1.y, g1.z, g1.w};
            float* r = &v.rec[((size_t)y * W + x) * 14];
            for (int k = 0; k < 7; ++k) { r[k] = T0[k]; r[7 + k] = T1[k] - T0[k]; }
        }
}

struct CostCfg {
    int P;
    float alpha, one_m_alpha, cmax, gmax;
    int arith;
    std::vector<float> prof;   /* (2P+1)^2 spatial profile */
};

static CostCfg make_cost_cfg(const cvtpm_params* p) {
    CostCfg c;
    c.P = p->patchsize;
    c.alpha = p->color_alpha;
    c.one_m_alpha = 1.0f - p->color_alpha;
    c.cmax = p->color_maxdiff;
    c.gmax = p->grad_maxdiff;
    c.arith = p->arith;
    int n = 2 * c.P + 1;
    c.prof.resize((size_t)n * n);
    for (int dy = -c.P; dy <= c.P; ++dy)
        for (int dx = -c.P; dx <= c.P; ++dx)
            c.prof[(size_t)(dy + c.P) * n + (dx + c.P)] = pm_profile(dx, dy, p->color_weight, p->weight_profile);
    return c;
}

/* patch_eval_color_grad_weighted, pmhstereo.cl:170-228. */
static float cost_eval(const CostCfg& k, const View& v1, const View& v2, int cx, int cy, F4 s) {
    if (!finite3(s)) return 1e5f;
    const int W = v1.W, H = v1.H, P = k.P, n = 2 * P + 1;
    const float Wf = (float)W, Hf = (float)H;
    const F4 vc = v1.col[(size_t)cy * W + cx];
    if (k.arith == CVTPM_ARITH_EXACT) {
        float wsum = 0.0f, ret = 0.0f;
        for (int dy = -P; dy <= P; ++dy) {
            for (int dx = -P; dx <= P; ++dx) {
                float px = (float)cx + (float)dx, py = (float)cy + (float)dy;
                if (px < 0 || px >= Wf || py < 0 || py >= Hf) continue;
                const F4 a1 = v1.col[(size_t)(int)py * W + (int)px];
                const F4 g1 = v1.grad[(size_t)(int)py * W + (int)px];
                float d = (fabsf(vc.x - a1.x) + fabsf(vc.y - a1.y)) + fabsf(vc.z - a1.z);
                float w1 = pm_wexp(-d * k.prof[(size_t)(dy + P) * n + (dx + P)]);
                float xp = s.x * px + s.y * py + s.z;
                if (!(xp >= 0.0f && xp < Wf)) continue;
                wsum += w1;
                /* read_imagef(SAMPLER_BILINEAR, (xp+0.5, py+0.5)): the row is exact,
                 * so the spec formula reduces to (1-a)*T0 + a*T1 */
                float u = xp + 0.5f;
                float t = u - 0.5f;
                float fi = floorf(t);
                float a = t - fi;
                int i0 = clampi((int)fi, 0, W - 1);
                int i1 = clampi((int)fi + 1, 0, W - 1);
                const F4 c0 = v2.col[(size_t)(int)py * W + i0], c1 = v2.col[(size_t)(int)py * W + i1];
                const F4 h0 = v2.grad[(size_t)(int)py * W + i0], h1 = v2.grad[(size_t)(int)py * W + i1];
                float oa = 1.0f - a;
                F4 a2 = f4(oa * c0.x + a * c1.x, oa * c0.y + a * c1.y, oa * c0.z + a * c1.z, 0.0f);
                F4 g2 = f4(oa * h0.x + a * h1.x, oa * h0.y + a * h1.y, oa * h0.z + a * h1.z, oa * h0.w + a * h1.w);
                float cc = (fminf(fabsf(a1.x - a2.x), k.cmax) + fminf(fabsf(a1.y - a2.y), k.cmax)) + fminf(fabsf(a1.z - a2.z), k.cmax);
                float gc = ((fminf(fabsf(g1.x - g2.x), k.gmax) + fminf(fabsf(g1.y - g2.y), k.gmax)) + fminf(fabsf(g1.z - g2.z), k.gmax)) + fminf(fabsf(g1.w - g2.w), k.gmax);
                float C = k.alpha * cc + k.one_m_alpha * gc;
                ret += w1 * C;
            }
        }
        if (wsum <= 1.1f) return 1e5f;
        return ret / wsum;
    }
    /* ARITH_FAST: mirror of the CUDA fast kernels: taps in raster order,
     * tap positions in Q31.32 fixed point (pm_fix_plane), (value, forward
     * difference) records of the other view, colour and gradient sums kept
     * apart. */
    float wsum = 0.0f, rc = 0.0f, rg = 0.0f;
    long long S0, S1, XC;
    pm_fix_plane(true, s.x, s.y, s.z, W / 2, H / 2, &S0, &S1, &XC);
    for (int dy = -P; dy <= P; ++dy) {
        int qy = cy + dy;
        if (qy < 0 || qy >= H) continue;
        const float* rrow = &v2.rec[(size_t)qy * W * 14];
        for (int dx = -P; dx <= P; ++dx) {
            int qx = cx + dx;
            if (qx < 0 || qx >= W) continue;
            const F4 a1 = v1.col[(size_t)qy * W + qx];
            const F4 g1 = v1.grad[(size_t)qy * W + qx];
            float d = (fabsf(vc.x - a1.x) + fabsf(vc.y - a1.y)) + fabsf(vc.z - a1.z);
            float w1 = pm_wexp(-d * k.prof[(size_t)(dy + P) * n + (dx + P)]);
            const long long X = XC + (long long)(qy - H / 2) * S1 + (long long)(qx - W / 2) * S0;
            const int xi = (int)(X >> 32);
            if ((unsigned)xi >= (unsigned)W) continue;
            float a = pm_fix_frac(X);
            const float* r = rrow + (size_t)xi * 14;
            float v[7];
            for (int c = 0; c < 7; ++c) v[c] = fmaf(a, r[7 + c], r[c]);
            float cc = (fminf(fabsf(a1.x - v[0]), k.cmax) + fminf(fabsf(a1.y - v[1]), k.cmax)) + fminf(fabsf(a1.z - v[2]), k.cmax);
            float gc = ((fminf(fabsf(g1.x - v[3]), k.gmax) + fminf(fabsf(g1.y - v[4]), k.gmax)) + fminf(fabsf(g1.z - v[5]), k.gmax)) + fminf(fabsf(g1.w - v[6]), k.gmax);
            rc = fmaf(w1, cc, rc);
            rg = fmaf(w1, gc, rg);
            wsum = wsum + w1;
        }
    }
    if (wsum <= 1.1f) return 1e5f;
    return fmaf(k.alpha, rc, k.one_m_alpha * rg) / wsum;
}

/* ------------------------------------------------------ preprocessing -- */
static inline float gray_at(const F4* img, int W, int H, int x, int y) {
    if (x < 0 || y < 0 || x >= W || y >= H) return 0.0f;             /* CLK_ADDRESS_CLAMP */
    F4 c = img[(size_t)y * W + x];
    return ((c.x * 0.2126f + c.y * 0.7152f) + c.z * 0.0722f) + c.w * 0.0f;
}
static void gradxy(const F4* img, int W, int H, F4* out) {             /* :785-831 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
#define B(dx_, dy_) gray_at(img, W, H, x + (dx_), y + (dy_))
            float dx = (B(1, 0) - B(-1, 0)) * 0.5f + (B(1, -1) - B(-1, -1)) * 0.25f + (B(1, 1) - B(-1, 1)) * 0.25f;
            float dy = (B(0, 1) - B(0, -1)) * 0.5f + (B(-1, 1) - B(-1, -1)) * 0.25f + (B(1, 1) - B(1, -1)) * 0.25f;
            float dxy = B(1, 1) - B(-1, -1);
            float dyx = B(-1, 1) - B(1, -1);
#undef B
            out[(size_t)y * W + x] = f4(dx, dy, dxy, dyx);
        }
}
static void edge_weight(const F4* img, int W, int H, float* out) {     /* :737-783 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float dx = gray_at(img, W, H, x + 1, y) - gray_at(img, W, H, x - 1, y);
            float gy = gray_at(img, W, H, x, y - 1);
            float dy = gy - gy;                                        /* the reference's dy (:769) */
            out[(size_t)y * W + x] = pm_exp(-3.0f * pm_pow(sqrtf(dx * dx + dy * dy), 0.8f)) + 0.0001f;
        }
}

/* ----------------------------------------------------------- view lists -- */
/* Up to 4 source x per target pixel, smallest source x first; -1 = empty.
 * Restates the scatter of pmhstereo.cl:394-400 (see the header). */
static void build_view_list(const F4* src, int W, int H, int16_t* list) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        std::vector<uint8_t> cnt(W, 0);
        int16_t* row = list + (size_t)y * W * 4;
        for (int i = 0; i < W * 4; ++i) row[i] = -1;
        for (int x = 0; x < W; ++x) {
            F4 s = src[(size_t)y * W + x];
            float v = transform_x(s, (float)x, (float)y) + 0.5f;
            if (v > -1.0f && v < (float)W) {
                int d = (int)v;
                if (cnt[d] < 4) row[d * 4 + cnt[d]++] = (int16_t)x;
            }
        }
    }
}

/* --------------------------------------------------------- init/prop -- */
struct Pass {
    const View* v1; const View* v2;
    const CostCfg* k;
    int lr, iter, rngkind; uint64_t seed;
    float depthmax, theta;
};

static inline uint32_t view_id(int lr) { return lr ? 0u : 1u; }

static void init_pass(const Pass& ps, F4* out) {                      /* :230-248 */
    const int W = ps.v1->W, H = ps.v1->H;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            Rng rng;
            uint32_t p = (uint32_t)(y * W + x);
            if (ps.rngkind == CVTPM_RNG_PHILOX) philox_init(rng, ps.seed, p, PHILOX_TAG_INIT, view_id(ps.lr));
            else mwc_init(rng, (uint64_t)p * 3u);
            F4 s = state_init(rng, (float)x, (float)y, ps.lr, 1.0f, ps.depthmax);
            s.w = cost_eval(*ps.k, *ps.v1, *ps.v2, x, y, s);
            out[(size_t)y * W + x] = s;
        }
}

/* pmhstereo_propagate_view, pmhstereo.cl:286-404, without the scatter
 * (build_view_list runs after the pass). */
/* color >= 0: only the pixels with (x + y) & 1 == color are updated, the
 * others take their old state (one half of a red/black pass). */
static void propagate_pass(const Pass& ps, const F4* old, const F4* smoothimg,
                           const int16_t* viewin, const F4* viewsrc, F4* out, uint8_t* winners, int color = -1) {
    const int W = ps.v1->W, H = ps.v1->H;
    const float dmax = ps.depthmax, theta = ps.theta;
    const int lr = ps.lr;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            if (color >= 0 && ((x + y) & 1) != color) { out[(size_t)y * W + x] = old[(size_t)y * W + x]; continue; }
            const float cx = (float)x, cy = (float)y;
            F4 sm = smoothimg[(size_t)y * W + x];                       /* :320-323 */
            float nf = fmaxf(sqrtf(sm.x * sm.x + sm.y * sm.y) + 0.001f, 1.0f);
            float smx = sm.x / nf, smy = sm.y / nf;
            F4 smooth = f4(smx, smy, sqrtf(1.0f - smx * smx - smy * smy), sm.z * dmax);
            F4 self = old[(size_t)y * W + x];                           /* :325 */
            int win = 0;
            Rng rng;                                                     /* :327 */
            uint32_t p = (uint32_t)(y * W + x);
            if (ps.rngkind == CVTPM_RNG_PHILOX) philox_init(rng, ps.seed, p, (uint32_t)ps.iter, view_id(lr));
            /* RNG_init(&rng, p + iter, ((3*3-1) + 3)*3 + 2*6): the macro body
             * `(linpos) * numdraws` takes numdraws unparenthesised, so the
             * skip distance is (p + iter)*(8 + 3)*3 + 2*6 = 33(p + iter) + 12
             * (RNG.cl:151-154, pmhstereo.cl:327). */
            else mwc_init(rng, ((uint64_t)p + (uint64_t)ps.iter) * 33u + 12u);
            auto consider = [&](F4 cand, int idx) {
                cand.w = cost_eval(*ps.k, *ps.v1, *ps.v2, x, y, cand);
                float da, db;
                smooth_distance(cand, self, smooth, cx, cy, dmax, lr, &da, &db);
                if (cand.w + theta * da <= self.w + theta * db) { self = cand; win = idx; }
            };
            int idx = 1;
            for (int py = -1; py <= 1; ++py)                             /* :330-342 */
                for (int px = -1; px <= 1; ++px) {
                    if (px == 0 && py == 0) continue;
                    int nx = clampi(x + px, 0, W - 1), ny = clampi(y + py, 0, H - 1);
                    consider(old[(size_t)ny * W + nx], idx++);
                }
            {                                                            /* :345-352 */
                F4 c = f4(1.0f - (-smooth.x / smooth.z), 0.0f - (-smooth.y / smooth.z),
                          0.0f - ((smooth.x * cx + smooth.y * cy) / smooth.z + smooth.w), 0.0f - 0.0f);
                if (!lr) c = viewprop(c);
                consider(c, 9);
            }
            for (int i = 0; i < 6; ++i) {                                /* :355-361 */
                int ox = (int)(rng_float(rng) * 7.0f + 0.5f);
                int oy = (int)(rng_float(rng) * 7.0f + 0.5f);
                int nx = clampi(x + ox, 0, W - 1), ny = clampi(y + oy, 0, H - 1);
                consider(old[(size_t)ny * W + nx], 10 + i);
            }
            consider(state_init(rng, cx, cy, lr, 2.0f, dmax), 16);      /* :364-368 */
            if (viewin) {                                                /* :372-379 */
                const int16_t* l = viewin + ((size_t)y * W + x) * 4;
                for (int i = 0; i < 4 && l[i] >= 0; ++i)
                    consider(viewprop(viewsrc[(size_t)y * W + l[i]]), 17 + i);
            }
            for (int i = 0; i < 2; ++i)                                  /* :383-389 */
                consider(state_refine(rng, self, cx, cy, dmax, lr), 21 + i);
            out[(size_t)y * W + x] = self;
            if (winners) winners[(size_t)y * W + x] = (uint8_t)win;
        }
}

/* One view pass under the parameters' schedule: Jacobi (the reference), or
 * red/black (pixels with (x + y) even from the old field, then the odd ones
 * from the field with the even ones updated; `old` ends as that field). */
static void propagate_view(const cvtpm_params* prm, const Pass& ps, std::vector<F4>& old, const F4* smoothimg,
                           const int16_t* viewin, const F4* viewsrc, std::vector<F4>& out, uint8_t* winners) {
    if (prm->schedule != CVTPM_SCHEDULE_REDBLACK) {
        propagate_pass(ps, old.data(), smoothimg, viewin, viewsrc, out.data(), winners);
        return;
    }
    propagate_pass(ps, old.data(), smoothimg, viewin, viewsrc, out.data(), winners, 0);
    old = out;
    propagate_pass(ps, old.data(), smoothimg, viewin, viewsrc, out.data(), winners, 1);
}

/* ------------------------------------------------- consistency / fill -- */
static void consistency(const F4* L, const F4* R, int W, int H, float maxdisp, float maxangle,
                        int lr, F4* out, uint8_t* valid) {             /* :428-464 */
    const float athr = maxangle / 180.0f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            F4 sl = L[(size_t)y * W + x];
            float x2 = transform_x(sl, (float)x, (float)y);
            F4 sr;
            if (x2 < 0 || x2 >= (float)W) sr = f4s(1e5f);
            else sr = R[(size_t)y * W + clampi(f2i_nan0(roundf(x2)), 0, W - 1)];
            float na[3], nb[3];
            if (lr) { to_normal(sl, na); to_normal(viewprop(sr), nb); }
            else { to_normal(sr, na); to_normal(viewprop(sl), nb); }
            float ndiff = (na[0] * nb[0] + na[1] * nb[1]) + na[2] * nb[2];
            float dm = fabsf((float)x - transform_x(sr, x2, (float)y));
            bool bad = (dm >= maxdisp) || (pm_acospi(ndiff) >= athr);
            out[(size_t)y * W + x] = bad ? f4s(0.0f) : sl;
            if (valid) valid[(size_t)y * W + x] = bad ? 0 : 1;
        }
}

/* pmhstereo_occmap, pmhstereo.cl:682-712: the test of the consistency check
 * with the angle bound fixed at 5 degrees; 1 where both views agree. */
static void occmap(const F4* L, const F4* R, int W, int H, float maxdiff, int lr, float* mask) {
    const float athr = 5.0f / 180.0f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            F4 sl = L[(size_t)y * W + x];
            float x2 = transform_x(sl, (float)x, (float)y);
            F4 sr;
            if (x2 < 0 || x2 >= (float)W) sr = f4s(1e5f);
            else sr = R[(size_t)y * W + clampi(f2i_nan0(roundf(x2)), 0, W - 1)];
            float na[3], nb[3];
            if (lr) { to_normal(sl, na); to_normal(viewprop(sr), nb); }
            else { to_normal(sr, na); to_normal(viewprop(sl), nb); }
            float ndiff = (na[0] * nb[0] + na[1] * nb[1]) + na[2] * nb[2];
            float dm = fabsf((float)x - transform_x(sr, x2, (float)y));
            bool bad = (dm >= maxdiff) || (pm_acospi(ndiff) >= athr);
            mask[(size_t)y * W + x] = bad ? 0.0f : 1.0f;
        }
}

/* pmhstereo_normal_depth, pmhstereo.cl:663-680: (n.x, n.y, d/dmax, 1). */
static void normal_depth(const F4* in, int W, int H, float depthmax, int lr, F4* out) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            F4 val = to_ref_normal_depth(in[(size_t)y * W + x], (float)x, (float)y, lr);
            out[(size_t)y * W + x] = f4(val.x, val.y, val.w / depthmax, 1.0f);
        }
}

/* nearest index to the left/right of each x whose value passes `ok` */
template <class OK>
static void row_neighbours(const F4* row, int W, OK ok, std::vector<int>& lft, std::vector<int>& rgt) {
    lft.assign(W, -1); rgt.assign(W, -1);
    int last = -1;
    for (int x = 0; x < W; ++x) { lft[x] = last; if (ok(row[x])) last = x; }
    last = -1;
    for (int x = W - 1; x >= 0; --x) { rgt[x] = last; if (ok(row[x])) last = x; }
}

static void fill_state(const F4* in, int W, int H, float depthmax, int lr, F4* out) {  /* :466-510 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        const F4* row = in + (size_t)y * W;
        std::vector<int> lft, rgt;
        row_neighbours(row, W, [](F4 v) { return !(len4(v) < 1e-1f); }, lft, rgt);
        for (int x = 0; x < W; ++x) {
            F4 st = row[x], val;
            const float cx = (float)x, cy = (float)y;
            if (len4(st) < 1e-1f) {
                F4 l = lft[x] >= 0 ? row[lft[x]] : f4s(1e5f);
                F4 r = rgt[x] >= 0 ? row[rgt[x]] : f4s(1e5f);
                l.w = fabsf(transform_x(l, cx, cy) - cx);
                r.w = fabsf(transform_x(r, cx, cy) - cx);
                val = (l.w < r.w) ? l : r;
            } else {
                val = st;
            }
            val = to_ref_normal_depth(val, cx, cy, lr);
            out[(size_t)y * W + x] = f4(val.x, val.y, val.w / depthmax, 1.0f);
        }
    }
}

static void fill_depthmap(const F4* in, int W, int H, float scale, float* out) {  /* :512-555 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        const F4* row = in + (size_t)y * W;
        std::vector<int> lft, rgt;
        row_neighbours(row, W, [](F4 v) { return !(len3(v) < 1e-1f); }, lft, rgt);
        for (int x = 0; x < W; ++x) {
            F4 st = row[x];
            const float cx = (float)x, cy = (float)y;
            float v;
            if (len3(st) < 1e-1f) {
                F4 l = lft[x] >= 0 ? row[lft[x]] : f4(-1e5f, -1e5f, -1e5f, row[0].w);
                F4 r = rgt[x] >= 0 ? row[rgt[x]] : f4(-1e5f, -1e5f, -1e5f, row[W - 1].w);
                float lw = -(transform_x(l, cx, cy) - cx);
                float rw = -(transform_x(r, cx, cy) - cx);
                v = fminf(lw, rw);
            } else {
                v = fabsf(transform_x(st, cx, cy) - cx);
            }
            out[(size_t)y * W + x] = v * scale;
        }
    }
}

static void fill_normalmap(const F4* in, int W, int H, F4* out) {      /* :557-603 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        const F4* row = in + (size_t)y * W;
        std::vector<int> lft, rgt;
        row_neighbours(row, W, [](F4 v) { return !(len3(v) < 1e-1f); }, lft, rgt);
        for (int x = 0; x < W; ++x) {
            F4 st = row[x];
            const float cx = (float)x, cy = (float)y;
            float n[3];
            if (len3(st) < 1e-1f) {
                F4 l = lft[x] >= 0 ? row[lft[x]] : f4(-1e5f, -1e5f, -1e5f, 0.0f);
                F4 r = rgt[x] >= 0 ? row[rgt[x]] : f4(-1e5f, -1e5f, -1e5f, 0.0f);
                float lw = -(transform_x(l, cx, cy) - cx);
                float rw = -(transform_x(r, cx, cy) - cx);
                to_normal((lw < rw) ? l : r, n);
            } else {
                to_normal(st, n);
            }
            out[(size_t)y * W + x] = f4(n[0], n[1], n[2], 0.0f);
        }
    }
}

/* ------------------------------------------------------------ PD ROF -- */
/* One PDHuberWeighted launch, PDHuberWeighted.cl:34-104. */
/* mask != NULL: one PDHuberWeightedInpaint launch, PDHuberWeightedInpaint.cl:
 * 34-102 — the dual projected per channel (:67) and the fidelity weight
 * lambda * mask(x, y) (:82). */
static void pd_step(F4* uout, F4* pout, const F4* last, const F4* pin, const F4* f,
                    const float* wgt, float lambda, int W, int H, const float* mask = nullptr) {
    const float SIGMA = 1.0f / sqrtf(8.0f), TAU = 1.0f / sqrtf(8.0f);
    const float THETA = 0.5f, ALPHA = 0.001f;
    auto U = [&](int x, int y) { return last[(size_t)clampi(y, 0, H - 1) * W + clampi(x, 0, W - 1)]; };
    auto pnew = [&](int qx, int qy, F4* lo, F4* hi) {                 /* :49-68 */
        bool in = qx >= 0 && qy >= 0 && qx < W && qy < H;
        float w = in ? wgt[(size_t)qy * W + qx] : 0.0f;
        F4 uq = U(qx, qy);
        F4 dx = w * (uq - U(qx + 1, qy));
        F4 dy = w * (uq - U(qx, qy + 1));
        F4 plo = in ? pin[((size_t)qy * W + qx) * 2] : f4s(0.0f);
        F4 phi = in ? pin[((size_t)qy * W + qx) * 2 + 1] : f4s(0.0f);
        float den = 1.0f + SIGMA * ALPHA / w;
        F4 l = (plo + SIGMA * dx) / f4s(den);
        F4 h = (phi + SIGMA * dy) / f4s(den);
        F4 pt = l * l + h * h;
        F4 pproj;
        if (mask) {
            pproj = f4(fmaxf(1.0f, sqrtf(pt.x)), fmaxf(1.0f, sqrtf(pt.y)), fmaxf(1.0f, sqrtf(pt.z)), fmaxf(1.0f, sqrtf(pt.w)));
        } else {
            float sxy = sqrtf(pt.x + pt.y);
            pproj = f4(fmaxf(1.0f, sxy), fmaxf(1.0f, sxy), fmaxf(1.0f, sqrtf(pt.z)), fmaxf(1.0f, sqrtf(0.0f)));
        }
        *lo = l / pproj; *hi = h / pproj;
    };
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            F4 lo, hi, lol, hil, lou, hiu;
            pnew(x, y, &lo, &hi);
            pnew(x - 1, y, &lol, &hil);
            pnew(x, y - 1, &lou, &hiu);
            F4 div = lo - lol + hi - hiu;                                 /* :73-74 */
            F4 img = f[(size_t)y * W + x];
            F4 uc = last[(size_t)y * W + x];
            float wc = wgt[(size_t)y * W + x];
            F4 lam = f4s(mask ? lambda * mask[(size_t)y * W + x] : lambda);
            F4 un = (uc + TAU * (lam * img - wc * div)) / (f4s(1.0f) + TAU * lam);  /* :76 */
            un = un + THETA * (un - uc);
            un.w = 1.0f;
            uout[(size_t)y * W + x] = un;
            pout[((size_t)y * W + x) * 2] = lo;
            pout[((size_t)y * W + x) * 2 + 1] = hi;
        }
}

/* PDROF::apply, cvt/gfx/PDROF.h:50-96 (mask == NULL), and
 * PDROFInpaint::apply, cvt/gfx/PDROFInpaint.h:50-98 (mask: the occlusion
 * map's x channel).  `output` is read as the warm start. */
static void pd_apply(F4* output, const F4* input, const float* wgt, float lambda, int iters, int W, int H,
                     const float* mask = nullptr) {
    size_t n = (size_t)W * H;
    std::vector<F4> tmp(input, input + n);
    std::vector<F4> p1(2 * n, f4s(0.0f)), p2(2 * n, f4s(0.0f));
    F4* img[2] = {tmp.data(), output};
    F4* pp[2] = {p1.data(), p2.data()};
    int swap = 0;
    for (int i = 0; i < iters; ++i) {
        swap = i & 1;
        pd_step(img[swap], pp[swap], img[1 - swap], pp[1 - swap], input, wgt, lambda, W, H, mask);
    }
    if (!swap) pd_step(img[1], pp[1], img[0], pp[0], input, wgt, lambda, W, H, mask);
}

static float smoothstep01(float x) {                                   /* cvt/math/Math.h:88-92 */
    float t = (x < 0.0f) ? 0.0f : (x > 1.0f) ? 1.0f : x;
    return t * t * (3.0f - 2.0f * t);
}

static bool check_params(const cvtpm_params* p) {
    return p && p->patchsize >= 1 && p->patchsize <= 31 && p->depthmax > 0.0f && p->iterations >= 1 &&
           p->pd_iterations >= 0 && (p->arith == CVTPM_ARITH_EXACT || p->arith == CVTPM_ARITH_FAST) &&
           (p->rng == CVTPM_RNG_MWC64X || p->rng == CVTPM_RNG_PHILOX);
}

struct Views {
    std::vector<F4> gl, gr;
    View L, R;
};

static void make_views(const float* left, const float* right, int W, int H, int arith, Views& v) {
    size_t n = (size_t)W * H;
    v.gl.resize(n); v.gr.resize(n);
    gradxy((const F4*)left, W, H, v.gl.data());
    gradxy((const F4*)right, W, H, v.gr.data());
    v.L.W = v.R.W = W; v.L.H = v.R.H = H;
    v.L.col = (const F4*)left; v.R.col = (const F4*)right;
    v.L.grad = v.gl.data(); v.R.grad = v.gr.data();
    if (arith == CVTPM_ARITH_FAST) { build_records(v.L); build_records(v.R); }
}

}  // namespace

/* ----------------------------------------------------------- FP64 -- */
/* The aggregated cost of pmhstereo.cl:170-228 and its adjoint, in double
 * precision on double images: gradients (:785-831), bilateral weights (exp),
 * the spatial profile (smoothstep), the sample position x' = s0*qx + s1*qy +
 * s2 and the linear interpolation along the row.  `edge` flags pixels with a
 * tap whose x' lies within `eps` of the validity bounds 0 and W, or whose
 * weight sum lies within 1e-6 of the 1.1 threshold (there the cost jumps). */
struct D4 { double x, y, z, w; };
struct ImgD {
    int W, H;
    const double* c;            /* RGBA, W*H*4 */
    std::vector<D4> g;          /* gradients */
    D4 col(int x, int y) const { const double* q = c + ((size_t)y * W + x) * 4; return {q[0], q[1], q[2], q[3]}; }
};
/* The gradient stencil of pmhstereo_gradxy as (dx, dy, component, weight)
 * terms on the grey image B (zero outside): G.comp(x, y) += weight * B(x+dx, y+dy). */
struct GradTerm { int dx, dy, comp; double w; };
static const GradTerm kGradTerms[] = {
    {1, 0, 0, 0.5}, {-1, 0, 0, -0.5}, {1, -1, 0, 0.25}, {-1, -1, 0, -0.25}, {1, 1, 0, 0.25}, {-1, 1, 0, -0.25},
    {0, 1, 1, 0.5}, {0, -1, 1, -0.5}, {-1, 1, 1, 0.25}, {-1, -1, 1, -0.25}, {1, 1, 1, 0.25}, {1, -1, 1, -0.25},
    {1, 1, 2, 1.0}, {-1, -1, 2, -1.0},
    {-1, 1, 3, 1.0}, {1, -1, 3, -1.0},
};
static const double kGrey[3] = {0.2126, 0.7152, 0.0722};
static void grad_f64(ImgD& im) {
    const int W = im.W, H = im.H;
    im.g.assign((size_t)W * H, D4{0, 0, 0, 0});
    auto B = [&](int x, int y) -> double {
        if (x < 0 || y < 0 || x >= W || y >= H) return 0.0;
        const double* q = im.c + ((size_t)y * W + x) * 4;
        return q[0] * kGrey[0] + q[1] * kGrey[1] + q[2] * kGrey[2];
    };
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double v[4] = {0, 0, 0, 0};
            for (const GradTerm& t : kGradTerms) v[t.comp] += t.w * B(x + t.dx, y + t.dy);
            im.g[(size_t)y * W + x] = D4{v[0], v[1], v[2], v[3]};
        }
}
/* Adjoint of grad_f64: dimg += d(grey)/d(RGB) * sum of the transposed stencil of dg. */
static void grad_f64_adjoint(const std::vector<D4>& dg, int W, int H, double* dimg) {
    for (int v = 0; v < H; ++v)
        for (int u = 0; u < W; ++u) {
            double dB = 0.0;
            for (const GradTerm& t : kGradTerms) {
                const int x = u - t.dx, y = v - t.dy;
                if (x < 0 || y < 0 || x >= W || y >= H) continue;
                const D4& q = dg[(size_t)y * W + x];
                const double comp = t.comp == 0 ? q.x : t.comp == 1 ? q.y : t.comp == 2 ? q.z : q.w;
                dB += t.w * comp;
            }
            double* o = dimg + ((size_t)v * W + u) * 4;
            for (int ch = 0; ch < 3; ++ch) o[ch] += kGrey[ch] * dB;
        }
}
static double profile_f64(int dx, int dy, double cw, int profile) {
    if (profile == CVTPM_PROFILE_CONSTANT) return cw;
    double len = std::sqrt((double)dx * dx + (double)dy * dy);
    double t = std::min(std::max(len / 26.0, 0.0), 1.0);
    return t * t * (3.0 - 2.0 * t) * 1.5 * cw + 5.0;
}
static inline double sgn(double v) { return (v > 0) - (v < 0); }

/* One tap of the window of (cx, cy): everything the cost and its adjoint need. */
struct TapF64 {
    bool valid;
    double w, prof, c, a, xp;
    int i0, i1, qx, qy;
    double e[3], eg[4];          /* image-1 minus interpolated image-2 (colour, gradient) */
    double D[3], Dg[4];          /* d(interpolated)/dx' */
    double dsign[3];             /* sign(I1(c) - I1(q)) per channel */
};
static void tap_f64(const cvtpm_params* prm, const ImgD& i1, const ImgD& i2, int cx, int cy, int dx, int dy,
                    const double s[3], TapF64& t) {
    const int W = i1.W;
    t.qx = cx + dx; t.qy = cy + dy;
    const D4 vc = i1.col(cx, cy), a1 = i1.col(t.qx, t.qy);
    const D4& b1 = i1.g[(size_t)t.qy * W + t.qx];
    const double dc[3] = {vc.x - a1.x, vc.y - a1.y, vc.z - a1.z};
    double d = 0.0;
    for (int ch = 0; ch < 3; ++ch) { d += std::fabs(dc[ch]); t.dsign[ch] = sgn(dc[ch]); }
    t.prof = profile_f64(dx, dy, prm->color_weight, prm->weight_profile);
    t.w = std::exp(-d * t.prof);
    t.xp = s[0] * t.qx + s[1] * t.qy + s[2];
    t.valid = t.xp >= 0.0 && t.xp < (double)W;
    if (!t.valid) return;
    const double fi = std::floor(t.xp);
    t.a = t.xp - fi;
    t.i0 = clampi((int)fi, 0, W - 1);
    t.i1 = clampi((int)fi + 1, 0, W - 1);
    const D4 p0 = i2.col(t.i0, t.qy), p1 = i2.col(t.i1, t.qy);
    const D4& h0 = i2.g[(size_t)t.qy * W + t.i0];
    const D4& h1 = i2.g[(size_t)t.qy * W + t.i1];
    const double T0[7] = {p0.x, p0.y, p0.z, h0.x, h0.y, h0.z, h0.w};
    const double T1[7] = {p1.x, p1.y, p1.z, h1.x, h1.y, h1.z, h1.w};
    const double A[7] = {a1.x, a1.y, a1.z, b1.x, b1.y, b1.z, b1.w};
    double cc = 0.0, gc = 0.0;
    for (int k = 0; k < 7; ++k) {
        const double v = (1.0 - t.a) * T0[k] + t.a * T1[k];
        const double e = A[k] - v;
        if (k < 3) { t.e[k] = e; t.D[k] = T1[k] - T0[k]; cc += std::min(std::fabs(e), (double)prm->color_maxdiff); }
        else { t.eg[k - 3] = e; t.Dg[k - 3] = T1[k] - T0[k]; gc += std::min(std::fabs(e), (double)prm->grad_maxdiff); }
    }
    t.c = prm->color_alpha * cc + (1.0 - prm->color_alpha) * gc;
}

/* States (s0, s1, s2) of plane (a, b, c) of view lr: x' = x - d (lr = 1) or
 * x + d (lr = 0), d = a*x + b*y + c; ds/d(a, b, c) = -1 (lr = 1) or +1. */
static inline void plane_state(const double* pl, int lr, double s[3]) {
    if (lr) { s[0] = 1.0 - pl[0]; s[1] = -pl[1]; s[2] = -pl[2]; }
    else { s[0] = 1.0 + pl[0]; s[1] = pl[1]; s[2] = pl[2]; }
}

/* Branch signature of one tap: validity, interpolation cell, and the sign
 * and truncation of every |.| term.  Two evaluations with equal signatures
 * over all taps lie on one smooth piece of the cost. */
static inline uint64_t sig_mix(uint64_t h, uint64_t v) { return (h ^ v) * 0x100000001B3ull; }
static uint64_t tap_signature(const cvtpm_params* prm, const TapF64& t, uint64_t h) {
    h = sig_mix(h, t.valid ? 1 : 2);
    for (int ch = 0; ch < 3; ++ch) h = sig_mix(h, (uint64_t)(sgn(t.dsign[ch]) + 1));
    if (!t.valid) return h;
    h = sig_mix(h, (uint64_t)(int64_t)t.i0 + 7);
    for (int ch = 0; ch < 3; ++ch)
        h = sig_mix(h, (uint64_t)(sgn(t.e[ch]) + 1) * 2 + (std::fabs(t.e[ch]) < prm->color_maxdiff));
    for (int k = 0; k < 4; ++k)
        h = sig_mix(h, (uint64_t)(sgn(t.eg[k]) + 1) * 2 + (std::fabs(t.eg[k]) < prm->grad_maxdiff));
    return h;
}

static double cost_f64(const cvtpm_params* prm, const ImgD& i1, const ImgD& i2, int cx, int cy,
                       const double s[3], double eps, bool* edge, double* wsum, uint64_t* sig = nullptr) {
    *edge = false;
    uint64_t h = 0xCBF29CE484222325ull;
    if (!std::isfinite(s[0]) || !std::isfinite(s[1]) || !std::isfinite(s[2])) {
        *wsum = 0;
        if (sig) *sig = h;
        return 1e5;
    }
    const int P = prm->patchsize, W = i1.W, H = i1.H;
    double ws = 0.0, ret = 0.0;
    TapF64 t;
    for (int dy = -P; dy <= P; ++dy)
        for (int dx = -P; dx <= P; ++dx) {
            if (cx + dx < 0 || cy + dy < 0 || cx + dx >= W || cy + dy >= H) continue;
            tap_f64(prm, i1, i2, cx, cy, dx, dy, s, t);
            if (sig) h = tap_signature(prm, t, h);
            if (std::fabs(t.xp) < eps || std::fabs(t.xp - W) < eps) *edge = true;
            if (!t.valid) continue;
            ws += t.w;
            ret += t.w * t.c;
        }
    *wsum = ws;
    if (sig) *sig = sig_mix(h, ws > 1.1 ? 3 : 4);
    if (std::fabs(ws - 1.1) < 1e-6) *edge = true;
    if (ws <= 1.1) return 1e5;
    return ret / ws;
}

/* Cost and adjoint of one pixel.  L = sum_p dcost_p * C_p; C = R / S with
 * S = sum w_t, R = sum w_t c_t over valid taps:
 *   dL/dc_t = g w_t / S,  dL/dw_t = g (c_t - C) / S,  dw_t/dd_t = -prof_t w_t,
 *   dc_t/dx' = -(alpha sum_ch s_ch D_ch + (1 - alpha) sum_k s_k Dg_k),
 * s = sign(e) where |e| is below its truncation (0 above), D = T1 - T0.
 * Validity changes and the 1.1 threshold are measure-zero and not
 * differentiated; a pixel with cost 1e5 has zero gradient. */
/* Entries an evaluation in another precision may differentiate on the other
 * side of a kink: taps within `keps` of a kink mark what their slope reaches
 * (the pixel's plane; the image-1 pixel q and the image-2 columns i0, i1,
 * with the 3x3 stencil of the gradient images where a gradient term is
 * involved); a tap near the validity bounds or a weight sum near 1.1 marks
 * everything the pixel's window reaches. */
struct Ambiguity {
    double keps;
    int W, H;
    uint8_t *pl, *im1, *im2;
    void mark(uint8_t* m, int x, int y, int r) const {
        if (!m) return;
        for (int yy = y - r; yy <= y + r; ++yy)
            for (int xx = x - r; xx <= x + r; ++xx)
                if (xx >= 0 && yy >= 0 && xx < W && yy < H) m[(size_t)yy * W + xx] = 1;
    }
};

static double adjoint_f64(const cvtpm_params* prm, const ImgD& i1, const ImgD& i2, int cx, int cy, const double s[3],
                          double g, double gs[3], double* dimg1, double* dimg2, std::vector<D4>& dg1,
                          std::vector<D4>& dg2, const Ambiguity* amb) {
    bool edge;
    double S;
    const double keps = amb ? amb->keps : 0.0;
    const double C = cost_f64(prm, i1, i2, cx, cy, s, keps, &edge, &S);
    gs[0] = gs[1] = gs[2] = 0.0;
    const int P = prm->patchsize, W = i1.W, H = i1.H;
    TapF64 t;
    if (amb && edge && g != 0.0) {             /* S may change: everything the window reaches */
        amb->mark(amb->pl, cx, cy, 0);
        for (int dy = -P; dy <= P; ++dy)
            for (int dx = -P; dx <= P; ++dx) {
                if (cx + dx < 0 || cy + dy < 0 || cx + dx >= W || cy + dy >= H) continue;
                tap_f64(prm, i1, i2, cx, cy, dx, dy, s, t);
                amb->mark(amb->im1, t.qx, t.qy, 1);
                if (t.valid) { amb->mark(amb->im2, t.i0, t.qy, 1); amb->mark(amb->im2, t.i1, t.qy, 1); }
            }
    }
    if (!(S > 1.1) || g == 0.0) return C;
    const double al = prm->color_alpha, cm = prm->color_maxdiff, gm = prm->grad_maxdiff;
    const double u = g / S;
    for (int dy = -P; dy <= P; ++dy)
        for (int dx = -P; dx <= P; ++dx) {
            if (cx + dx < 0 || cy + dy < 0 || cx + dx >= W || cy + dy >= H) continue;
            tap_f64(prm, i1, i2, cx, cy, dx, dy, s, t);
            if (!t.valid) continue;
            if (amb) {
                bool kc = false, kg = false;
                for (int ch = 0; ch < 3; ++ch)
                    kc |= std::fabs(t.e[ch]) < keps || std::fabs(std::fabs(t.e[ch]) - cm) < keps;
                for (int k = 0; k < 4; ++k)
                    kg |= std::fabs(t.eg[k]) < keps || std::fabs(std::fabs(t.eg[k]) - gm) < keps;
                const bool kx = std::fabs(t.xp - std::nearbyint(t.xp)) < keps;
                if (kc || kg || kx) amb->mark(amb->pl, cx, cy, 0);
                if (kc) { amb->mark(amb->im1, t.qx, t.qy, 0); amb->mark(amb->im2, t.i0, t.qy, 0); amb->mark(amb->im2, t.i1, t.qy, 0); }
                if (kg) { amb->mark(amb->im1, t.qx, t.qy, 1); amb->mark(amb->im2, t.i0, t.qy, 1); amb->mark(amb->im2, t.i1, t.qy, 1); }
                if (kx) for (int c = t.i0 - 1; c <= t.i0 + 2; ++c) amb->mark(amb->im2, c, t.qy, 1);
            }
            const double gc = u * t.w;                       /* dL/dc_t */
            const double gd = u * (t.c - C) * (-t.prof * t.w); /* dL/dd_t */
            double sc[3], sg[4], gx = 0.0;
            for (int ch = 0; ch < 3; ++ch) {
                sc[ch] = std::fabs(t.e[ch]) < cm ? sgn(t.e[ch]) : 0.0;
                gx -= al * sc[ch] * t.D[ch];
            }
            for (int k = 0; k < 4; ++k) {
                sg[k] = std::fabs(t.eg[k]) < gm ? sgn(t.eg[k]) : 0.0;
                gx -= (1.0 - al) * sg[k] * t.Dg[k];
            }
            gx *= gc;
            gs[0] += gx * t.qx; gs[1] += gx * t.qy; gs[2] += gx;
            double* dc = dimg1 + ((size_t)cy * W + cx) * 4;
            double* dq = dimg1 + ((size_t)t.qy * W + t.qx) * 4;
            double* d0 = dimg2 + ((size_t)t.qy * W + t.i0) * 4;
            double* d1 = dimg2 + ((size_t)t.qy * W + t.i1) * 4;
            for (int ch = 0; ch < 3; ++ch) {
                dc[ch] += gd * t.dsign[ch];
                dq[ch] += -gd * t.dsign[ch] + gc * al * sc[ch];
                d0[ch] -= gc * al * sc[ch] * (1.0 - t.a);
                d1[ch] -= gc * al * sc[ch] * t.a;
            }
            D4& q1 = dg1[(size_t)t.qy * W + t.qx];
            D4& r0 = dg2[(size_t)t.qy * W + t.i0];
            D4& r1 = dg2[(size_t)t.qy * W + t.i1];
            double* q1v[4] = {&q1.x, &q1.y, &q1.z, &q1.w};
            double* r0v[4] = {&r0.x, &r0.y, &r0.z, &r0.w};
            double* r1v[4] = {&r1.x, &r1.y, &r1.z, &r1.w};
            for (int k = 0; k < 4; ++k) {
                const double v = gc * (1.0 - al) * sg[k];
                *q1v[k] += v;
                *r0v[k] -= v * (1.0 - t.a);
                *r1v[k] -= v * t.a;
            }
        }
    return C;
}

/* ===================================================== extern "C" API == */
extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_gradxy(const float* img, int W, int H, float* out) { gradxy((const F4*)img, W, H, (F4*)out); }
void orc_edge_weight(const float* img, int W, int H, float* out) { edge_weight((const F4*)img, W, H, out); }

float orc_exp(float x) { return pm_exp(x); }
float orc_wexp(float x) { return pm_wexp(x); }
float orc_pow(float x, float y) { return pm_pow(x, y); }
float orc_acospi(float x) { return pm_acospi(x); }
void orc_exp_array(const float* x, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = pm_exp(x[i]); }
void orc_wexp_array(const float* x, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = pm_wexp(x[i]); }
void orc_pow_array(const float* x, float e, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = pm_pow(x[i], e); }
void orc_acospi_array(const float* x, float* y, long n) { for (long i = 0; i < n; ++i) y[i] = pm_acospi(x[i]); }

uint64_t orc_mwc_mulmod_serial(uint64_t a, uint64_t b) { return mwc_mulmod_serial(a, b, MWC_M); }
uint64_t orc_mwc_mulmod(uint64_t a, uint64_t b) { return mwc_mulmod(a, b, MWC_M); }
/* n consecutive floats of the stream RNG_init(linpos, numdraws) */
void orc_mwc_stream(uint64_t distance, int n, float* out) {
    Rng r; mwc_init(r, distance);
    for (int i = 0; i < n; ++i) out[i] = mwc_float(r);
}
/* state (x, c) after skipping `distance` steps */
void orc_mwc_state(uint64_t distance, uint32_t* x, uint32_t* c) {
    Rng r; mwc_init(r, distance); *x = r.x; *c = r.c;
}
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox10(ctr, key, out); }
void orc_philox_stream(uint64_t seed, uint32_t pixel, uint32_t tag, uint32_t view, int n, float* out) {
    Rng r; philox_init(r, seed, pixel, tag, view);
    for (int i = 0; i < n; ++i) out[i] = philox_float(r);
}

/* Aggregated cost of every pixel for a fixed state field (float4 per pixel). */
int orc_cost_field(const cvtpm_params* prm, const float* img1, const float* img2, int W, int H,
                   const float* states, float* cost) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    Views v;
    make_views(img1, img2, W, H, prm->arith, v);
    CostCfg k = make_cost_cfg(prm);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float* s = states + ((size_t)y * W + x) * 4;
            cost[(size_t)y * W + x] = cost_eval(k, v.L, v.R, x, y, f4(s[0], s[1], s[2], s[3]));
        }
    return CVTPM_OK;
}

/* pmhstereo_init for view lr (img1 = that view). */
int orc_init(const cvtpm_params* prm, const float* img1, const float* img2, int W, int H, int lr, float* out) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    Views v;
    make_views(img1, img2, W, H, prm->arith, v);
    CostCfg k = make_cost_cfg(prm);
    Pass ps = {&v.L, &v.R, &k, lr, 0, prm->rng, prm->seed, prm->depthmax, 0.0f};
    init_pass(ps, (F4*)out);
    return CVTPM_OK;
}

/* One propagation pass of view lr (img1 = that view) with optional view list
 * (W*H*4 int16, sources in viewsrc, the other view's states). */
int orc_propagate(const cvtpm_params* prm, const float* img1, const float* img2, int W, int H, int lr,
                  int iter, float theta, const float* old, const float* smooth,
                  const int16_t* viewin, const float* viewsrc, float* out, uint8_t* winners) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    Views v;
    make_views(img1, img2, W, H, prm->arith, v);
    CostCfg k = make_cost_cfg(prm);
    Pass ps = {&v.L, &v.R, &k, lr, iter, prm->rng, prm->seed, prm->depthmax, theta};
    propagate_pass(ps, (const F4*)old, (const F4*)smooth, viewin, (const F4*)viewsrc, (F4*)out, winners);
    return CVTPM_OK;
}

void orc_view_list(const float* src, int W, int H, int16_t* list) { build_view_list((const F4*)src, W, H, list); }

void orc_consistency(const float* L, const float* R, int W, int H, float maxdisp, float maxangle, int lr,
                     float* out, uint8_t* valid) {
    consistency((const F4*)L, (const F4*)R, W, H, maxdisp, maxangle, lr, (F4*)out, valid);
}
void orc_fill_state(const float* in, int W, int H, float depthmax, int lr, float* out) {
    fill_state((const F4*)in, W, H, depthmax, lr, (F4*)out);
}
void orc_fill_depthmap(const float* in, int W, int H, float scale, float* out) {
    fill_depthmap((const F4*)in, W, H, scale, out);
}
void orc_fill_normalmap(const float* in, int W, int H, float* out) {
    fill_normalmap((const F4*)in, W, H, (F4*)out);
}
void orc_pd_step(float* uout, float* pout, const float* last, const float* pin, const float* f,
                 const float* wgt, float lambda, int W, int H) {
    pd_step((F4*)uout, (F4*)pout, (const F4*)last, (const F4*)pin, (const F4*)f, wgt, lambda, W, H);
}
void orc_pd_apply(float* output, const float* input, const float* wgt, float lambda, int iters, int W, int H) {
    pd_apply((F4*)output, (const F4*)input, wgt, lambda, iters, W, H);
}

/* PMHuberStereo::depthMap, PMHuberStereo.cpp:64-291. */
int orc_depthmap(const cvtpm_params* prm, const float* left, const float* right, int W, int H,
                 float* dmap, float* normalmap, float* states_out, uint8_t* winners, uint8_t* valid) {
    if (!check_params(prm) || !left || !right || !dmap || W < 1 || H < 1) return CVTPM_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)W * H;
    const int N = prm->iterations;
    const float dmax = prm->depthmax;
    const float dscale = prm->dscale <= 0.0f ? 1.0f / dmax : prm->dscale;
    Views v;
    make_views(left, right, W, H, prm->arith, v);
    CostCfg k = make_cost_cfg(prm);
    std::vector<float> wl(n), wr(n);                                   /* :99-106 */
    edge_weight((const F4*)left, W, H, wl.data());
    edge_weight((const F4*)right, W, H, wr.data());
    std::vector<F4> smL(n, f4s(0.0f)), smR(n, f4s(0.0f));              /* :108-113 */
    std::vector<F4> SL[2] = {std::vector<F4>(n), std::vector<F4>(n)};
    std::vector<F4> SR[2] = {std::vector<F4>(n), std::vector<F4>(n)};
    std::vector<F4> tmp(n), tmp2(n);
    std::vector<int16_t> list1(n * 4, -1), list2(n * 4, -1);
    std::vector<uint8_t> winL(n, 0), winR(n, 0);
    Pass pl = {&v.L, &v.R, &k, 1, 0, prm->rng, prm->seed, dmax, 0.0f};
    Pass pr = {&v.R, &v.L, &k, 0, 0, prm->rng, prm->seed, dmax, 0.0f};
    init_pass(pl, SL[0].data());                                       /* :124-143 */
    init_pass(pr, SR[0].data());
    float theta = 0.0f;
    for (int iter = 0; iter < N; ++iter) {                             /* :151-266 */
        int swap = iter & 1;
        pl.iter = pr.iter = iter;
        pl.theta = pr.theta = theta;
        propagate_view(prm, pl, SL[swap], smL.data(), list2.data(), SR[swap].data(), SL[1 - swap], winL.data());
        build_view_list(SL[1 - swap].data(), W, H, list1.data());
        propagate_view(prm, pr, SR[swap], smR.data(), list1.data(), SL[1 - swap].data(), SR[1 - swap], winR.data());
        build_view_list(SR[1 - swap].data(), W, H, list2.data());
        float lambda = theta * prm->thetascale + 5.0f;
        consistency(SL[1 - swap].data(), SR[1 - swap].data(), W, H, prm->maxdispdiff, prm->maxanglediff, 1, tmp.data(), nullptr);
        fill_state(tmp.data(), W, H, dmax, 1, tmp2.data());
        pd_apply(smL.data(), tmp2.data(), wl.data(), lambda, prm->pd_iterations, W, H);
        consistency(SR[1 - swap].data(), SL[1 - swap].data(), W, H, prm->maxdispdiff, prm->maxanglediff, 0, tmp.data(), nullptr);
        fill_state(tmp.data(), W, H, dmax, 0, tmp2.data());
        pd_apply(smR.data(), tmp2.data(), wr.data(), lambda, prm->pd_iterations, W, H);
        if (iter >= 5) theta = smoothstep01(((float)iter - 5.0f) / ((float)N - 5.0f)) * 1.0f;
    }
    int fin = 1 - ((N - 1) & 1);
    consistency(SL[fin].data(), SR[fin].data(), W, H, prm->maxdispdiff, prm->maxanglediff, 1, tmp.data(), valid);
    fill_depthmap(tmp.data(), W, H, dscale, dmap);
    if (normalmap) fill_normalmap(tmp.data(), W, H, (F4*)normalmap);
    if (states_out) {
        memcpy(states_out, SL[fin].data(), n * sizeof(F4));
        memcpy(states_out + 4 * n, SR[fin].data(), n * sizeof(F4));
    }
    if (winners) { memcpy(winners, winL.data(), n); memcpy(winners + n, winR.data(), n); }
    return CVTPM_OK;
}

/* PMHuberStereo::depthMapInpaint, PMHuberStereo.cpp:293-506: the depthMap
 * schedule with the occlusion-masked smoother (PDROFInpaint, 100 steps,
 * lambda = 20*theta + 5), theta ramped from iteration 4, the final check on
 * state buffer 1 (the reference reads clmatches[1] whatever the iteration
 * count, :491-496) with 1 px / 5 degrees, and the disparity in pixels
 * (scale 1, :503).  states_out: the last propagation outputs. */
int orc_depthmap_inpaint(const cvtpm_params* prm, const float* left, const float* right, int W, int H,
                         float* dmap, float* states_out, uint8_t* winners, uint8_t* valid) {
    if (!check_params(prm) || !left || !right || !dmap || W < 1 || H < 1) return CVTPM_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)W * H;
    const int N = prm->iterations;
    const float dmax = prm->depthmax;
    Views v;
    make_views(left, right, W, H, prm->arith, v);
    CostCfg k = make_cost_cfg(prm);
    std::vector<float> wl(n), wr(n), mask(n);
    edge_weight((const F4*)left, W, H, wl.data());
    edge_weight((const F4*)right, W, H, wr.data());
    std::vector<F4> smL(n, f4s(0.0f)), smR(n, f4s(0.0f));
    std::vector<F4> SL[2] = {std::vector<F4>(n), std::vector<F4>(n)};
    std::vector<F4> SR[2] = {std::vector<F4>(n), std::vector<F4>(n)};
    std::vector<F4> tmp(n), tmp2(n);
    std::vector<int16_t> list1(n * 4, -1), list2(n * 4, -1);
    std::vector<uint8_t> winL(n, 0), winR(n, 0);
    Pass pl = {&v.L, &v.R, &k, 1, 0, prm->rng, prm->seed, dmax, 0.0f};
    Pass pr = {&v.R, &v.L, &k, 0, 0, prm->rng, prm->seed, dmax, 0.0f};
    init_pass(pl, SL[0].data());                                       /* :345-363 */
    init_pass(pr, SR[0].data());
    float theta = 0.0f;
    for (int iter = 0; iter < N; ++iter) {                             /* :371-482 */
        int swap = iter & 1;
        pl.iter = pr.iter = iter;
        pl.theta = pr.theta = theta;
        propagate_view(prm, pl, SL[swap], smL.data(), list2.data(), SR[swap].data(), SL[1 - swap], winL.data());
        build_view_list(SL[1 - swap].data(), W, H, list1.data());
        propagate_view(prm, pr, SR[swap], smR.data(), list1.data(), SL[1 - swap].data(), SR[1 - swap], winR.data());
        build_view_list(SR[1 - swap].data(), W, H, list2.data());
        const float lambda = theta * 20.0f + 5.0f;
        occmap(SL[1 - swap].data(), SR[1 - swap].data(), W, H, 0.5f, 1, mask.data());
        normal_depth(SL[1 - swap].data(), W, H, dmax, 1, tmp2.data());
        pd_apply(smL.data(), tmp2.data(), wl.data(), lambda, 100, W, H, mask.data());
        occmap(SR[1 - swap].data(), SL[1 - swap].data(), W, H, 0.5f, 0, mask.data());
        normal_depth(SR[1 - swap].data(), W, H, dmax, 0, tmp2.data());
        pd_apply(smR.data(), tmp2.data(), wr.data(), lambda, 100, W, H, mask.data());
        if (iter >= 4) theta = smoothstep01(((float)iter - 4.0f) / ((float)N - 4.0f)) * 1.0f;
    }
    consistency(SL[1].data(), SR[1].data(), W, H, 1.0f, 5.0f, 1, tmp.data(), valid);
    fill_depthmap(tmp.data(), W, H, 1.0f, dmap);
    const int fin = 1 - ((N - 1) & 1);
    if (states_out) {
        memcpy(states_out, SL[fin].data(), n * sizeof(F4));
        memcpy(states_out + 4 * n, SR[fin].data(), n * sizeof(F4));
    }
    if (winners) { memcpy(winners, winL.data(), n); memcpy(winners + n, winR.data(), n); }
    return CVTPM_OK;
}

void orc_occmap(const float* L, const float* R, int W, int H, float maxdiff, int lr, float* mask) {
    occmap((const F4*)L, (const F4*)R, W, H, maxdiff, lr, mask);
}
void orc_normal_depth(const float* in, int W, int H, float depthmax, int lr, float* out) {
    normal_depth((const F4*)in, W, H, depthmax, lr, (F4*)out);
}
void orc_pd_apply_inpaint(float* output, const float* input, const float* wgt, const float* mask, float lambda,
                          int iters, int W, int H) {
    pd_apply((F4*)output, (const F4*)input, wgt, lambda, iters, W, H, mask);
}

/* FP64 cost of a fixed state field (FP32 images and states, widened);
 * edge[p] = 1 where a tap sits within eps of the validity bounds or the
 * weight sum within 1e-6 of 1.1. */
int orc_cost_field_f64(const cvtpm_params* prm, const float* img1, const float* img2, int W, int H,
                       const float* states, double eps, double* cost, uint8_t* edge) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)W * H;
    std::vector<double> c1(img1, img1 + n * 4), c2(img2, img2 + n * 4);
    ImgD i1{W, H, c1.data(), {}}, i2{W, H, c2.data(), {}};
    grad_f64(i1);
    grad_f64(i2);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float* st = states + ((size_t)y * W + x) * 4;
            const double s[3] = {st[0], st[1], st[2]};
            bool e = false;
            double ws;
            cost[(size_t)y * W + x] = cost_f64(prm, i1, i2, x, y, s, eps, &e, &ws);
            if (edge) edge[(size_t)y * W + x] = e ? 1 : 0;
        }
    return CVTPM_OK;
}

/* FP64 cost of per-pixel planes (a, b, c, unused) of view lr on double
 * images (RGBA, W*H*4); sig (optional) receives each pixel's branch
 * signature. */
int orc_cost_planes_f64(const cvtpm_params* prm, const double* img1, const double* img2, int W, int H,
                        const double* planes, int lr, double eps, double* cost, uint8_t* edge, uint64_t* sig) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    ImgD i1{W, H, img1, {}}, i2{W, H, img2, {}};
    grad_f64(i1);
    grad_f64(i2);
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            double s[3];
            plane_state(planes + ((size_t)y * W + x) * 4, lr, s);
            bool e = false;
            double ws;
            cost[(size_t)y * W + x] = cost_f64(prm, i1, i2, x, y, s, eps, &e, &ws, sig ? sig + (size_t)y * W + x : nullptr);
            if (edge) edge[(size_t)y * W + x] = e ? 1 : 0;
        }
    return CVTPM_OK;
}

/* FP64 adjoint: given dcost = dL/dC per pixel, the cost and dL/d(planes),
 * dL/d(img1), dL/d(img2) (alpha channel 0).  Sequential (the image
 * gradients are scattered).  With kink_eps > 0 the amb_* masks (optional,
 * W*H) flag the entries a tap within kink_eps of a kink reaches. */
int orc_cost_adjoint_f64(const cvtpm_params* prm, const double* img1, const double* img2, int W, int H,
                         const double* planes, int lr, const double* dcost, double* cost, double* dplanes,
                         double* dimg1, double* dimg2, double kink_eps, uint8_t* amb_planes, uint8_t* amb_img1,
                         uint8_t* amb_img2) {
    if (!check_params(prm)) return CVTPM_ERR_INVALID_ARGUMENT;
    ImgD i1{W, H, img1, {}}, i2{W, H, img2, {}};
    grad_f64(i1);
    grad_f64(i2);
    const size_t n = (size_t)W * H;
    std::fill(dimg1, dimg1 + n * 4, 0.0);
    std::fill(dimg2, dimg2 + n * 4, 0.0);
    std::vector<D4> dg1(n, D4{0, 0, 0, 0}), dg2(n, D4{0, 0, 0, 0});
    const double ds = lr ? -1.0 : 1.0;
    Ambiguity amb{kink_eps, W, H, amb_planes, amb_img1, amb_img2};
    for (uint8_t* m : {amb_planes, amb_img1, amb_img2})
        if (m) std::fill(m, m + n, (uint8_t)0);
    const bool track = kink_eps > 0.0 && (amb_planes || amb_img1 || amb_img2);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * W + x;
            double s[3], gs[3];
            plane_state(planes + o * 4, lr, s);
            cost[o] = adjoint_f64(prm, i1, i2, x, y, s, dcost[o], gs, dimg1, dimg2, dg1, dg2, track ? &amb : nullptr);
            dplanes[o * 4 + 0] = ds * gs[0];
            dplanes[o * 4 + 1] = ds * gs[1];
            dplanes[o * 4 + 2] = ds * gs[2];
            dplanes[o * 4 + 3] = 0.0;
        }
    grad_f64_adjoint(dg1, W, H, dimg1);
    grad_f64_adjoint(dg2, W, H, dimg2);
    return CVTPM_OK;
}

}  // extern "C"

/* ---------------------------------------------------------------------
 * Stereo rectification and bilinear warps (the input side of the path).
 *
 *   orc_stereo_rectify  StereoCameraCalibration(first, second, extrinsics)
 *                       .undistortRectify (cvt/vision/StereoCameraCalibration.h:
 *                       124-130, 166-277) with UndistortRectifyWarp (:79-92)
 *                       evaluated per map pixel as IWarp::warpGeneric does
 *                       (cvt/gfx/ifilter/IWarp.h:80-99)
 *   orc_warp            IWarp::apply's row loops (cvt/gfx/ifilter/IWarp.cpp:
 *                       254-376) over SIMD::warpBilinear1f / 4f / 1u8 / 4u8
 *                       (cvt/util/SIMD.cpp:4497-4710, _floor :732-739,
 *                       _mix4U8 :702-717)
 * Float arithmetic in the reference's order (flat row-major arrays here),
 * the C library's sqrtf / sinf / cosf / acosf as the reference's Math::
 * wrappers call them.  Map coordinates that are not finite or beyond the
 * fixed-point range give the fill value (undefined in the reference).
 * --------------------------------------------------------------------- */
namespace {

void mat3_mul(const float* a, const float* b, float* r) {      /* Matrix3.h:275-286 */
    float t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    memcpy(r, t, sizeof t);
}

void mat3_vec(const float* a, const float* v, float* r) {      /* Matrix3.h:257-262 */
    float t[3];
    for (int i = 0; i < 3; ++i) t[i] = a[i * 3] * v[0] + a[i * 3 + 1] * v[1] + a[i * 3 + 2] * v[2];
    memcpy(r, t, sizeof t);
}

void vec3_normalize(float* v) {                                 /* Vector3.h:344-352 */
    const float ls = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const float inv = 1.0f / sqrtf(ls);
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}

void set_rotation(const float* ax_in, float rad, float* m) {    /* Matrix3.h:508-553 */
    float a[3] = {ax_in[0], ax_in[1], ax_in[2]};
    vec3_normalize(a);
    const float c = cosf(rad * 0.5f), s = sinf(rad * 0.5f);
    const float x = a[0] * s, y = a[1] * s, z = a[2] * s;
    const float x2 = x + x, y2 = y + y, z2 = z + z;
    const float xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
    const float wx = c * x2, wy = c * y2, wz = c * z2;
    const float r[9] = {1.0f - (yy + zz), xy - wz, xz + wy,
                        xy + wz, 1.0f - (xx + zz), yz - wx,
                        xz - wy, yz + wx, 1.0f - (xx + yy)};
    memcpy(m, r, sizeof r);
}

/* Quaternion(Matrix3) (Quaternion.h:128-164) + toAxisAngle (:517-523) */
void to_axis_angle(const float* m, float* axis, float* angle) {
    float q[4];    /* x, y, z, w */
    const float tr = m[0] + m[4] + m[8];
    if (tr > 0.0f) {
        float root = sqrtf(tr + 1.0f);
        q[3] = 0.5f * root;
        root = 0.5f / root;
        q[0] = (m[7] - m[5]) * root;
        q[1] = (m[2] - m[6]) * root;
        q[2] = (m[3] - m[1]) * root;
    } else {
        int i = 0;
        if (m[4] > m[0]) i = 1;
        if (m[8] > m[i * 4]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        float root = sqrtf(m[i * 4] - m[j * 4] - m[k * 4] + 1.0f);
        q[i] = 0.5f * root;
        root = 0.5f / root;
        q[3] = (m[k * 3 + j] - m[j * 3 + k]) * root;
        q[j] = (m[j * 3 + i] + m[i * 3 + j]) * root;
        q[k] = (m[k * 3 + i] + m[i * 3 + k]) * root;
    }
    *angle = acosf(q[3]) * 2.0f;
    const float s = sinf(*angle * 0.5f);
    axis[0] = q[0] / s; axis[1] = q[1] / s; axis[2] = q[2] / s;
    vec3_normalize(axis);
}

void homog_col3(const float* E, float* t) {                     /* Vector3(Vector4), Vector3.h:120-126 */
    const float invw = (float)(1.0 / (double)E[15]);
    t[0] = invw * E[3]; t[1] = invw * E[7]; t[2] = invw * E[11];
}

/* rectificationMatrices(Rleft, Rright), horizontal (:166-197) */
void rect_rotations(const float* E, float* Rl, float* Rr) {
    const float R[9] = {E[0], E[1], E[2], E[4], E[5], E[6], E[8], E[9], E[10]};
    float axis[3], angle, t[3], c[3];
    to_axis_angle(R, axis, &angle);
    set_rotation(axis, 0.5f * angle, Rl);
    set_rotation(axis, -0.5f * angle, Rr);
    homog_col3(E, c);
    mat3_vec(Rr, c, t);
    float u[3] = {1.0f, 0.0f, 0.0f};
    if (t[0] * u[0] + t[1] * u[1] + t[2] * u[2] < 0.0f) { u[0] = -u[0]; u[1] = -u[1]; u[2] = -u[2]; }
    float ax[3] = {t[1] * u[2] - t[2] * u[1], t[2] * u[0] - t[0] * u[2], t[0] * u[1] - t[1] * u[0]};
    vec3_normalize(ax);
    const float d = u[0] * t[0] + u[1] * t[1] + u[2] * t[2];
    const float len = sqrtf(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const float ang = acosf(fabsf(d) / len);
    float R2[9];
    set_rotation(ax, ang, R2);
    mat3_mul(R2, Rr, Rr);
    mat3_mul(R2, Rl, Rl);
}

/* UndistortRectifyWarp::operator()(Vector2f(x, y)) (:79-92) */
void rect_point(float x, float y, float fn, float cnx, float cny, const float* rt, const float* K, const float* rad,
                const float* tan, float* mx, float* my) {
    const float dx = (x - cnx) / fn, dy = (y - cny) / fn;
    float px = rt[0] * dx + rt[1] * dy + rt[2];
    float py = rt[3] * dx + rt[4] * dy + rt[5];
    const float w = rt[6] * dx + rt[7] * dy + rt[8];
    px /= w;
    py /= w;
    const float r2 = px * px + py * py, r4 = r2 * r2, r6 = r2 * r4;
    const float poly = 1.0f + rad[0] * r2 + rad[1] * r4 + rad[2] * r6;
    const float xy2 = 2.0f * px * py;
    *mx = K[0] * (px * poly + xy2 * tan[0] + tan[1] * (r2 + 2.0f * px * px)) + K[2];
    *my = K[4] * (py * poly + xy2 * tan[1] + tan[0] * (r2 + 2.0f * py * py)) + K[5];
}

int floor_ref(float v) {                                        /* SIMD.cpp:732-739 */
    uint32_t bits;
    memcpy(&bits, &v, 4);
    return (int)v - (int)(bits >> 31);
}

uint32_t mix4(uint32_t a, uint32_t b, uint32_t t) {             /* SIMD.cpp:702-717 */
    uint32_t hi = (((b >> 8) & 0xff00ffu) - ((a >> 8) & 0xff00ffu)) * t;
    hi = (hi + (a & 0xff00ff00u)) & 0xff00ff00u;
    uint32_t lo = ((b & 0xff00ffu) - (a & 0xff00ffu)) * t;
    lo = ((lo >> 8) + (a & 0xff00ffu)) & 0xff00ffu;
    return hi + lo;
}

}  // namespace

extern "C" {

/* maps: W*H (x, y) pairs each; K0new/K1new 9, Enew 16, Rl/Rr 9 floats. */
int orc_stereo_rectify(const float* K0, const float* rad0, const float* tan0, const float* K1, const float* rad1,
                       const float* tan1, const float* E, int vertical, int W, int H, float* map0, float* map1,
                       float* K0new, float* K1new, float* Enew, float* Rl, float* Rr) {
    rect_rotations(E, Rl, Rr);
    float c[3], t[3], u[3];
    homog_col3(E, c);
    mat3_vec(Rr, c, t);
    mat3_vec(Rr, t, u);
    for (int i = 0; i < 16; ++i) Enew[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    Enew[3] = u[0]; Enew[7] = u[1]; Enew[11] = u[2];
    const float fl = K0[4], fr = K1[4];
    const float fn = (fl < fr) ? fl : fr;
    float clx = K0[2], cly = K0[5], crx = K1[2], cry = K1[5];
    if (vertical) {
        clx = crx = (clx + crx) * 0.5f;
    } else {
        const float ny = (cly + cry) * 0.5f;
        cly = ny;
        cry = ny;
    }
    const float a0[9] = {fn, 0.0f, clx, 0.0f, fn, cly, 0.0f, 0.0f, 1.0f};
    const float a1[9] = {fn, 0.0f, crx, 0.0f, fn, cry, 0.0f, 0.0f, 1.0f};
    memcpy(K0new, a0, sizeof a0);
    memcpy(K1new, a1, sizeof a1);
    float RlT[9], RrT[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { RlT[i * 3 + j] = Rl[j * 3 + i]; RrT[i * 3 + j] = Rr[j * 3 + i]; }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = 2 * ((size_t)y * W + x);
            rect_point((float)x, (float)y, fn, clx, cly, RlT, K0, rad0, tan0, &map0[o], &map0[o + 1]);
            rect_point((float)x, (float)y, fn, crx, cry, RrT, K1, rad1, tan1, &map1[o], &map1[o + 1]);
        }
    return 0;
}

/* kind: 0 GRAY_FLOAT, 1 RGBA/BGRA_FLOAT, 2 GRAY_UINT8, 3 RGBA/BGRA_UINT8;
 * map W*H (x, y) pairs (rows of mstride bytes); strides in bytes. */
int orc_warp(int kind, const void* src, size_t sstride, int sw, int sh, const float* map, size_t mstride, int W, int H,
             void* dst, size_t dstride) {
    const uint8_t* s = (const uint8_t*)src;
#pragma omp parallel for schedule(static)   /* rows are independent */
    for (int y = 0; y < H; ++y) {
        const float* m = (const float*)((const uint8_t*)map + (size_t)y * mstride);
        uint8_t* d = (uint8_t*)dst + (size_t)y * dstride;
        for (int x = 0; x < W; ++x) {
            const float cx = m[2 * x], cy = m[2 * x + 1];
            if (kind == 0 || kind == 1) {
                const int C = kind == 0 ? 1 : 4;
                const float fill[4] = {0.0f, 0.0f, 0.0f, kind == 0 ? 0.0f : 1.0f};
                float* o = (float*)d + (size_t)x * C;
                const bool rep = std::isfinite(cx) && std::isfinite(cy) && fabsf(cx) < 2147483520.0f &&
                                 fabsf(cy) < 2147483520.0f;
                const int lx = rep ? floor_ref(cx) : -2, ly = rep ? floor_ref(cy) : -2;
                if (lx < -1 || lx >= sw || ly < -1 || ly >= sh) {
                    for (int k = 0; k < C; ++k) o[k] = fill[k];
                    continue;
                }
                const float a1 = cx - (float)lx, a2 = cy - (float)ly;
                for (int k = 0; k < C; ++k) {
                    auto at = [&](int px, int py) {
                        return (px >= 0 && px < sw && py >= 0 && py < sh)
                                   ? ((const float*)(s + (size_t)py * sstride))[(size_t)px * C + k] : fill[k];
                    };
                    const float v00 = at(lx, ly), v10 = at(lx + 1, ly), v01 = at(lx, ly + 1), v11 = at(lx + 1, ly + 1);
                    const float v1 = v00 + (v10 - v00) * a1;
                    const float v2 = v01 + (v11 - v01) * a1;
                    o[k] = v1 + (v2 - v1) * a2;
                }
            } else if (kind == 2) {
                if (!(std::isfinite(cx) && std::isfinite(cy) && fabsf(cx) < 32768.0f && fabsf(cy) < 32768.0f)) {
                    d[x] = 0;
                    continue;
                }
                const int fx = (int)(cx * 65536.0f), fy = (int)(cy * 65536.0f);
                const int lx = fx >> 16, ly = fy >> 16, ax = fx & 0xffff, ay = fy & 0xffff;
                if (lx < -1 || lx >= sw || ly < -1 || ly >= sh) {
                    d[x] = 0;
                    continue;
                }
                auto at = [&](int px, int py) {
                    return (px >= 0 && px < sw && py >= 0 && py < sh) ? (int)s[(size_t)py * sstride + px] : 0;
                };
                const int v1 = at(lx, ly) + (((at(lx + 1, ly) - at(lx, ly)) * ax) >> 16);
                const int v2 = at(lx, ly + 1) + (((at(lx + 1, ly + 1) - at(lx, ly + 1)) * ax) >> 16);
                d[x] = (uint8_t)(v1 + (((v2 - v1) * ay) >> 16));
            } else {
                const uint32_t fill = 0xff000000u;
                uint32_t* o = (uint32_t*)d + x;
                if (!(std::isfinite(cx) && std::isfinite(cy) && fabsf(cx) < 8388608.0f && fabsf(cy) < 8388608.0f)) {
                    *o = fill;
                    continue;
                }
                const int fx = (int)(cx * 256.0f), fy = (int)(cy * 256.0f);
                const int lx = fx >> 8, ly = fy >> 8;
                if (lx < -1 || lx >= sw || ly < -1 || ly >= sh) {
                    *o = fill;
                    continue;
                }
                auto at = [&](int px, int py) {
                    uint32_t v;
                    if (!(px >= 0 && px < sw && py >= 0 && py < sh)) return fill;
                    memcpy(&v, s + (size_t)py * sstride + (size_t)px * 4, 4);
                    return v;
                };
                const uint32_t a1 = (uint32_t)fx & 0xffu, a2 = (uint32_t)fy & 0xffu;
                const uint32_t v1 = mix4(at(lx, ly), at(lx + 1, ly), a1);
                const uint32_t v2 = mix4(at(lx, ly + 1), at(lx + 1, ly + 1), a1);
                *o = mix4(v1, v2, a2);
            }
        }
    }
    return 0;
}

}  // extern "C"

/* ---------------------------------------------------------------------
 * TSDF fusion (cvt::TSDFVolume, cvt/vision/TSDFVolume.cpp; kernels
 * cvt/cl/kernel/TSDFVolume/TSDFVolume.cl) on the CPU.  Volume: W*H*D pairs
 * (tsdf, weight), x fastest.  Matrices row-major 4x4.
 *   orc_tsdf_matrices  projall = proj * g2w (Matrix4.h:269-288) and its
 *                      inverse (Matrix.cpp:109-196; unchanged if |det| <
 *                      FLT_EPSILON)
 *   orc_tsdf_clear / orc_tsdf_add / orc_tsdf_raycast / orc_tsdf_slice
 *                      the kernels, with OpenCL's dot summed left to right and
 *                      normalize = v * (1 / sqrt(dot(v, v))); the ray march
 *                      stops after max_steps steps (its float loop need not
 *                      end otherwise).
 * --------------------------------------------------------------------- */
namespace {

void m4mul(const float* a, const float* b, float* r) {
    float t[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            t[i * 4 + j] = a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j] + a[i * 4 + 2] * b[2 * 4 + j] +
                           a[i * 4 + 3] * b[3 * 4 + j];
    memcpy(r, t, sizeof t);
}

void m4inv(const float* m, float* out) {
    auto A = [&](int i, int j) { return m[i * 4 + j]; };
    /* 2x2 minors of rows (r0, r1), columns (c0, c1) */
    auto d2 = [&](int r0, int r1, int c0, int c1) { return A(r0, c0) * A(r1, c1) - A(r1, c0) * A(r0, c1); };
    /* 3x3 minors: row r with the 2x2 minors of rows (p, q) */
    auto d3 = [&](int r, int p, int q, int c0, int c1, int c2) {
        return A(r, c0) * d2(p, q, c1, c2) - A(r, c1) * d2(p, q, c0, c2) + A(r, c2) * d2(p, q, c0, c1);
    };
    const float det = A(0, 0) * d3(1, 2, 3, 1, 2, 3) - A(0, 1) * d3(1, 2, 3, 0, 2, 3) +
                      A(0, 2) * d3(1, 2, 3, 0, 1, 3) - A(0, 3) * d3(1, 2, 3, 0, 1, 2);
    if (fabsf(det) < FLT_EPSILON) { memcpy(out, m, 16 * sizeof(float)); return; }
    const float inv = 1.0f / det;
    /* cofactor of element (j, i): rows without j, columns without i */
    const int rows[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            const int* rr = rows[j];
            const int* cc = rows[i];
            const float c = d3(rr[0], rr[1], rr[2], cc[0], cc[1], cc[2]);
            r[i * 4 + j] = ((i + j) & 1) ? -c * inv : c * inv;
        }
    memcpy(out, r, sizeof r);
}

struct V4 { float x, y, z, w; };
inline float dot4f(const float* r, V4 v) { return ((r[0] * v.x + r[1] * v.y) + r[2] * v.z) + r[3] * v.w; }
inline float mixo(float a, float b, float t) { return a + (b - a) * t; }

float tsdf_trilinear(const float* cv, int W, int H, int D, float px, float py, float pz) {
    px = std::fmin(std::fmax(0.0f, px), (float)(W - 2));
    py = std::fmin(std::fmax(0.0f, py), (float)(H - 2));
    pz = std::fmin(std::fmax(0.0f, pz), (float)(D - 2));
    const float bx = std::floor(px), by = std::floor(py), bz = std::floor(pz);
    const int ix = (int)bx, iy = (int)by, iz = (int)bz;
    float v[8];
    for (int k = 0; k < 8; ++k) {
        const size_t o = 2 * (((size_t)(iz + (k >> 2)) * H + (size_t)(iy + ((k >> 1) & 1))) * W + (size_t)(ix + (k & 1)));
        if (cv[o + 1] < 1.0f) return 1e10f;
        v[k] = cv[o];
    }
    const float az = pz - bz, ay = py - by, ax = px - bx;
    const float y0 = mixo(mixo(v[0], v[4], az), mixo(v[2], v[6], az), ay);
    const float y1 = mixo(mixo(v[1], v[5], az), mixo(v[3], v[7], az), ay);
    return mixo(y0, y1, ax);
}

}  // namespace

extern "C" {

int orc_tsdf_matrices(const float* proj, const float* g2w, float* tg2cam, float* tcam2g) {
    m4mul(proj, g2w, tg2cam);
    m4inv(tg2cam, tcam2g);
    return 0;
}

int orc_tsdf_clear(float* cv, int W, int H, int D, float init) {
    for (size_t i = 0; i < (size_t)W * H * D; ++i) { cv[2 * i] = 1.0f; cv[2 * i + 1] = init; }
    return 0;
}

int orc_tsdf_add(float* cv, int W, int H, int D, const float* dmap, int iw, int ih, float dscale, const float* T,
                 float trunc) {
#pragma omp parallel for schedule(static)   /* voxels are independent */
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const V4 p{(float)x, (float)y, (float)z, 1.0f};
                const float gx = dot4f(T, p), gy = dot4f(T + 4, p), gz = dot4f(T + 8, p);
                const float u = gx / gz, v = gy / gz;
                if (!(u < (float)iw && v < (float)ih && u >= 0.0f && v >= 0.0f)) continue;
                const float d = dmap[(size_t)(int)std::floor(v) * iw + (size_t)(int)std::floor(u)] * dscale;
                if (!(d > 0.0f && gz > 0.0f)) continue;
                const float sdf = d - gz;
                const float t = sdf / trunc;
                if (!(std::fabs(sdf) <= trunc)) continue;
                float* c = cv + 2 * (((size_t)z * H + y) * W + x);
                const float w = 1.0f;
                const float nx = (c[0] * c[1] + t * w) / (c[1] + w), ny = c[1] + w;
                c[0] = nx;
                c[1] = ny;
            }
    return 0;
}

int orc_tsdf_raycast(float* out, int iw, int ih, const float* cv, int W, int H, int D, const float* Ti,
                     const float* T, float scale, int max_steps) {
    for (int gy = 0; gy < ih; ++gy)
        for (int gx = 0; gx < iw; ++gx) {
            const V4 z0{0.0f, 0.0f, 0.0f, 1.0f}, p1{(float)gx, (float)gy, 1.0f, 1.0f};
            const float ox = dot4f(Ti, z0), oy = dot4f(Ti + 4, z0), oz = dot4f(Ti + 8, z0);
            float dx = dot4f(Ti, p1) - ox, dy = dot4f(Ti + 4, p1) - oy, dz = dot4f(Ti + 8, p1) - oz;
            const float n = 1.0f / std::sqrt((dx * dx + dy * dy) + dz * dz);
            dx *= n; dy *= n; dz *= n;
            const float sx = ((dx > 0.0f ? 0.0f : (float)W) - ox) / dx, sy = ((dy > 0.0f ? 0.0f : (float)H) - oy) / dy;
            const float sz = ((dz > 0.0f ? 0.0f : (float)D) - oz) / dz;
            const float ex = ((dx > 0.0f ? (float)W : 0.0f) - ox) / dx, ey = ((dy > 0.0f ? (float)H : 0.0f) - oy) / dy;
            const float ez = ((dz > 0.0f ? (float)D : 0.0f) - oz) / dz;
            const float rs = std::fmax(std::fmax(sx, sy), sz), re = std::fmin(std::fmin(ex, ey), ez);
            float ret = 0.0f;
            if (rs < re && std::isfinite(rs) && std::isfinite(re) && std::isfinite(dx) && std::isfinite(dy) &&
                std::isfinite(dz)) {
                const float span = re - rs;
                const float vx = std::fabs(dx * span), vy = std::fabs(dy * span), vz = std::fabs(dz * span);
                const float len = std::sqrt((vx * vx + vy * vy) + vz * vz);
                const float step = 0.5f * len / std::fmax(vx, std::fmax(vy, vz));
                float qx = ox + dx * rs, qy = oy + dy * rs, qz = oz + dz * rs;
                float prev = tsdf_trilinear(cv, W, H, D, qx, qy, qz);
                int k = 0;
                for (float lam = rs + step; lam <= re && k < max_steps; lam += step, ++k) {
                    const float px = ox + dx * lam, py = oy + dy * lam, pz = oz + dz * lam;
                    const float val = tsdf_trilinear(cv, W, H, D, px, py, pz);
                    if (prev < 0.0f && val > 0.0f) break;
                    if (prev > 0.0f && val < 0.0f) {
                        const float a = -val / (prev - val);
                        const float g = mixo(pz, qz, a);
                        ret = std::fmax(-dot4f(T + 8, V4{g, g, g, 1.0f}) * scale, 0.0f);
                        break;
                    }
                    prev = val;
                    qx = px; qy = py; qz = pz;
                }
            }
            out[(size_t)gy * iw + gx] = ret;
        }
    return 0;
}

int orc_tsdf_slice(float* rgba, int axis, int v, const float* cv, int W, int H, int D) {
    const int ow = axis == 0 ? H : W, oh = axis == 2 ? H : D;
    for (int b = 0; b < oh; ++b)
        for (int a = 0; a < ow; ++a) {
            const int x = axis == 0 ? v : a, y = axis == 0 ? a : (axis == 1 ? v : b), z = axis == 2 ? v : b;
            const float t = std::fmin(std::fmax(cv[2 * (((size_t)z * H + y) * W + x)] + 0.5f, 0.0f), 1.0f);
            float* o = rgba + 4 * ((size_t)b * ow + a);
            o[0] = o[1] = o[2] = t;
            o[3] = 1.0f;
        }
    return 0;
}

}  // extern "C"

/* ---------------------------------------------------------------------
 * StereoGCVFilter (cvt/gfx/ifilter/StereoGCVFilter.cpp:71-244) on the CPU,
 * in the reference's order: per disparity, whole-image passes of its
 * kernels, every 16 x 16 work-group executed as OpenCL defines it.
 *   orc_gcv_depthmap   StereoGCVFilter::depthmap (:91-244), point cost
 *                      (USEPOINTSAD); the integral images that only the
 *                      box-SAD and NCC costs read (:143-153) are not formed
 *   orc_gcv_apply      StereoGCVFilter::apply (:71-89): both views and
 *                      stereogcv_occlusioncheck, without the PNG saves
 * Images follow the formats the reference allocates: GRAY (CL_INTENSITY, read
 * as (v, v, v, v), written from .x), GRAYALPHA (CL_RG, read as (r, g, 0, 1))
 * and RGBA.  Reads outside the image return 0 (CLK_ADDRESS_CLAMP's border;
 * also where a CLK_ADDRESS_NONE kernel reads outside, which OpenCL leaves
 * undefined); a linear sampler at integer coordinates (costdepthconv.cl:38,
 * undefined in OpenCL) reads the texel; linear reads at float coordinates
 * follow OpenCL 1.2 section 8.2.  dot sums left to right; mix(a, b, t) =
 * a + (b - a) * t.
 * --------------------------------------------------------------------- */
namespace gcv {

struct F4 {
    float x, y, z, w;
};
inline F4 operator+(F4 a, F4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline F4 operator-(F4 a, F4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline F4 operator*(F4 a, F4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
inline F4 splat(float v) { return {v, v, v, v}; }
inline float dot(F4 a, F4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline F4 fabs4(F4 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z), std::fabs(a.w)}; }

struct Img {
    int w = 0, h = 0, c = 4;
    std::vector<float> d;
    Img() {}
    Img(int w_, int h_, int c_) : w(w_), h(h_), c(c_), d((size_t)w_ * h_ * c_, 0.0f) {}
    F4 rd(int x, int y) const {
        if (x < 0 || y < 0 || x >= w || y >= h) return splat(0.0f);
        const float* p = &d[((size_t)y * w + x) * c];
        if (c == 1) return splat(p[0]);
        if (c == 2) return {p[0], p[1], 0.0f, 1.0f};
        return {p[0], p[1], p[2], p[3]};
    }
    void wr(int x, int y, F4 v) {
        if (x < 0 || y < 0 || x >= w || y >= h) return;
        float* p = &d[((size_t)y * w + x) * c];
        p[0] = v.x;
        if (c >= 2) p[1] = v.y;
        if (c == 4) { p[2] = v.z; p[3] = v.w; }
    }
    /* read_imagef with a linear sampler at (u, v), OpenCL 1.2 section 8.2 */
    F4 lin(float u, float v) const {
        const float tu = u - 0.5f, tv = v - 0.5f;
        const float fu = std::floor(tu), fv = std::floor(tv);
        const float a = tu - fu, b = tv - fv;
        const int i0 = (int)fu, j0 = (int)fv;
        const F4 t00 = rd(i0, j0), t10 = rd(i0 + 1, j0), t01 = rd(i0, j0 + 1), t11 = rd(i0 + 1, j0 + 1);
        return ((splat((1.0f - a) * (1.0f - b)) * t00 + splat(a * (1.0f - b)) * t10) + splat((1.0f - a) * b) * t01) +
               splat(a * b) * t11;
    }
};

const int BS = 16;   /* the integral filter's block size (IntegralFilter.cpp) */

/* prefixsum_pblock / _mul2 / _outerrgb (prefixsum/prefixsum_pblock*.cl:25-63):
 * per 16 x 16 work-group, Hillis-Steele steps, x then y per offset.  The
 * outer-product variant scans 8 channels (two outputs). */
void pblock(Img& out, Img* out2, const Img& in, const Img* in2, bool outer) {
    const int gw = (in.w + BS - 1) / BS, gh = (in.h + BS - 1) / BS;
#pragma omp parallel for schedule(static)
    for (int by = 0; by < gh; ++by)
        for (int bx = 0; bx < gw; ++bx) {
            std::vector<F4> lo(BS * BS), hi(BS * BS), blo(BS * BS), bhi(BS * BS);
            for (int ly = 0; ly < BS; ++ly)
                for (int lx = 0; lx < BS; ++lx) {
                    const int x = bx * BS + lx, y = by * BS + ly, l = ly * BS + lx;
                    const F4 v = in.rd(x, y);
                    if (outer) {
                        lo[l] = {v.x * v.x, v.x * v.y, v.x * v.z, 0.0f};   /* (rgb.x * rgb.xyz, 0, */
                        hi[l] = {v.y * v.y, v.y * v.z, v.z * v.z, 0.0f};   /*  rgb.y * rgb.yz, rgb.z * rgb.z, 0) */
                    } else {
                        lo[l] = in2 ? v * in2->rd(x, y) : v;
                    }
                }
            for (int off = 1; off < BS; off <<= 1) {
                blo = lo;
                bhi = hi;
                for (int l = 0; l < BS * BS; ++l)
                    if (l % BS >= off) {
                        lo[l] = lo[l] + blo[l - off];
                        if (outer) hi[l] = hi[l] + bhi[l - off];
                    }
                blo = lo;
                bhi = hi;
                for (int l = 0; l < BS * BS; ++l)
                    if (l / BS >= off) {
                        lo[l] = lo[l] + blo[l - BS * off];
                        if (outer) hi[l] = hi[l] + bhi[l - BS * off];
                    }
            }
            for (int ly = 0; ly < BS; ++ly)
                for (int lx = 0; lx < BS; ++lx) {
                    out.wr(bx * BS + lx, by * BS + ly, lo[ly * BS + lx]);
                    if (outer) out2->wr(bx * BS + lx, by * BS + ly, hi[ly * BS + lx]);
                }
        }
}

/* prefixsum_horiz / prefixsum_vert (:25-45), in place: running sums over
 * the block-boundary columns of each row, then the boundary rows of each
 * column */
void horiz_vert(Img& m) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < m.h; ++y) {
        F4 acc = splat(0.0f);
        for (int x = BS - 1; x < m.w; x += BS) {
            acc = acc + m.rd(x, y);
            m.wr(x, y, acc);
        }
    }
#pragma omp parallel for schedule(static)
    for (int x = 0; x < m.w; ++x) {
        F4 acc = splat(0.0f);
        for (int y = BS - 1; y < m.h; y += BS) {
            acc = acc + m.rd(x, y);
            m.wr(x, y, acc);
        }
    }
}

/* prefixsum_block2 (prefixsum_block2.cl:79-152), in place: each work-group's
 * window shifted by (-1, -1) gets its left column and top row added; the
 * rows and columns that no window covers get the fix-ups of :139-149.
 * Windows of different work-groups are disjoint, and the fix-ups read only
 * pixels no window writes, so work-group order does not matter. */
void block2(Img& m) {
    const int gw = (m.w + BS - 1) / BS, gh = (m.h + BS - 1) / BS;
#pragma omp parallel for schedule(static)
    for (int gy = 0; gy < gh; ++gy)
        for (int gx = 0; gx < gw; ++gx) {
            F4 buf[BS][BS];
            const int bx = gx * BS, by = gy * BS;
            for (int ly = 0; ly < BS; ++ly)
                for (int lx = 0; lx < BS; ++lx) buf[ly][lx] = m.rd(bx + lx - 1, by + ly - 1);
            for (int ly = 0; ly < BS; ++ly)
                for (int lx = 1; lx < BS; ++lx) buf[ly][lx] = buf[ly][lx] + buf[ly][0];
            for (int ly = 1; ly < BS; ++ly)
                for (int lx = 0; lx < BS; ++lx) buf[ly][lx] = buf[ly][lx] + buf[0][lx];
            std::vector<std::pair<std::pair<int, int>, F4>> fix;
            for (int ly = 0; ly < BS; ++ly)
                for (int lx = 0; lx < BS; ++lx) {
                    const int x = bx + lx, y = by + ly;
                    if (x > m.w || y > m.h || !x || !y) continue;
                    m.wr(x - 1, y - 1, buf[ly][lx]);
                    if (y == m.h - 1 && lx < BS - 1 && ly == BS - 1 && x < m.w)
                        fix.push_back({{x, y}, m.rd(x, y) + m.rd(bx - 1, by + ly)});
                    if (x == m.w - 1 && ly < BS - 1 && lx == BS - 1 && y < m.h)
                        fix.push_back({{x, y}, m.rd(x, y) + m.rd(bx + lx, by - 1)});
                }
            for (auto& f : fix) m.wr(f.first.first, f.first.second, f.second);
        }
}

/* IntegralFilter::apply / applyOuterRGB: the four passes */
void integral(Img& dst, const Img& src, const Img* src2) {
    pblock(dst, nullptr, src, src2, false);
    horiz_vert(dst);
    block2(dst);
}

/* boxfilter_prefixsum (boxfilter/boxfilter_prefixsum.cl:46-71) */
void box(Img& out, const Img& in, int r) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < out.h; ++y)
        for (int x = 0; x < out.w; ++x) {
            const int x0 = std::max(0, x - (r + 1)), y0 = std::max(0, y - (r + 1));
            const int x1 = std::min(out.w - 1, x + r), y1 = std::min(out.h - 1, y + r);
            F4 v = in.rd(x0, y0);
            v = v - in.rd(x0, y1);
            v = v - in.rd(x1, y0);
            v = v + in.rd(x1, y1);
            const float area = (float)((x1 - x0) * (y1 - y0));
            out.wr(x, y, {v.x / area, v.y / area, v.z / area, v.w / area});
        }
}

/* StereoGCVFilter::depthmap (:91-244) */
void depthmap(float* dst, const Img& cam0, const Img& cam1, float dmin, float dmax, float dt) {
    const int W = cam0.w, H = cam0.h, R = 9;
    const float EPS = 1e-3f;
    Img cost(W, H, 1), costgf(W, H, 1), c[2] = {Img(W, H, 2), Img(W, H, 2)}, g0(W, H, 4), g1(W, H, 4);
    Img ia(W, H, 4), ib(W, H, 4), iint(W, H, 4), iint2(W, H, 4), meanG(W, H, 4), meanS(W, H, 1), meanGS(W, H, 4);
    Img mRR(W, H, 4), mGG(W, H, 4);
    int index = 0;
    for (int y = 0; y < H; ++y)                                        /* fill (:124-128) */
        for (int x = 0; x < W; ++x) c[!index].wr(x, y, {1e9f, 0.0f, 0.0f, 0.0f});
    for (int y = 0; y < H; ++y)                                        /* gradx.cl:25-54 */
        for (int x = 0; x < W; ++x) {
            g0.wr(x, y, cam0.rd(x + 1, y) - cam0.rd(x - 1, y));
            g1.wr(x, y, cam1.rd(x + 1, y) - cam1.rd(x - 1, y));
        }
    integral(iint, cam1, nullptr);                                     /* :141-142 */
    box(meanG, iint, R);
    pblock(iint, &iint2, cam1, nullptr, true);                         /* :156-158 */
    horiz_vert(iint);
    horiz_vert(iint2);
    block2(iint);
    block2(iint2);
    box(mRR, iint, R);
    box(mGG, iint2, R);
    if (dmax < dmin && dt > 0) dt = -dt;
    size_t n = (size_t)(std::fabs(dmax - dmin) / std::fabs(dt));
    const F4 dm = {0.3333f, 0.3333f, 0.3333f, 0.0f};
    for (float d = dmin; n--; d += dt) {
        /* stereogcv_costdepthgrad (costdepthgrad.cl:61-135): img0 = cam1,
         * img1 = cam0, grad0 = g1, grad1 = g0 (:169-175) */
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const float u = (float)x + 0.5f - d, v = (float)y + 0.5f;
                float cv;
                if (u < 0.0f || u >= (float)W || v < 0.0f || v >= (float)H) {
                    cv = 0.008f + 0.028f;
                } else {
                    const F4 I0 = cam1.rd(x, y), G0 = g1.rd(x, y), I1 = cam0.lin(u, v), G1 = g0.lin(u, v);
                    const float ci = std::fmin(dot(fabs4(I1 - I0), dm), 0.028f);
                    const float cg = std::fmin(dot(fabs4(G1 - G0), dm), 0.008f);
                    cv = ci + (cg - ci) * 0.10f;
                }
                cost.wr(x, y, splat(cv));
            }
        /* the guided filter (:203-227) */
        Img ig(W, H, 1);
        integral(ig, cost, nullptr);
        box(meanS, ig, R);
        integral(iint, cam1, &cost);
        box(meanGS, iint, R);
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)                                    /* guidedfilter_calcab_outerrgb.cl:76-128 */
            for (int x = 0; x < W; ++x) {
                const F4 g = meanG.rd(x, y), s = meanS.rd(x, y), sg = meanGS.rd(x, y);
                F4 rr = mRR.rd(x, y), gg = mGG.rd(x, y);
                F4 cov = sg - g * s;
                cov.w = 0.0f;
                rr.x = rr.x - g.x * g.x; rr.y = rr.y - g.x * g.y; rr.z = rr.z - g.x * g.z;
                gg.x = gg.x - g.y * g.y; gg.y = gg.y - g.y * g.z;
                gg.z = gg.z - g.z * g.z;
                float m0[3] = {rr.x, rr.y, rr.z}, m1[3] = {rr.y, gg.x, gg.y}, m2[3] = {rr.z, gg.y, gg.z};
                m0[0] = m0[0] + 1.0f * EPS;
                m1[1] = m1[1] + 1.0f * EPS;
                m2[2] = m2[2] + 1.0f * EPS;
                /* LUSolve (:51-74) */
                m1[0] = m1[0] / m0[0];
                m2[0] = m2[0] / m0[0];
                m1[1] = m1[1] - m1[0] * m0[1]; m1[2] = m1[2] - m1[0] * m0[2];
                m2[1] = m2[1] - m2[0] * m0[1]; m2[2] = m2[2] - m2[0] * m0[2];
                m2[1] = m2[1] / m1[1];
                m2[2] = m2[2] - m2[1] * m1[2];
                float bx = cov.x, byv = cov.y, bz = cov.z;
                byv = byv - m1[0] * bx;
                bz = bz - (m2[0] * bx + m2[1] * byv);
                const float xz = bz / m2[2];
                const float xy = (byv - m1[2] * xz) / m1[1];
                const float xx = (bx - (m0[1] * xy + m0[2] * xz)) / m0[0];
                const F4 a = {xx, xy, xz, 0.0f};
                ia.wr(x, y, a);
                ib.wr(x, y, s - splat(dot(g, a)));
            }
        integral(iint, ia, nullptr);
        box(ia, iint, R);
        integral(iint, ib, nullptr);
        box(ib, iint, R);
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)                                    /* guidedfilter_applyab_gc_outer.cl:25-47 */
            for (int x = 0; x < W; ++x) {
                F4 o = splat(dot(ia.rd(x, y), cam1.rd(x, y))) + ib.rd(x, y);
                o.w = 1.0f;
                costgf.wr(x, y, o);
            }
        const float nd = std::fabs(d - dmin) / std::fabs(dmax - dmin);
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; ++y)                                    /* stereogcv_costmin (costmin.cl:26-52) */
            for (int x = 0; x < W; ++x) {
                F4 cc = c[!index].rd(x, y);
                const float nv = costgf.rd(x, y).x;
                if (nv < cc.x) { cc.x = nv; cc.y = nd; }
                c[index].wr(x, y, cc);
            }
        index = 1 - index;
    }
    for (int y = 0; y < H; ++y)                                        /* stereogcv_costdepthconv (:25-43) */
        for (int x = 0; x < W; ++x) {
            const float v = c[!index].rd(x, y).y;
            dst[(size_t)y * W + x] = v >= 1.0f ? 0.0f : v * 1.0f + 0.0f;
        }
}

Img rgba(const float* p, int W, int H) {
    Img m(W, H, 4);
    memcpy(m.d.data(), p, sizeof(float) * 4 * (size_t)W * H);
    return m;
}

}  // namespace gcv

extern "C" {

int orc_gcv_depthmap(float* dst, const float* cam0, const float* cam1, int W, int H, float dmin, float dmax,
                     float dt) {
    gcv::depthmap(dst, gcv::rgba(cam0, W, H), gcv::rgba(cam1, W, H), dmin, dmax, dt);
    return 0;
}

int orc_gcv_apply(uint8_t* dst, float* d0, float* d1, const float* cam0, const float* cam1, int W, int H, float dmin,
                  float dmax, float dt) {
    const gcv::Img a = gcv::rgba(cam0, W, H), b = gcv::rgba(cam1, W, H);
    gcv::depthmap(d0, a, b, dmin, dmax, dt);
    gcv::depthmap(d1, b, a, -dmin, -dmax, -dt);
    gcv::Img i0(W, H, 1), i1(W, H, 1);
    memcpy(i0.d.data(), d0, sizeof(float) * (size_t)W * H);
    memcpy(i1.d.data(), d1, sizeof(float) * (size_t)W * H);
    const float ds = std::fabs(dmax);
    for (int y = 0; y < H; ++y)                                        /* stereogcv_occlusioncheck (:27-52) */
        for (int x = 0; x < W; ++x) {
            const float din0 = i0.rd(x, y).x;
            const float dd0 = din0 * ds;
            const float din1 = i1.lin(-dd0 + (float)x + 0.5f, (float)y + 0.5f).x;
            const float dd1 = din1 * ds;
            const float v = std::fabs(-dd0 + dd1) <= 2.0f ? (din0 + din1) * 0.5f : 0.0f;
            /* CL_UNORM_INT8 write: convert_uchar_sat_rte(v * 255) */
            const float q = std::nearbyint(v * 255.0f);
            dst[(size_t)y * W + x] = (uint8_t)(q > 0.0f ? (q < 255.0f ? q : 255.0f) : 0.0f);
        }
    return 0;
}

}  // extern "C"

/* Vision::disparityToDepthmap (cvt/vision/Vision.cpp:147-168) */
extern "C" int orc_disparity_to_depth(float* depth, const float* disp, int W, int H, float dispscale,
                                      float focallength, float baseline, float dispthres) {
    const float fb = focallength * baseline;
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        const float d = disp[i] * dispscale;
        depth[i] = d > dispthres ? fb / d : 0.0f;
    }
    return 0;
}
