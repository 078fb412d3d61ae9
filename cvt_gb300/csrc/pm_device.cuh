/*
 * pm_device.cuh — device-side building blocks of the PatchMatch kernels:
 * float4 helpers, the plane-state algebra of cvt/cl/kernel/pmhstereo.cl,
 * the two random streams and the aggregated ASW cost.
 *
 * All of it is compiled with -fmad=false: an expression such as a*b + c is two
 * IEEE operations, exactly as in the reference's OpenCL source read literally;
 * fused multiply-adds appear only where fmaf() is written.
 */
#ifndef CVT_GB300_PM_DEVICE_CUH
#define CVT_GB300_PM_DEVICE_CUH

#include <stdint.h>
#include <cuda_runtime.h>
#include "pm_math.h"

#define PM_DEV __device__ __forceinline__

/* ------------------------------------------------------------ float4 -- */
PM_DEV float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
PM_DEV float4 f4s(float s) { return make_float4(s, s, s, s); }
PM_DEV float4 operator+(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
PM_DEV float4 operator-(float4 a, float4 b) { return f4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
PM_DEV float4 operator*(float4 a, float4 b) { return f4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
PM_DEV float4 operator/(float4 a, float4 b) { return f4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
PM_DEV float4 operator*(float s, float4 a) { return f4(s * a.x, s * a.y, s * a.z, s * a.w); }
PM_DEV bool finite3(float4 s) { return isfinite(s.x) && isfinite(s.y) && isfinite(s.z); }
PM_DEV float len4(float4 a) { return pm_sqrt(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w); }
PM_DEV float len3(float4 a) { return pm_sqrt((a.x * a.x + a.y * a.y) + a.z * a.z); }
PM_DEV float dot4(float4 a, float4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
PM_DEV int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
PM_DEV int f2i_nan0(float v) { return (v != v) ? 0 : (int)v; }

/* ---------------------------------------------------------------- RNG -- */
/* MWC64X (cvt/cl/kernel/RNG.cl:35-156).  The skip-ahead A^d mod M
 * (RNG.cl:66-84) multiplies table entries A^(2^k) mod M for the set bits of d;
 * each 64x64 -> 128-bit product is reduced with 2^64 = M + E exactly, so the
 * residue equals the reference's bit-serial MulMod64. */
#define PM_MWC_A 4294883355u
#define PM_MWC_M 18446383549859758079ull
#define PM_MWC_E 360523849793537ull   /* 2^64 - M */
#define PM_MWC_BASEID 4077358422479273989ull

/* The constant tables are defined in the kernels' translation unit only
 * (pm_kernels.cu defines PM_KERNELS_TU); other units include this header for
 * the host-visible types. */
#ifdef PM_KERNELS_TU
__constant__ unsigned long long c_mwc_pow2[64];   /* A^(2^k) mod M */
#endif

PM_DEV unsigned long long mwc_mulmod(unsigned long long a, unsigned long long b) {
    unsigned long long lo = a * b;
    unsigned long long hi = __umul64hi(a, b);
#pragma unroll 1
    for (int i = 0; i < 8 && hi != 0ull; ++i) {      /* hi*2^64 == hi*E (mod M) */
        unsigned long long l = hi * PM_MWC_E;
        unsigned long long h = __umul64hi(hi, PM_MWC_E);
        unsigned long long s = lo + l;
        h += (s < lo) ? 1ull : 0ull;
        lo = s;
        hi = h;
    }
    if (lo >= PM_MWC_M) lo -= PM_MWC_M;
    return lo;
}

struct PmRng {
    uint32_t a, b;          /* MWC64X: x, c.  Philox: draw index, unused */
    uint32_t ctr0, ctr1, ctr2, key0, key1;
    uint32_t buf[4];
    int kind;
};

#ifdef PM_KERNELS_TU
PM_DEV void mwc_seed(PmRng& r, unsigned long long distance) {
    unsigned long long m = 1ull;
#pragma unroll 1
    for (int k = 0; k < 64 && distance != 0ull; ++k, distance >>= 1)
        if (distance & 1ull) m = mwc_mulmod(m, c_mwc_pow2[k]);
    unsigned long long v = mwc_mulmod(PM_MWC_BASEID, m);
    r.kind = 0;
    r.a = (uint32_t)(v / PM_MWC_A);
    r.b = (uint32_t)(v % PM_MWC_A);
}
#endif

PM_DEV void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define PM_PHILOX_TAG_INIT 0xFFFFFFFFu

PM_DEV void philox_seed(PmRng& r, uint32_t key0, uint32_t key1, uint32_t pixel, uint32_t tag, uint32_t view) {
    r.kind = 1;
    r.a = 0;
    r.ctr0 = pixel; r.ctr1 = tag; r.ctr2 = view;
    r.key0 = key0; r.key1 = key1;
}

PM_DEV float rng_float(PmRng& r) {
    uint32_t res;
    if (r.kind == 0) {                                  /* RNG.cl:108-118,142-147 */
        uint32_t X = r.a, C = r.b;
        res = X ^ C;
        uint32_t Xn = PM_MWC_A * X + C;
        uint32_t carry = (uint32_t)(Xn < C);
        r.b = __umulhi(PM_MWC_A, X) + carry;
        r.a = Xn;
    } else {
        if ((r.a & 3u) == 0u) philox10(r.ctr0, r.ctr1, r.ctr2, r.a >> 2, r.key0, r.key1, r.buf);
        uint32_t i = r.a & 3u;
        res = (i == 0) ? r.buf[0] : (i == 1) ? r.buf[1] : (i == 2) ? r.buf[2] : r.buf[3];
        r.a++;
    }
    return 2.3283064365386962890625e-10f * __uint2float_rn(res);
}

/* ------------------------------------------------------ plane algebra -- */
PM_DEV float4 viewprop(float4 n) { return f4(1.0f / n.x, -n.y / n.x, -n.z / n.x, 0.0f); }   /* :119-124 */
PM_DEV float transform_x(float4 s, float cx, float cy) { return s.x * cx + s.y * cy + s.z; } /* :126-129 */

PM_DEV float4 state_init(PmRng& rng, float cx, float cy, int lr, float normmul, float depthmax) { /* :50-68 */
    float z = rng_float(rng) * depthmax;
    float nx = (rng_float(rng) - 0.5f) * normmul * 0.95f;
    float ny = (rng_float(rng) - 0.5f) * normmul * 0.95f;
    nx = pm_clamp(nx, -0.95f, 0.95f);
    ny = pm_clamp(ny, -0.95f, 0.95f);
    float nfactor = fmaxf(pm_sqrt(nx * nx + ny * ny) + 0.001f, 1.0f);
    nx = nx / nfactor; ny = ny / nfactor;
    float nz = pm_sqrt(1.0f - nx * nx - ny * ny);
    float4 ret = f4(1.0f - (-nx / nz), 0.0f - (-ny / nz), 0.0f - ((nx * cx + ny * cy) / nz + z), 0.0f - 0.0f);
    if (!lr) ret = viewprop(ret);
    return ret;
}

PM_DEV float4 to_ref_normal_depth(float4 state, float cx, float cy, int lr) {       /* :70-86 */
    float4 s = lr ? state : viewprop(state);
    s = f4(1.0f - s.x, 0.0f - s.y, 0.0f - s.z, 0.0f - s.w);
    float4 ret;
    ret.w = s.x * cx + s.y * cy + s.z;
    ret.z = pm_rsqrt(s.x * s.x + s.y * s.y + 1.0f);
    ret.x = -s.x * ret.z;
    ret.y = -s.y * ret.z;
    if (!finite3(ret)) return f4(0.0f, 0.0f, 1.0f, 0.0f);
    return ret;
}

PM_DEV float4 state_refine(PmRng& rng, float4 in, float cx, float cy, float depthmax, int lr) { /* :88-117 */
    float4 state = lr ? in : viewprop(in);
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
    float nfactor = fmaxf(pm_sqrt(nx * nx + ny * ny) + 0.001f, 1.0f);
    nx = nx / nfactor; ny = ny / nfactor;
    nz = pm_sqrt(1.0f - nx * nx - ny * ny);
    float4 ret = f4(-nx / nz, -ny / nz, (nx * cx + ny * cy) / nz + z, 0.0f);
    ret = f4(1.0f - ret.x, 0.0f - ret.y, 0.0f - ret.z, 0.0f - ret.w);
    if (!lr) return viewprop(state);   /* the reference's right-view branch (:114-115) */
    return ret;
}

PM_DEV void to_normal(float4 st, float& nx, float& ny, float& nz) {               /* :144-153 */
    float4 s = f4(1.0f - st.x, 0.0f - st.y, 0.0f - st.z, 0.0f - st.w);
    nz = pm_rsqrt(s.x * s.x + s.y * s.y + 1.0f);
    nx = -s.x * nz;
    ny = -s.y * nz;
}

PM_DEV void smooth_distance(float4 sa, float4 sb, float4 smooth, float cx, float cy, float depthmax,
                            int lr, float& dA, float& dB) {                      /* :266-283 */
    float4 a = to_ref_normal_depth(sa, cx, cy, lr);
    float4 b = to_ref_normal_depth(sb, cx, cy, lr);
    float4 diag = f4(1.0f, 1.0f, 0.0f, 1.0f / (depthmax * depthmax));
    if (!finite3(sa) || !finite3(sb)) { dA = 0.0f; dB = 0.0f; return; }
    float4 da = a - smooth;
    dA = dot4(da, diag * da);
    float4 db = b - smooth;
    dB = dot4(db, diag * db);
}

/* -------------------------------------------------------------- cost -- */
/* Spatial ASW profile, indexed (dy+31)*63 + (dx+31). */
#define PM_PMAX 31
#define PM_PROF_N (2 * PM_PMAX + 1)
#ifdef PM_KERNELS_TU
__constant__ float c_prof[PM_PROF_N * PM_PROF_N];
#endif

struct PmView {
    const float4* col;    /* RGBA, tight rows          */
    const float4* grad;   /* (dx, dy, dxy, dyx)         */
    const float4* recA;   /* fast records: values (c0,c1,c2,g0)          */
    const float4* recB;   /*   their differences (dc0,dc1,dc2,dg0)        */
    const float4* recC;   /*   (g1,g2,dg1,dg2): values and differences    */
    const float2* recD;   /*   (g3,dg3)                                   */
};

struct PmCostConsts {
    int W, H, P;
    float Wf, Hf;
    float alpha, oma, cmax, gmax;
    int rp;          /* row pitch (elements) of the record planes */
};

/* Packed FP32 pairs (sm_100 and later): one instruction applies the IEEE
 * round-to-nearest add, subtract or fused multiply-add to both halves, so a
 * pair gives the bits of the two scalar operations.  One exception, measured:
 * a packed multiply whose result feeds a packed add does not give the two
 * scalar roundings (36 % of random triples differ, as a fused multiply-add
 * would; the scalar mul.rn/add.rn pair keeps both), so no packed product
 * here feeds a packed add or subtract. */
PM_DEV unsigned long long pk2(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
PM_DEV float2 upk2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
PM_DEV float2 ffma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)), "l"(pk2(c)));
    return upk2(d);
}
PM_DEV float2 fadd2(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
PM_DEV float2 fsub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
PM_DEV float2 fmul2(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
PM_DEV float2 f2s(float v) { return make_float2(v, v); }

/* The matching terms of one tap in the FAST arithmetic: colour and gradient
 * truncated-L1 distances between image 1 at the tap (a1, g1) and the other
 * view interpolated from record j with weight a.  They depend on the tap
 * and the plane only, not on the pixel whose window holds the tap.  The
 * record planes keep each value beside its difference partner, so the
 * interpolations and differences run as packed pairs: channel k is
 * fmaf(a, dT_k, T_k) and a_k - that, as the scalar form computes it. */
/* Record and pixel indices are 64-bit: with 32-bit unsigned indices (whose
 * wrap-around the compiler must keep) the propagation pass measured 33.4 ms
 * against 30.7 ms. */
typedef size_t pm_idx;

/* One row of the other view's record planes.  A window row is one image row
 * for every candidate, so the row's four plane pointers are formed once per
 * row and a tap addresses each plane with its signed column alone. */
struct PmRecRow {
    const float4 *A, *B, *C;
    const float2* D;
};
PM_DEV PmRecRow rec_row(const PmView& v, int rp, int y) {
    const pm_idx o = (pm_idx)y * (pm_idx)rp;
    return {v.recA + o, v.recB + o, v.recC + o, v.recD + o};
}

PM_DEV void fast_tap_terms(const PmCostConsts& k, const PmRecRow& row, int xi, float a, float4 a1, float4 g1,
                           float& cc, float& gc) {
    const float4 A = __ldg(row.A + xi);
    const float4 B = __ldg(row.B + xi);
    const float4 Cc = __ldg(row.C + xi);
    const float2 D = __ldg(row.D + xi);
    const float2 aa = make_float2(a, a);
    const float2 v01 = ffma2(aa, make_float2(B.x, B.y), make_float2(A.x, A.y));     /* c0, c1 */
    const float2 v23 = ffma2(aa, make_float2(B.z, B.w), make_float2(A.z, A.w));     /* c2, g0 */
    const float2 v45 = ffma2(aa, make_float2(Cc.z, Cc.w), make_float2(Cc.x, Cc.y)); /* g1, g2 */
    const float v6 = fmaf(a, D.y, D.x);                                              /* g3 */
    const float2 d01 = fsub2(make_float2(a1.x, a1.y), v01);
    const float2 d23 = fsub2(make_float2(a1.z, g1.x), v23);
    const float2 d45 = fsub2(make_float2(g1.y, g1.z), v45);
    const float d6 = g1.w - v6;
    const float m0 = fminf(fabsf(d01.x), k.cmax), m1 = fminf(fabsf(d01.y), k.cmax), m2 = fminf(fabsf(d23.x), k.cmax);
    const float m3 = fminf(fabsf(d23.y), k.gmax), m4 = fminf(fabsf(d45.x), k.gmax), m5 = fminf(fabsf(d45.y), k.gmax);
    const float m6 = fminf(fabsf(d6), k.gmax);
    const float2 s = fadd2(fadd2(make_float2(m0, m3), make_float2(m1, m4)), make_float2(m2, m5));
    cc = s.x;                                      /* (m0 + m1) + m2 */
    gc = s.y + m6;                                 /* ((m3 + m4) + m5) + m6 */
}

/* The bilateral weight of tap (centre colour vc, tap colour a1, profile
 * value prof): the FAST and EXACT paths and k_nbcost share it. */
PM_DEV float tap_weight(float4 vc, float4 a1, float prof) {
    const float d = (fabsf(vc.x - a1.x) + fabsf(vc.y - a1.y)) + fabsf(vc.z - a1.z);
    return pm_wexp(-d * prof);
}

/* tap_weight of two taps (colours a, b; profile values pa, pb) on packed
 * pairs: each half of every packed operation is the scalar operation
 * tap_weight and pm_wexp perform on that tap, so wa and wb are their floats.
 * -d * prof is formed as -(d * prof) (the same float: RN is symmetric), and
 * fmaf(-kf, c, r) as a fused kf * (-c) + r (the same exact product). */
PM_DEV void tap_weight2(float4 vc, float4 a, float4 b, float pa, float pb, float& wa, float& wb) {
    const float2 ex = fsub2(f2s(vc.x), make_float2(a.x, b.x));
    const float2 ey = fsub2(f2s(vc.y), make_float2(a.y, b.y));
    const float2 ez = fsub2(f2s(vc.z), make_float2(a.z, b.z));
    const float da = (fabsf(ex.x) + fabsf(ey.x)) + fabsf(ez.x);
    const float db = (fabsf(ex.y) + fabsf(ey.y)) + fabsf(ez.y);
    const float2 y = fmul2(make_float2(da, db), make_float2(pa, pb));
    const float2 xc = make_float2(fminf(fmaxf(-y.x, -87.3f), 88.7f), fminf(fmaxf(-y.y, -87.3f), 88.7f));
    const float2 big = ffma2(xc, f2s(1.44269504088896341f), f2s(12582912.0f));
    const float2 kf = fsub2(big, f2s(12582912.0f));
    float2 r = ffma2(kf, f2s(-0.693145751953125f), xc);
    r = ffma2(kf, f2s(-1.4286068202862268e-06f), r);
    float2 p = f2s(1.98412698e-04f);
    p = ffma2(p, r, f2s(1.38888889e-03f));
    p = ffma2(p, r, f2s(8.33333333e-03f));
    p = ffma2(p, r, f2s(4.16666667e-02f));
    p = ffma2(p, r, f2s(1.66666667e-01f));
    p = ffma2(p, r, f2s(0.5f));
    p = ffma2(p, r, f2s(1.0f));
    p = ffma2(p, r, f2s(1.0f));
    wa = __int_as_float(__float_as_int(p.x) + ((__float_as_int(big.x) - 0x4B400000) << 23));
    wb = __int_as_float(__float_as_int(p.y) + ((__float_as_int(big.y) - 0x4B400000) << 23));
}

#ifdef PM_KERNELS_TU
/* Aggregated ASW cost (patch_eval_color_grad_weighted, pmhstereo.cl:170-228)
 * of K candidate planes at pixel (x, y), sharing the image-1 reads and the
 * bilateral weight of every tap.  Each candidate's sum is accumulated in the
 * reference's tap order, so its value equals a separate evaluation.
 * Candidates with act[k] == false contribute nothing and return 1e5. */
/* FAST sweeps of at most PM_PAIR_TAPS_MAXK candidates form their weights two
 * taps at a time (tap_weight2).  Measured per depthMap of the 1242x375 bench
 * pair, same bits: 517.6 -> 509.8 ms with every FAST sweep of 1-4 (the
 * neighbour kernel's weight phase alone: 513.6; sweeps of 3-4 or 2-4 only:
 * within 0.5 ms of 1-4).  The EXACT sweeps keep one tap per step: paired,
 * its stage-1 sweeps of 4 took 148 registers and one block per SM (596 ->
 * 681 ms). */
#ifndef PM_PAIR_TAPS_MAXK
#define PM_PAIR_TAPS_MAXK 4
#endif
#ifndef PM_PAIR_TAPS_MINK
#define PM_PAIR_TAPS_MINK 1
#endif
#ifndef PM_PAIR_TAPS_EXACT
#define PM_PAIR_TAPS_EXACT 0
#endif
template <int K, bool EXACT>
PM_DEV void eval_costs(const PmCostConsts& k, const PmView& v1, const PmView& v2, int x, int y,
                       const float4 (&s)[K], const bool (&act)[K], float (&cost)[K]) {
    float sx[K], sy[K], sz[K];
    /* FAST: X is the candidate's Q31.32 position at the current tap, S0 its
     * step along a row and D the step from a row's end to the next row's
     * start (S1 - n * S0 for rows of n taps).  Integer adds are exact, so X
     * at every tap equals XC + (qy - H/2) * S1 + (qx - W/2) * S0 formed
     * directly, with two fewer 64-bit values per candidate held over the
     * sweep. */
    long long S0[K], D[K], X[K];
    bool live[K];
    const int P = k.P;
    const int dxlo = max(-P, -x), dxhi = min(P, k.W - 1 - x);
    const int qy0 = max(y - P, 0), qy1 = min(y + P, k.H - 1);
#pragma unroll
    for (int c = 0; c < K; ++c) {
        live[c] = act[c] && finite3(s[c]);
        if (EXACT) {
            sx[c] = live[c] ? s[c].x : 0.0f;
            sy[c] = live[c] ? s[c].y : 0.0f;
            sz[c] = live[c] ? s[c].z : -1.0e30f;    /* never inside [0, W) */
        } else {
            long long S1, XC;
            pm_fix_plane(live[c], s[c].x, s[c].y, s[c].z, k.W / 2, k.H / 2, &S0[c], &S1, &XC);
            X[c] = XC + (long long)(qy0 - k.H / 2) * S1 + (long long)(x + dxlo - k.W / 2) * S0[c];
            D[c] = S1 - (long long)(dxhi - dxlo + 1) * S0[c];
        }
    }
    float ws[K], r1[K], r2[K];
#pragma unroll
    for (int c = 0; c < K; ++c) { ws[c] = 0.0f; r1[c] = 0.0f; r2[c] = 0.0f; }
    const float4 vc = __ldg(&v1.col[(size_t)y * k.W + x]);
    for (int qy = qy0; qy <= qy1; ++qy) {
        const int dy = qy - y;
        const float qyf = (float)qy;
        const float4* c1row = v1.col + (size_t)qy * k.W;
        const float4* g1row = v1.grad + (size_t)qy * k.W;
        const float* prow = c_prof + (dy + PM_PMAX) * PM_PROF_N + PM_PMAX;
        const PmRecRow rrow = rec_row(v2, k.rp, qy);
        /* candidate c's terms at tap column qx, folded into its sums */
        auto one = [&](int c, int qx, float4 a1, float4 g1, float w1) {
                if (EXACT) {
                    const float qxf = (float)qx;
                    const float xp = sx[c] * qxf + sy[c] * qyf + sz[c];
                    if (!(xp >= 0.0f && xp < k.Wf)) return;
                    ws[c] += w1;
                    const float u = xp + 0.5f;
                    const float t = u - 0.5f;
                    const float fi = floorf(t);
                    const float a = t - fi;
                    const int i0 = clampi((int)fi, 0, k.W - 1);
                    const int i1 = clampi((int)fi + 1, 0, k.W - 1);
                    const pm_idx rb = (pm_idx)qy * (pm_idx)k.W;
                    const float4 c0 = __ldg(&v2.col[rb + i0]), cc1 = __ldg(&v2.col[rb + i1]);
                    const float4 h0 = __ldg(&v2.grad[rb + i0]), h1 = __ldg(&v2.grad[rb + i1]);
                    const float oa = 1.0f - a;
                    const float a2x = oa * c0.x + a * cc1.x, a2y = oa * c0.y + a * cc1.y, a2z = oa * c0.z + a * cc1.z;
                    const float g2x = oa * h0.x + a * h1.x, g2y = oa * h0.y + a * h1.y;
                    const float g2z = oa * h0.z + a * h1.z, g2w = oa * h0.w + a * h1.w;
                    const float cc = (fminf(fabsf(a1.x - a2x), k.cmax) + fminf(fabsf(a1.y - a2y), k.cmax)) + fminf(fabsf(a1.z - a2z), k.cmax);
                    const float gc = ((fminf(fabsf(g1.x - g2x), k.gmax) + fminf(fabsf(g1.y - g2y), k.gmax)) + fminf(fabsf(g1.z - g2z), k.gmax)) + fminf(fabsf(g1.w - g2w), k.gmax);
                    const float C = k.alpha * cc + k.oma * gc;
                    r1[c] += w1 * C;
                } else {
                    const long long Xt = X[c];
                    X[c] += S0[c];
                    const int xi = (int)(Xt >> 32);
                    if ((unsigned)xi >= (unsigned)k.W) return;
                    float cc, gc;
                    fast_tap_terms(k, rrow, xi, pm_fix_frac(Xt), a1, g1, cc, gc);
                    const float2 r = ffma2(make_float2(w1, w1), make_float2(cc, gc), make_float2(r1[c], r2[c]));
                    r1[c] = r.x;                   /* fmaf(w1, cc, r1), fmaf(w1, gc, r2) */
                    r2[c] = r.y;
                    ws[c] = ws[c] + w1;
                }
        };
        int dx = dxlo;
        if (K >= PM_PAIR_TAPS_MINK && K <= PM_PAIR_TAPS_MAXK && (!EXACT || PM_PAIR_TAPS_EXACT)) {
            /* two taps per step: their weights on packed pairs; each
             * candidate still takes tap dx before tap dx + 1 */
            for (; dx < dxhi; dx += 2) {
                const int qx = x + dx;
                const float4 a1 = __ldg(&c1row[qx]), a1b = __ldg(&c1row[qx + 1]);
                const float4 g1 = __ldg(&g1row[qx]), g1b = __ldg(&g1row[qx + 1]);
                float w1, w1b;
                tap_weight2(vc, a1, a1b, prow[dx], prow[dx + 1], w1, w1b);
#pragma unroll
                for (int c = 0; c < K; ++c) {
                    one(c, qx, a1, g1, w1);
                    one(c, qx + 1, a1b, g1b, w1b);
                }
            }
        }
        for (; dx <= dxhi; ++dx) {
            const int qx = x + dx;
            const float4 a1 = __ldg(&c1row[qx]);
            const float4 g1 = __ldg(&g1row[qx]);
            const float w1 = tap_weight(vc, a1, prow[dx]);
#pragma unroll
            for (int c = 0; c < K; ++c) one(c, qx, a1, g1, w1);
        }
        if (!EXACT) {
#pragma unroll
            for (int c = 0; c < K; ++c) X[c] += D[c];
        }
    }
#pragma unroll
    for (int c = 0; c < K; ++c) {
        float v;
        if (EXACT) v = r1[c] / ws[c];
        else v = fmaf(k.alpha, r1[c], k.oma * r2[c]) / ws[c];
        cost[c] = (!live[c] || ws[c] <= 1.1f) ? 1e5f : v;
    }
}
#endif


#endif
