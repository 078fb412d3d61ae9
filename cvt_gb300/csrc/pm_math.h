/*
 * pm_math.h — the project's own elementary functions, shared by the CUDA
 * kernels and the CPU oracle so that both produce identical bits.
 *
 * The reference evaluates its ASW weight with `native_exp`
 * (cvt/cl/kernel/pmhstereo.cl:199), its PD edge weight with `exp`/`pow`
 * (pmhstereo.cl:781) and its normal-angle test with `acospi`
 * (pmhstereo.cl:462).  OpenCL leaves the accuracy of `native_*` to the
 * implementation and allows several ulp for the others, so the reference has
 * no bit-level definition of these functions.  This header fixes one:
 *
 *   pm_exp     Cody–Waite range reduction x = k ln2 + r with an FMA-split ln2,
 *              then the degree-7 Taylor polynomial of e^r (|r| <= ln2/2,
 *              truncation error < 2.6e-9), scaled by 2^k in two exact steps so
 *              that subnormal results are rounded once.
 *   pm_wexp    the ASW weight's exponential (native_exp, :199), evaluated once
 *              per tap and pixel: the same reduction and polynomial on x
 *              clamped to [-87.3, 88.7], scaled by adding k to the exponent
 *              bits (the clamp keeps the result normal).  So the weight has a
 *              floor of e^-87.3 (1.2e-38) and a NaN argument gives the floor.
 *   pm_log     x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *              s = (m-1)/(m+1), by its odd power series to s^13.
 *   pm_pow     exp(y log x) for x >= 0.
 *   pm_acospi  acos via the arcsine Taylor series (coefficients
 *              (2n)!/(4^n (n!)^2 (2n+1)), n <= 11) on |z| <= 1/2, using
 *              acos x = pi/2 - asin x for |x| <= 1/2 and
 *              acos x = 2 asin(sqrt((1-x)/2)) (mirrored for x < 0) otherwise.
 *
 * Every operation is written out explicitly (fmaf where an FMA is meant,
 * plain * and + otherwise).  Device code is compiled with -fmad=false and
 * host code with -ffp-contract=off, IEEE division/sqrt and no flush-to-zero on
 * both sides, so a given input produces the same float on CPU and GPU.
 */
#ifndef CVT_GB300_PM_MATH_H
#define CVT_GB300_PM_MATH_H

#include <stdint.h>
#include <math.h>
#if !defined(__CUDACC__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define PM_HD __host__ __device__ __forceinline__
#else
#define PM_HD static inline
#endif

PM_HD float pm_i2f(int32_t i) {
#if defined(__CUDA_ARCH__)
    return __int_as_float(i);
#else
    float f; memcpy(&f, &i, 4); return f;
#endif
}
PM_HD int32_t pm_f2i(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(f);
#else
    int32_t i; memcpy(&i, &f, 4); return i;
#endif
}
PM_HD uint32_t pm_f2u(float f) { return (uint32_t)pm_f2i(f); }

/* IEEE-rounded reciprocal square root: 1 / sqrt(x), two correctly rounded
 * operations (the reference's native_rsqrt, pmhstereo.cl:78, fixed this way). */
PM_HD float pm_rsqrt(float x) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(__fsqrt_rn(x));
#else
    return 1.0f / sqrtf(x);
#endif
}
PM_HD float pm_sqrt(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}
PM_HD float pm_div(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

/* Round-to-nearest-even conversions and the double FMA, one definition per
 * side; IEEE fixes each result, so CPU and GPU agree bit for bit. */
PM_HD long long pm_f2ll_rn(float x) {
#if defined(__CUDA_ARCH__)
    return __float2ll_rn(x);
#else
    return llrintf(x);
#endif
}
PM_HD long long pm_d2ll_rn(double x) {
#if defined(__CUDA_ARCH__)
    return __double2ll_rn(x);
#else
    return llrint(x);
#endif
}
PM_HD float pm_u2f_rn(unsigned x) {
#if defined(__CUDA_ARCH__)
    return __uint2float_rn(x);
#else
    return (float)x;
#endif
}
PM_HD double pm_fma_d(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

/* Tap positions of the FAST arithmetic in fixed point.  The sample column
 * x' = s0*qx + s1*qy + s2 of tap (qx, qy) is carried in Q31.32 (int64 with
 * 32 fraction bits), anchored at the image centre (ax, ay) = (W/2, H/2):
 *   X(q) = XA + (qx - ax)*S0 + (qy - ay)*S1,
 *   S = round(s * 2^32), XA = round(x'(ax, ay) * 2^32) formed in double.
 * The anchor depends on the image only, so a plane's tap positions are the
 * same integers whichever pixel evaluates it (a window can be shared by all
 * pixels testing one plane).  Slopes with |s| >= 2^-9 are exact in Q32, so a
 * position is within half a unit of 2^-32 px of x' (plus 2^-33 px per
 * coordinate of distance for smaller slopes) at any image width; an FP32
 * evaluation is off by up to half an ulp of x', 6e-5 px at x' ~ 1000.  The
 * integer part is the record index, the fraction the interpolation weight.
 * Planes with |s0| or |s1| >= 2^14 or |x'(ax, ay)| >= 2^30 are not
 * representable (with W <= 2^14 and H <= 2^16, |X| < 2^31 * 2^32 then):
 * they get XA = PM_FIX_NONE and S = 0, which no tap reaches. */
#define PM_FIX_NONE (-(1LL << 62))
PM_HD bool pm_fix_plane(bool live, float s0, float s1, float s2, int ax, int ay,
                        long long* S0, long long* S1, long long* XA) {
    const float one = 4294967296.0f;                               /* 2^32 */
    const bool ok0 = live && isfinite(s0) && isfinite(s1) && isfinite(s2) &&
                     fabsf(s0) < 16384.0f && fabsf(s1) < 16384.0f;
    const double xa = ok0 ? pm_fma_d((double)s0, (double)ax, pm_fma_d((double)s1, (double)ay, (double)s2)) : 0.0;
    const bool ok = ok0 && fabs(xa) < 1073741824.0;               /* 2^30 */
    *S0 = ok ? pm_f2ll_rn(s0 * one) : 0;
    *S1 = ok ? pm_f2ll_rn(s1 * one) : 0;
    *XA = ok ? pm_d2ll_rn(xa * 4294967296.0) : PM_FIX_NONE;
    return ok;
}
/* The interpolation weight: the 32 fraction bits, rounded to float. */
PM_HD float pm_fix_frac(long long X) { return pm_u2f_rn((unsigned)X) * 2.3283064365386963e-10f; }

/* 2^n as a float for -126 <= n <= 127. */
PM_HD float pm_pow2i(int n) { return pm_i2f((n + 127) << 23); }

PM_HD float pm_exp(float x) {
    const float L2E = 1.44269504088896341f;
    const float LN2_HI = 0.693145751953125f;      /* 16 significant bits */
    const float LN2_LO = 1.4286068202862268e-06f; /* ln2 - LN2_HI */
    const float SHIFT = 12582912.0f;              /* 1.5 * 2^23: round to integer */
    float xc = fminf(fmaxf(x, -104.0f), 89.0f);
    float t = xc * L2E;
    float big = t + SHIFT;                        /* SHIFT + round(t): the integer sits in the low bits */
    float kf = big - SHIFT;                       /* round to nearest even */
    float r = fmaf(-kf, LN2_HI, xc);
    r = fmaf(-kf, LN2_LO, r);
    float p = 1.98412698e-04f;                    /* 1/7! */
    p = fmaf(p, r, 1.38888889e-03f);              /* 1/6! */
    p = fmaf(p, r, 8.33333333e-03f);              /* 1/5! */
    p = fmaf(p, r, 4.16666667e-02f);              /* 1/4! */
    p = fmaf(p, r, 1.66666667e-01f);              /* 1/3! */
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = pm_f2i(big) - 0x4B400000;             /* == (int)kf, without a float-to-int conversion */
    int ka = k >> 1;                              /* floor(k/2) */
    int kb = k - ka;
    float res = (p * pm_pow2i(ka)) * pm_pow2i(kb);
    return (x != x) ? x : res;
}

PM_HD float pm_wexp(float x) {
    const float L2E = 1.44269504088896341f;
    const float LN2_HI = 0.693145751953125f;      /* 16 significant bits */
    const float LN2_LO = 1.4286068202862268e-06f; /* ln2 - LN2_HI */
    const float SHIFT = 12582912.0f;              /* 1.5 * 2^23 */
    const float xc = fminf(fmaxf(x, -87.3f), 88.7f);
    const float big = fmaf(xc, L2E, SHIFT);       /* SHIFT + k, k = round(xc / ln2) */
    const float kf = big - SHIFT;
    float r = fmaf(-kf, LN2_HI, xc);
    r = fmaf(-kf, LN2_LO, r);
    float p = 1.98412698e-04f;                    /* 1/7! */
    p = fmaf(p, r, 1.38888889e-03f);              /* 1/6! */
    p = fmaf(p, r, 8.33333333e-03f);              /* 1/5! */
    p = fmaf(p, r, 4.16666667e-02f);              /* 1/4! */
    p = fmaf(p, r, 1.66666667e-01f);              /* 1/3! */
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    /* k in [-126, 128] and p in [0.70, 1.42]: 2^k p stays normal */
    return pm_i2f(pm_f2i(p) + ((pm_f2i(big) - 0x4B400000) << 23));
}

PM_HD float pm_log(float x) {
    /* x > 0 finite; zero, negative, inf and NaN handled by pm_pow's caller. */
    const float LN2_HI = 0.693145751953125f;
    const float LN2_LO = 1.4286068202862268e-06f;
    int e = 0;
    float xs = x;
    if (xs < 1.17549435e-38f) { xs = xs * 8388608.0f; e = -23; }  /* subnormal */
    int32_t b = pm_f2i(xs);
    e += ((b >> 23) & 0xff) - 127;
    float m = pm_i2f((b & 0x007fffff) | 0x3f800000);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    float s = pm_div(m - 1.0f, m + 1.0f);
    float z = s * s;
    float q = 0.0769230769f;                      /* 1/13 */
    q = fmaf(q, z, 0.0909090909f);                /* 1/11 */
    q = fmaf(q, z, 0.111111111f);                 /* 1/9 */
    q = fmaf(q, z, 0.142857143f);                 /* 1/7 */
    q = fmaf(q, z, 0.2f);                         /* 1/5 */
    q = fmaf(q, z, 0.333333333f);                 /* 1/3 */
    q = q * z;
    float lm = fmaf(2.0f * s, q, 2.0f * s);       /* 2s(1 + z q') */
    float ef = (float)e;
    return fmaf(ef, LN2_LO, lm) + ef * LN2_HI;
}

PM_HD float pm_pow(float x, float y) {
    /* Only x >= 0 is used (|gradient| ** 0.8 in the PD edge weight). */
    if (x != x || y != y) return x + y;
    if (x == 0.0f) return (y > 0.0f) ? 0.0f : ((y == 0.0f) ? 1.0f : INFINITY);
    if (x == INFINITY) return (y > 0.0f) ? INFINITY : ((y == 0.0f) ? 1.0f : 0.0f);
    if (x < 0.0f) return NAN;
    return pm_exp(y * pm_log(x));
}

PM_HD float pm_asin_core(float z) {
    /* asin(z) for |z| <= 1/2 by the Taylor series of arcsine. */
    float z2 = z * z;
    float p = 0.0073125258735988454f;
    p = fmaf(p, z2, 0.008390335809616815f);
    p = fmaf(p, z2, 0.009761609529194078f);
    p = fmaf(p, z2, 0.011551800896139705f);
    p = fmaf(p, z2, 0.01396484375f);
    p = fmaf(p, z2, 0.017352764423076924f);
    p = fmaf(p, z2, 0.022372159090909092f);
    p = fmaf(p, z2, 0.030381944444444444f);
    p = fmaf(p, z2, 0.044642857142857144f);
    p = fmaf(p, z2, 0.075f);
    p = fmaf(p, z2, 0.16666666666666666f);
    return fmaf(z * z2, p, z);
}

PM_HD float pm_acospi(float x) {
    const float PI_F = 3.14159274f;
    const float HALF_PI_F = 1.57079637f;
    const float INV_PI_F = 0.318309873f;
    float ax = fabsf(x);
    float a;
    if (ax <= 0.5f) {
        a = HALF_PI_F - pm_asin_core(x);
    } else {
        float t = pm_sqrt((1.0f - ax) * 0.5f);    /* NaN for |x| > 1 */
        float as2 = 2.0f * pm_asin_core(t);
        a = (x > 0.0f) ? as2 : (PI_F - as2);
    }
    return a * INV_PI_F;
}

/* OpenCL smoothstep(e0, e1, x) = t*t*(3-2t), t = clamp((x-e0)/(e1-e0), 0, 1). */
PM_HD float pm_smoothstep(float e0, float e1, float x) {
    float t = pm_div(x - e0, e1 - e0);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return (t * t) * (3.0f - 2.0f * t);
}

/* OpenCL clamp(x, lo, hi) = fmin(fmax(x, lo), hi). */
PM_HD float pm_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

/* The ASW spatial profile of pmhstereo.cl:199 for tap (dx, dy):
 * smoothstep(0, 26, length(d)) * 1.5 * colorweight + 5 (profile 0), or the
 * constant colorweight (profile 1, the gamma-style weight exp(-dc*255/gamma)). */
PM_HD float pm_profile(int dx, int dy, float colorweight, int profile) {
    if (profile == 1) return colorweight;
    float fx = (float)dx, fy = (float)dy;
    float len = pm_sqrt(fx * fx + fy * fy);
    return (pm_smoothstep(0.0f, 26.0f, len) * 1.5f) * colorweight + 5.0f;
}

#endif
