/*
 * pm_adjoint.cu — the adjoint of the aggregated ASW cost
 * (patch_eval_color_grad_weighted, cvt/cl/kernel/pmhstereo.cl:170-228) with
 * respect to the per-pixel planes and both input images.
 *
 * The cost of pixel p with plane state s is C = R / S over the valid taps t
 * of its window, S = sum w_t, R = sum w_t c_t, where
 *   w_t = exp(-d_t prof_t),  d_t = sum_ch |I1(p) - I1(q)|,
 *   c_t = alpha sum_ch min(|e_ch|, cmax) + (1 - alpha) sum_k min(|eg_k|, gmax),
 *   e = I1(q) - lerp(I2, x'),  eg = G1(q) - lerp(G2, x'),  x' = s . (qx, qy, 1),
 * and G = the gradient images of pmhstereo.cl:785-831 (linear in the grey
 * image).  Given g = dL/dC per pixel:
 *   dL/dc_t = g w_t / S,   dL/dw_t = g (c_t - C) / S,   dw_t/dd_t = -prof_t w_t,
 *   dc_t/dx' = -(alpha sum_ch s_ch D_ch + (1 - alpha) sum_k s_k Dg_k),
 * with s = sign(e) where |e| is below its truncation (0 above) and D the
 * record's forward difference T(i0 + 1) - T(i0) (the slope of the lerp).
 * Validity changes, the 1.1 threshold and kinks are not differentiated (the
 * one-sided slope of the piece the point lies on is used); a pixel with cost
 * 1e5 has zero gradient.
 *
 * Layout of the work: one thread per pixel sweeps its window twice — once for
 * S and R (the cost), once for the gradients — so the window weights are
 * recomputed, never stored.  The plane gradient is a register sum; the image
 * terms at the centre pixel are summed in registers, the terms at the window
 * pixel q and at the two interpolation columns of the other image are added
 * with 128-bit float atomics into four accumulators (colour and gradient-
 * image adjoints of each image).  A second kernel pulls the gradient-image
 * adjoints back through the transposed 3x3 stencil and the grey weights and
 * writes dL/d(image).  Summation order of the atomics is not fixed, so image
 * gradients vary in the last bits from run to run.
 *
 * Tap positions are Q31.32 fixed point (as in the FAST cost), formed from the
 * plane in double, so x' is exact to ~4e-9 px.
 */
#define PM_KERNELS_TU 1
#include "pm_kernels.cuh"

namespace {

/* Fixed-point plane from double state coefficients (see pm_fix_plane). */
__device__ __forceinline__ bool fix_plane_d(double s0, double s1, double s2, int x, int y, long long& S0,
                                            long long& S1, long long& XC) {
    const bool ok0 = isfinite(s0) && isfinite(s1) && isfinite(s2) && fabs(s0) < 16777216.0 && fabs(s1) < 16777216.0;
    const double xc = ok0 ? __fma_rn(s0, (double)x, __fma_rn(s1, (double)y, s2)) : 0.0;
    const bool ok = ok0 && fabs(xc) < 1073741824.0;
    S0 = ok ? __double2ll_rn(s0 * 4294967296.0) : 0;
    S1 = ok ? __double2ll_rn(s1 * 4294967296.0) : 0;
    XC = ok ? __double2ll_rn(xc * 4294967296.0) : PM_FIX_NONE;
    return ok;
}

__device__ __forceinline__ float sgnf(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
/* sign(e) inside the truncation, 0 outside (the slope of min(|e|, cap)). */
__device__ __forceinline__ float tsgn(float e, float cap) { return fabsf(e) < cap ? sgnf(e) : 0.0f; }

/* One tap's interpolated values of the other view (colour 0-2, gradient
 * 3-6) and their slopes along x'. */
struct TapVals {
    float v[7], D[7];
};
__device__ __forceinline__ void load_tap(const PmView& v2, size_t j, float af, TapVals& t) {
    const float4 A = __ldg(&v2.recA[j]);
    const float4 B = __ldg(&v2.recB[j]);
    const float4 Cc = __ldg(&v2.recC[j]);
    const float2 D = __ldg(&v2.recD[j]);
    const float T[7] = {A.x, A.y, A.z, A.w, Cc.x, Cc.y, D.x};
    const float S[7] = {B.x, B.y, B.z, B.w, Cc.z, Cc.w, D.y};
#pragma unroll
    for (int k = 0; k < 7; ++k) { t.D[k] = S[k]; t.v[k] = fmaf(af, S[k], T[k]); }
}

}  // namespace

struct PmAdjArgs {
    PmCostConsts k;
    PmView v1, v2;
    const float4* planes;
    int lr;
    const float* dcost;        /* NULL: cost only */
    float* cost;               /* may be NULL */
    float4* dplanes;           /* may be NULL */
    float4 *dI1, *dG1, *dI2, *dG2;   /* accumulators (IMG kernels only) */
};

template <bool IMG>
__global__ void __launch_bounds__(256) k_cost_adjoint(PmAdjArgs a) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    const int W = a.k.W, H = a.k.H, P = a.k.P;
    if (x >= W || y >= H) return;
    const size_t o = (size_t)y * W + x;
    const float4 pl = a.planes[o];
    const float ds = a.lr ? -1.0f : 1.0f;               /* d(state)/d(plane) */
    long long S0, S1, XC;
    const bool live = fix_plane_d(1.0 + (double)ds * pl.x, (double)ds * pl.y, (double)ds * pl.z, x, y, S0, S1, XC);
    const float4 vc = __ldg(&a.v1.col[o]);
    const int dxlo = max(-P, -x), dxhi = min(P, W - 1 - x);

    /* sweep 1: the cost (same operations as the FAST evaluator) */
    float ws = 0.0f, r1 = 0.0f, r2 = 0.0f;
    for (int dy = -P; dy <= P; ++dy) {
        const int qy = y + dy;
        if (qy < 0 || qy >= H) continue;
        const float* prow = c_prof + (dy + PM_PMAX) * PM_PROF_N + PM_PMAX;
        long long X = XC + (long long)dy * S1 + (long long)dxlo * S0;
        for (int dx = dxlo; dx <= dxhi; ++dx) {
            const long long Xt = X;
            X += S0;
            const int xi = (int)(Xt >> 32);
            if ((unsigned)xi >= (unsigned)W) continue;
            const size_t q = (size_t)qy * W + x + dx;
            const float4 a1 = __ldg(&a.v1.col[q]);
            const float4 g1 = __ldg(&a.v1.grad[q]);
            const float d = (fabsf(vc.x - a1.x) + fabsf(vc.y - a1.y)) + fabsf(vc.z - a1.z);
            const float w1 = pm_wexp(-d * prow[dx]);
            TapVals t;
            load_tap(a.v2, (size_t)qy * a.k.rp + xi, pm_fix_frac(Xt), t);
            const float cc = (fminf(fabsf(a1.x - t.v[0]), a.k.cmax) + fminf(fabsf(a1.y - t.v[1]), a.k.cmax)) +
                             fminf(fabsf(a1.z - t.v[2]), a.k.cmax);
            const float gc = ((fminf(fabsf(g1.x - t.v[3]), a.k.gmax) + fminf(fabsf(g1.y - t.v[4]), a.k.gmax)) +
                              fminf(fabsf(g1.z - t.v[5]), a.k.gmax)) + fminf(fabsf(g1.w - t.v[6]), a.k.gmax);
            r1 = fmaf(w1, cc, r1);
            r2 = fmaf(w1, gc, r2);
            ws = ws + w1;
        }
    }
    const bool valid = live && ws > 1.1f;
    const float C = valid ? fmaf(a.k.alpha, r1, a.k.oma * r2) / ws : 1e5f;
    if (a.cost) a.cost[o] = C;
    if (!a.dcost) return;

    /* sweep 2: gradients */
    const float g = a.dcost[o];
    float gs0 = 0.0f, gs1 = 0.0f, gs2 = 0.0f;
    float cr = 0.0f, cgc = 0.0f, cb = 0.0f;                   /* centre colour */
    if (valid && g != 0.0f) {
        const float u = g / ws;
        const float al = a.k.alpha, oma = a.k.oma;
        for (int dy = -P; dy <= P; ++dy) {
            const int qy = y + dy;
            if (qy < 0 || qy >= H) continue;
            const float* prow = c_prof + (dy + PM_PMAX) * PM_PROF_N + PM_PMAX;
            long long X = XC + (long long)dy * S1 + (long long)dxlo * S0;
            const float qyf = (float)qy;
            for (int dx = dxlo; dx <= dxhi; ++dx) {
                const long long Xt = X;
                X += S0;
                const int xi = (int)(Xt >> 32);
                if ((unsigned)xi >= (unsigned)W) continue;
                const int qx = x + dx;
                const size_t q = (size_t)qy * W + qx;
                const float4 a1 = __ldg(&a.v1.col[q]);
                const float4 g1 = __ldg(&a.v1.grad[q]);
                const float dcx = vc.x - a1.x, dcy = vc.y - a1.y, dcz = vc.z - a1.z;
                const float prof = prow[dx];
                const float w1 = pm_wexp(-((fabsf(dcx) + fabsf(dcy)) + fabsf(dcz)) * prof);
                const float af = pm_fix_frac(Xt);
                TapVals t;
                load_tap(a.v2, (size_t)qy * a.k.rp + xi, af, t);
                const float e[7] = {a1.x - t.v[0], a1.y - t.v[1], a1.z - t.v[2],
                                    g1.x - t.v[3], g1.y - t.v[4], g1.z - t.v[5], g1.w - t.v[6]};
                const float cc = (fminf(fabsf(e[0]), a.k.cmax) + fminf(fabsf(e[1]), a.k.cmax)) + fminf(fabsf(e[2]), a.k.cmax);
                const float gc = ((fminf(fabsf(e[3]), a.k.gmax) + fminf(fabsf(e[4]), a.k.gmax)) +
                                  fminf(fabsf(e[5]), a.k.gmax)) + fminf(fabsf(e[6]), a.k.gmax);
                const float ct = fmaf(al, cc, oma * gc);
                const float gct = u * w1;                            /* dL/dc_t */
                const float gdt = -(u * (ct - C)) * (prof * w1);     /* dL/dd_t */
                float sc[7];
#pragma unroll
                for (int k = 0; k < 3; ++k) sc[k] = al * tsgn(e[k], a.k.cmax);
#pragma unroll
                for (int k = 3; k < 7; ++k) sc[k] = oma * tsgn(e[k], a.k.gmax);
                float slope = 0.0f;
#pragma unroll
                for (int k = 0; k < 7; ++k) slope = fmaf(sc[k], t.D[k], slope);
                const float gx = -gct * slope;                       /* dL/dx' */
                gs0 = fmaf(gx, (float)qx, gs0);
                gs1 = fmaf(gx, qyf, gs1);
                gs2 += gx;
                if (IMG) {
                    const float sx = sgnf(dcx), sy = sgnf(dcy), sz = sgnf(dcz);
                    cr = fmaf(gdt, sx, cr);
                    cgc = fmaf(gdt, sy, cgc);
                    cb = fmaf(gdt, sz, cb);
                    atomicAdd(&a.dI1[q], make_float4(fmaf(gct, sc[0], -gdt * sx), fmaf(gct, sc[1], -gdt * sy),
                                                     fmaf(gct, sc[2], -gdt * sz), 0.0f));
                    atomicAdd(&a.dG1[q], make_float4(gct * sc[3], gct * sc[4], gct * sc[5], gct * sc[6]));
                    const float w0 = -gct * (1.0f - af), w1i = -gct * af;
                    const size_t j0 = (size_t)qy * W + xi, j1 = (size_t)qy * W + min(xi + 1, W - 1);
                    atomicAdd(&a.dI2[j0], make_float4(w0 * sc[0], w0 * sc[1], w0 * sc[2], 0.0f));
                    atomicAdd(&a.dI2[j1], make_float4(w1i * sc[0], w1i * sc[1], w1i * sc[2], 0.0f));
                    atomicAdd(&a.dG2[j0], make_float4(w0 * sc[3], w0 * sc[4], w0 * sc[5], w0 * sc[6]));
                    atomicAdd(&a.dG2[j1], make_float4(w1i * sc[3], w1i * sc[4], w1i * sc[5], w1i * sc[6]));
                }
            }
        }
    }
    if (a.dplanes) a.dplanes[o] = make_float4(ds * gs0, ds * gs1, ds * gs2, 0.0f);
    if (IMG && (cr != 0.0f || cgc != 0.0f || cb != 0.0f)) atomicAdd(&a.dI1[o], make_float4(cr, cgc, cb, 0.0f));
}

/* dL/d(image) = colour accumulator + grey weights x (transposed gradient
 * stencil applied to the gradient-image accumulator).  The stencil of
 * pmhstereo_gradxy as (dx, dy, component, weight): G.comp(x, y) +=
 * weight * B(x + dx, y + dy), B the grey image (zero outside). */
__global__ void __launch_bounds__(256) k_adjoint_finish(const float4* __restrict__ dI, const float4* __restrict__ dG,
                                                        int W, int H, float* __restrict__ out) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= W || y >= H) return;
    struct Term { int dx, dy, comp; float w; };
    const Term terms[16] = {
        {1, 0, 0, 0.5f}, {-1, 0, 0, -0.5f}, {1, -1, 0, 0.25f}, {-1, -1, 0, -0.25f}, {1, 1, 0, 0.25f}, {-1, 1, 0, -0.25f},
        {0, 1, 1, 0.5f}, {0, -1, 1, -0.5f}, {-1, 1, 1, 0.25f}, {-1, -1, 1, -0.25f}, {1, 1, 1, 0.25f}, {1, -1, 1, -0.25f},
        {1, 1, 2, 1.0f}, {-1, -1, 2, -1.0f}, {-1, 1, 3, 1.0f}, {1, -1, 3, -1.0f}};
    float dB = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int sx = x - terms[i].dx, sy = y - terms[i].dy;
        if (sx < 0 || sy < 0 || sx >= W || sy >= H) continue;
        const float4 v = dG[(size_t)sy * W + sx];
        const float c = terms[i].comp == 0 ? v.x : terms[i].comp == 1 ? v.y : terms[i].comp == 2 ? v.z : v.w;
        dB = fmaf(terms[i].w, c, dB);
    }
    const size_t o = (size_t)y * W + x;
    const float4 v = dI[o];
    out[o * 4 + 0] = fmaf(0.2126f, dB, v.x);
    out[o * 4 + 1] = fmaf(0.7152f, dB, v.y);
    out[o * 4 + 2] = fmaf(0.0722f, dB, v.z);
    out[o * 4 + 3] = 0.0f;
}

cudaError_t pm_adjoint_upload_profile(const float* prof, cudaStream_t st) {
    return cudaMemcpyToSymbolAsync(c_prof, prof, sizeof(float) * PM_PROF_N * PM_PROF_N, 0, cudaMemcpyHostToDevice, st);
}

cudaError_t pm_launch_cost_adjoint(const PmCostConsts& k, const PmView& v1, const PmView& v2, const float4* planes,
                                   int lr, const float* dcost, float* cost, float4* dplanes, float4* dI1, float4* dG1,
                                   float4* dI2, float4* dG2, cudaStream_t st) {
    PmAdjArgs a;
    a.k = k; a.v1 = v1; a.v2 = v2; a.planes = planes; a.lr = lr; a.dcost = dcost; a.cost = cost;
    a.dplanes = dplanes; a.dI1 = dI1; a.dG1 = dG1; a.dI2 = dI2; a.dG2 = dG2;
    dim3 grid((k.W + 31) / 32, (k.H + 7) / 8), block(32, 8);
    if (dI1) k_cost_adjoint<true><<<grid, block, 0, st>>>(a);
    else k_cost_adjoint<false><<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t pm_launch_adjoint_finish(const float4* dI, const float4* dG, int W, int H, float* out, cudaStream_t st) {
    dim3 grid((W + 31) / 32, (H + 7) / 8), block(32, 8);
    k_adjoint_finish<<<grid, block, 0, st>>>(dI, dG, W, H, out);
    return cudaGetLastError();
}

/* ------------------------------------------------- plane polishing -- */
/* Levenberg-Marquardt ("adjoint-driven Gauss-Newton") polishing of a plane
 * field: per pixel, `steps` trial steps on the plane that minimise its
 * aggregated cost C (the FAST evaluation above).  One window sweep at a
 * plane gives C, the gradient g = dC/ds of the adjoint (ds = state), and a
 * Gauss-Newton matrix from the truncated-L1 terms read as reweighted least
 * squares (|e| ~ e^2 / (2 |e0|) near the current residual e0):
 *   H = (1/S) sum_t w_t sum_k beta_k [|e_k| < cap_k] D_k^2 / max(|e_k|, eps_k) g_t g_t^T,
 * g_t = (qx, qy, 1), D_k the slope of the interpolated channel along x'.
 * A step solves (H + mu diag(H) + tiny I) delta = -g in double and is kept
 * only if C decreases (then mu /= 10, else mu *= 10), so C never grows.
 * Costs of 1e5 (no support) are left alone. */
struct PmGnArgs {
    PmCostConsts k;
    PmView v1, v2;
    float4* planes;            /* (a, b, c, -) in/out */
    int lr, steps;
    float* cost;               /* may be NULL */
};

/* One sweep: cost, gradient and GN matrix (upper triangle) at state s. */
__device__ float gn_sweep(const PmGnArgs& a, int x, int y, double s0, double s1, double s2, float* g, float* Hm) {
    const int W = a.k.W, H = a.k.H, P = a.k.P;
    long long S0, S1, XC;
    const bool live = fix_plane_d(s0, s1, s2, x, y, S0, S1, XC);
    const float4 vc = __ldg(&a.v1.col[(size_t)y * W + x]);
    const int dxlo = max(-P, -x), dxhi = min(P, W - 1 - x);
    const float al = a.k.alpha, oma = a.k.oma;
    const float epsc = 0.05f * a.k.cmax, epsg = 0.05f * a.k.gmax;
    float ws = 0.0f, r1 = 0.0f, r2 = 0.0f;
    float gs[3] = {0.0f, 0.0f, 0.0f}, hs[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int dy = -P; dy <= P; ++dy) {
        const int qy = y + dy;
        if (qy < 0 || qy >= H) continue;
        const float* prow = c_prof + (dy + PM_PMAX) * PM_PROF_N + PM_PMAX;
        long long X = XC + (long long)dy * S1 + (long long)dxlo * S0;
        const float qyf = (float)qy;
        for (int dx = dxlo; dx <= dxhi; ++dx) {
            const long long Xt = X;
            X += S0;
            const int xi = (int)(Xt >> 32);
            if ((unsigned)xi >= (unsigned)W) continue;
            const int qx = x + dx;
            const size_t q = (size_t)qy * W + qx;
            const float4 a1 = __ldg(&a.v1.col[q]);
            const float4 g1 = __ldg(&a.v1.grad[q]);
            const float w1 = tap_weight(vc, a1, prow[dx]);
            TapVals t;
            load_tap(a.v2, (size_t)qy * a.k.rp + xi, pm_fix_frac(Xt), t);
            const float e[7] = {a1.x - t.v[0], a1.y - t.v[1], a1.z - t.v[2],
                                g1.x - t.v[3], g1.y - t.v[4], g1.z - t.v[5], g1.w - t.v[6]};
            const float cc = (fminf(fabsf(e[0]), a.k.cmax) + fminf(fabsf(e[1]), a.k.cmax)) + fminf(fabsf(e[2]), a.k.cmax);
            const float gc = ((fminf(fabsf(e[3]), a.k.gmax) + fminf(fabsf(e[4]), a.k.gmax)) +
                              fminf(fabsf(e[5]), a.k.gmax)) + fminf(fabsf(e[6]), a.k.gmax);
            r1 = fmaf(w1, cc, r1);
            r2 = fmaf(w1, gc, r2);
            ws = ws + w1;
            float slope = 0.0f, curv = 0.0f;
#pragma unroll
            for (int k = 0; k < 7; ++k) {
                const bool colour = k < 3;
                const float cap = colour ? a.k.cmax : a.k.gmax;
                if (!(fabsf(e[k]) < cap)) continue;
                const float beta = colour ? al : oma;
                slope = fmaf(beta * tsgn(e[k], cap), t.D[k], slope);
                curv = fmaf(beta * t.D[k], t.D[k] / fmaxf(fabsf(e[k]), colour ? epsc : epsg), curv);
            }
            const float gx = -w1 * slope, hx = w1 * curv;
            const float qxf = (float)qx;
            gs[0] = fmaf(gx, qxf, gs[0]); gs[1] = fmaf(gx, qyf, gs[1]); gs[2] += gx;
            hs[0] = fmaf(hx, qxf * qxf, hs[0]); hs[1] = fmaf(hx, qxf * qyf, hs[1]); hs[2] = fmaf(hx, qxf, hs[2]);
            hs[3] = fmaf(hx, qyf * qyf, hs[3]); hs[4] = fmaf(hx, qyf, hs[4]); hs[5] += hx;
        }
    }
    if (!live || !(ws > 1.1f)) return 1e5f;
    const float inv = 1.0f / ws;
    for (int i = 0; i < 3; ++i) g[i] = gs[i] * inv;
    for (int i = 0; i < 6; ++i) Hm[i] = hs[i] * inv;
    return fmaf(a.k.alpha, r1, a.k.oma * r2) / ws;
}

__global__ void __launch_bounds__(256) k_gn_polish(PmGnArgs a) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= a.k.W || y >= a.k.H) return;
    const size_t o = (size_t)y * a.k.W + x;
    const float4 pl = a.planes[o];
    const double ds = a.lr ? -1.0 : 1.0;
    double s[3] = {1.0 + ds * pl.x, ds * pl.y, ds * pl.z};
    float g[3], Hm[6];
    float C = gn_sweep(a, x, y, s[0], s[1], s[2], g, Hm);
    double mu = 1e-3;
    for (int it = 0; it < a.steps && C < 1e4f; ++it) {
        /* (H + mu diag(H) + tiny) delta = -g, symmetric 3x3 by Cramer's rule in double */
        const double tiny = 1e-9 * (fabs((double)Hm[0]) + fabs((double)Hm[3]) + fabs((double)Hm[5]) + 1e-12);
        const double m00 = Hm[0] * (1.0 + mu) + tiny, m11 = Hm[3] * (1.0 + mu) + tiny, m22 = Hm[5] * (1.0 + mu) + tiny;
        const double m01 = Hm[1], m02 = Hm[2], m12 = Hm[4];
        const double c00 = m11 * m22 - m12 * m12, c01 = m02 * m12 - m01 * m22, c02 = m01 * m12 - m02 * m11;
        const double det = m00 * c00 + m01 * c01 + m02 * c02;
        if (!(fabs(det) > 0.0) || !isfinite(det)) break;
        const double c11 = m00 * m22 - m02 * m02, c12 = m01 * m02 - m00 * m12, c22 = m00 * m11 - m01 * m01;
        const double b0 = -g[0], b1 = -g[1], b2 = -g[2];
        const double d0 = (c00 * b0 + c01 * b1 + c02 * b2) / det;
        const double d1 = (c01 * b0 + c11 * b1 + c12 * b2) / det;
        const double d2 = (c02 * b0 + c12 * b1 + c22 * b2) / det;
        float g2[3], H2[6];
        const float C2 = gn_sweep(a, x, y, s[0] + d0, s[1] + d1, s[2] + d2, g2, H2);
        if (C2 < C) {
            s[0] += d0; s[1] += d1; s[2] += d2;
            C = C2;
            for (int i = 0; i < 3; ++i) g[i] = g2[i];
            for (int i = 0; i < 6; ++i) Hm[i] = H2[i];
            mu = fmax(mu * 0.1, 1e-9);
        } else {
            mu *= 10.0;
        }
    }
    a.planes[o] = make_float4((float)(ds * (s[0] - 1.0)), (float)(ds * s[1]), (float)(ds * s[2]), pl.w);
    if (a.cost) a.cost[o] = C;
}

cudaError_t pm_launch_gn_polish(const PmCostConsts& k, const PmView& v1, const PmView& v2, float4* planes, int lr,
                                int steps, float* cost, cudaStream_t st) {
    PmGnArgs a;
    a.k = k; a.v1 = v1; a.v2 = v2; a.planes = planes; a.lr = lr; a.steps = steps; a.cost = cost;
    dim3 grid((k.W + 31) / 32, (k.H + 7) / 8), block(32, 8);
    k_gn_polish<<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}
