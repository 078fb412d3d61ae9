"""FP32 aggregated cost against an FP64 evaluation of the same formula.

The per-plane cost evaluator (patch_eval_color_grad_weighted,
cvt/cl/kernel/pmhstereo.cl:170-228) runs in FP32.  The oracle's FP64
evaluator computes the same quantity in double precision from the same FP32
images and planes; it is pinned here against a plain numpy restatement on a
small case.  The FAST arithmetic (fixed-point tap positions) stays within
1e-5 relative of FP64 on every pixel whose result is not decided by a tap
lying within 1e-3 px of the image border or by a weight sum within 1e-6 of
the 1.1 threshold.  The reference's own operation order (EXACT) rounds the tap
position x' = s0*qx + s1*qy + s2 in FP32, which costs up to half an ulp of x'
(6e-5 px at x' ~ 1000); its error is measured and bounded, not held to 1e-5.
"""
import numpy as np
import pytest

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_REFERENCE, PRESET_BASELINE, ARITH_EXACT, ARITH_FAST

TOL_FAST = 1e-5


def _crop_states(sc, x0, y0, w, h, seed):
    """Ground-truth planes of a crop plus N(0, 0.01) on a, b and N(0, 1) on c
    (a, b clamped to [-0.3, 0.3]), as plane states (1 - a, -b, -c)."""
    rng = np.random.default_rng(seed)
    pf = sc.plane_field()[y0:y0 + h, x0:x0 + w].astype(np.float64)
    a = np.clip(pf[..., 0] + rng.normal(0, 0.01, (h, w)), -0.3, 0.3)
    b = np.clip(pf[..., 1] + rng.normal(0, 0.01, (h, w)), -0.3, 0.3)
    c = pf[..., 2] + a * x0 + b * y0 + rng.normal(0, 1.0, (h, w))
    st = np.zeros((h, w, 4), np.float32)
    st[..., 0] = 1.0 - a
    st[..., 1] = -b
    st[..., 2] = -c
    L = np.ascontiguousarray(sc.left[y0:y0 + h, x0:x0 + w])
    R = np.ascontiguousarray(sc.right[y0:y0 + h, x0:x0 + w])
    return L, R, st


def _cases():
    """A 64x64 crop of a 640x480 scene and a 1242-wide band of the
    1242x375 scene (tap positions up to x' ~ 1240)."""
    sc1 = scenes.make_scene(640, 480, 8, 64.0, seed=4000)
    sc2 = scenes.config_scene(2, 0)
    return [("crop64", _crop_states(sc1, 300, 200, 64, 64, 4)),
            ("band1242x48", _crop_states(sc2, 0, 160, 1242, 48, 7))]


def _rel(c32, c64, edge):
    ok = (c64 < 1e4) & ~edge
    return np.abs(c32.astype(np.float64) - c64)[ok] / np.abs(c64[ok]), ok


def _numpy_cost_f64(p, L, R, st):
    """Plain-loop FP64 restatement of pmhstereo.cl:170-228 (with the gradient
    images of :785-831), for a few pixels."""
    H, W = L.shape[:2]
    P = p.patchsize

    def gray(img, x, y):
        if x < 0 or y < 0 or x >= W or y >= H:
            return 0.0
        c = img[y, x].astype(np.float64)
        return c[0] * 0.2126 + c[1] * 0.7152 + c[2] * 0.0722

    def grad(img):
        g = np.zeros((H, W, 4))
        for y in range(H):
            for x in range(W):
                B = lambda dx, dy: gray(img, x + dx, y + dy)
                g[y, x] = [(B(1, 0) - B(-1, 0)) * 0.5 + (B(1, -1) - B(-1, -1)) * 0.25 + (B(1, 1) - B(-1, 1)) * 0.25,
                           (B(0, 1) - B(0, -1)) * 0.5 + (B(-1, 1) - B(-1, -1)) * 0.25 + (B(1, 1) - B(1, -1)) * 0.25,
                           B(1, 1) - B(-1, -1), B(-1, 1) - B(1, -1)]
        return g

    g1, g2 = grad(L), grad(R)
    L64, R64 = L.astype(np.float64), R.astype(np.float64)
    out = np.zeros((H, W))
    for cy in range(H):
        for cx in range(W):
            s = st[cy, cx].astype(np.float64)
            ws = ret = 0.0
            for dy in range(-P, P + 1):
                for dx in range(-P, P + 1):
                    qx, qy = cx + dx, cy + dy
                    if not (0 <= qx < W and 0 <= qy < H):
                        continue
                    d = np.abs(L64[cy, cx, :3] - L64[qy, qx, :3]).sum()
                    ln = np.hypot(dx, dy)
                    t = min(max(ln / 26.0, 0.0), 1.0)
                    prof = t * t * (3 - 2 * t) * 1.5 * p.color_weight + 5.0
                    w = np.exp(-d * prof)
                    xp = s[0] * qx + s[1] * qy + s[2]
                    if not (0.0 <= xp < W):
                        continue
                    ws += w
                    i = int(np.floor(xp))
                    a = xp - i
                    i0, i1 = min(max(i, 0), W - 1), min(max(i + 1, 0), W - 1)
                    v = (1 - a) * R64[qy, i0, :3] + a * R64[qy, i1, :3]
                    u = (1 - a) * g2[qy, i0] + a * g2[qy, i1]
                    cc = np.minimum(np.abs(L64[qy, qx, :3] - v), p.color_maxdiff).sum()
                    gc = np.minimum(np.abs(g1[qy, qx] - u), p.grad_maxdiff).sum()
                    ret += w * (p.color_alpha * cc + (1 - p.color_alpha) * gc)
            out[cy, cx] = 1e5 if ws <= 1.1 else ret / ws
    return out


def test_fp64_evaluator_matches_numpy_restatement(oracle):
    sc = scenes.make_scene(24, 14, 3, 6.0, seed=5)
    L, R, st = _crop_states(sc, 0, 0, 24, 14, 9)
    p = default_params(PRESET_REFERENCE, patchsize=4)
    got, _ = oracle.cost_field_f64(p, L, R, st)
    want = _numpy_cost_f64(p, L, R, st)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE])
def test_fast_cost_within_1e5_of_fp64(oracle, preset):
    for name, (L, R, st) in _cases():
        c64, edge = oracle.cost_field_f64(default_params(preset), L, R, st, eps=1e-3)
        c32 = oracle.cost_field(default_params(preset, arith=ARITH_FAST), L, R, st)
        rel, ok = _rel(c32, c64, edge)
        assert ok.mean() > 0.9, name
        assert rel.max() < TOL_FAST, (name, rel.max())
        # the 1e5 decisions (weight sum <= 1.1) agree wherever the FP64 sum is clear of the threshold
        assert np.array_equal((c32 >= 1e4)[~edge], (c64 >= 1e4)[~edge]), name


@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE])
def test_reference_order_cost_error_vs_fp64(oracle, preset):
    """The reference's operation order: median error ~1e-6, the worst pixels
    of a 1242-wide image a few 1e-4 (x' rounded to FP32)."""
    for name, (L, R, st) in _cases():
        c64, edge = oracle.cost_field_f64(default_params(preset), L, R, st, eps=1e-3)
        c32 = oracle.cost_field(default_params(preset, arith=ARITH_EXACT), L, R, st)
        rel, _ = _rel(c32, c64, edge)
        assert np.median(rel) < 3e-6, name
        assert rel.max() < 2e-3, (name, rel.max())


@pytest.mark.gpu
@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE])
def test_gpu_cost_within_1e5_of_fp64(oracle, cuda, preset):
    import torch
    from cvt_gb300.stereo import PMHuberStereo
    ctx = PMHuberStereo(0)
    for name, (L, R, st) in _cases():
        c64, edge = oracle.cost_field_f64(default_params(preset), L, R, st, eps=1e-3)
        ctx.set_params(default_params(preset, arith=ARITH_FAST))
        got = ctx.cost(torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda(), torch.from_numpy(st).cuda())
        c32 = got.cpu().numpy()
        rel, ok = _rel(c32, c64, edge)
        assert ok.mean() > 0.9, name
        assert rel.max() < TOL_FAST, (name, rel.max())
