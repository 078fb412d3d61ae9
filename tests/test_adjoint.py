"""Adjoint of the aggregated ASW cost (cvtpm_cost_adjoint) with respect to
the per-pixel planes (a, b, c) and both images.

Checks:
* the FP64 adjoint of the oracle against FP64 central finite differences;
* the CUDA adjoint (FP32) against the FP64 adjoint and against FP64 finite
  differences;
* the torch.autograd.Function wrapper against the C ABI call.

The cost is piecewise smooth: the linear interpolation has a kink at every
integer sample position, and |.|, the truncations and the sample validity
add more.  A central difference that straddles a kink averages two slopes, so
finite differences are compared only on entries whose +h and -h evaluations
take every branch the same way as the unperturbed one (equal branch
signatures from the FP64 oracle); there the cost is analytic and the central
difference is accurate to O(h^2).  Plane steps: 1e-3 for c (at that step
about 1 % of the pixels cross no kink), 1e-5 for a, b, c (x' moves by h*x);
image steps 1e-6.

Inputs (the 64x64 case): a crop of a 640x480 scene (8 planes, dmax 64), its
ground-truth planes + N(0, 0.01) on a, b and N(0, 1) on c (a, b clamped to
[-0.3, 0.3], c to [0, 64]); upstream gradient dL/dC ~ N(0, 1).
"""
import numpy as np
import pytest

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_REFERENCE, PRESET_BASELINE

TOL = 1e-3


def _case(n=64, seed=4):
    sc = scenes.make_scene(640, 480, 8, 64.0, seed=4000)
    x0, y0 = 300, 200
    L = sc.left[y0:y0 + n, x0:x0 + n].astype(np.float64)
    R = sc.right[y0:y0 + n, x0:x0 + n].astype(np.float64)
    rng = np.random.default_rng(seed)
    pf = sc.plane_field()[y0:y0 + n, x0:x0 + n].astype(np.float64)
    pl = np.zeros((n, n, 4))
    pl[..., 0] = np.clip(pf[..., 0] + rng.normal(0, 0.01, (n, n)), -0.3, 0.3)
    pl[..., 1] = np.clip(pf[..., 1] + rng.normal(0, 0.01, (n, n)), -0.3, 0.3)
    # crop coordinates: d(x, y) = a (x + x0) + b (y + y0) + c0
    c = pf[..., 2] + pf[..., 0] * x0 + pf[..., 1] * y0
    pl[..., 2] = np.clip(c + (pl[..., 0] - pf[..., 0]) * x0 + (pl[..., 1] - pf[..., 1]) * y0
                         + rng.normal(0, 1.0, (n, n)), 0.0, 64.0)
    # the GPU takes FP32 inputs: evaluate the FP64 side on the same values
    L, R, pl = (v.astype(np.float32).astype(np.float64) for v in (L, R, pl))
    g = rng.normal(0, 1, (n, n))
    return L, R, pl, g, rng


def _plane_fd(oracle, p, L, R, pl, k, h):
    C0, _, s0 = oracle.cost_planes_f64(p, L, R, pl)
    pp = pl.copy(); pp[..., k] += h
    pm = pl.copy(); pm[..., k] -= h
    Cp, _, sp = oracle.cost_planes_f64(p, L, R, pp)
    Cm, _, sm = oracle.cost_planes_f64(p, L, R, pm)
    stable = (C0 < 1e4) & (sp == s0) & (sm == s0)
    return (Cp - Cm) / (2 * h), stable


def _image_fd(oracle, p, L, R, pl, g, which, entries, h=1e-6):
    C0, _, s0 = oracle.cost_planes_f64(p, L, R, pl)
    out = []
    for (y, x, ch) in entries:
        img = (L if which == 1 else R).copy()
        img[y, x, ch] += h
        Cp, _, sp = oracle.cost_planes_f64(p, img, R, pl) if which == 1 else oracle.cost_planes_f64(p, L, img, pl)
        img[y, x, ch] -= 2 * h
        Cm, _, sm = oracle.cost_planes_f64(p, img, R, pl) if which == 1 else oracle.cost_planes_f64(p, L, img, pl)
        stable = np.array_equal(sp, s0) and np.array_equal(sm, s0)
        m = C0 < 1e4
        out.append((stable, float((g[m] * (Cp[m] - Cm[m])).sum() / (2 * h))))
    return out


@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE])
def test_fp64_adjoint_matches_fp64_finite_differences(oracle, preset):
    p = default_params(preset)
    L, R, pl, g, rng = _case()
    C, dpl, d1, d2 = oracle.cost_adjoint_f64(p, L, R, pl, g)
    C0, _, _ = oracle.cost_planes_f64(p, L, R, pl)
    assert np.array_equal(C, C0)
    for k, h, min_stable in ((2, 1e-3, 20), (0, 1e-5, 500), (1, 1e-5, 500), (2, 1e-5, 2500)):
        fd, stable = _plane_fd(oracle, p, L, R, pl, k, h)
        assert stable.sum() >= min_stable, (k, h, stable.sum())
        rel = np.abs(g * fd - dpl[..., k])[stable] / np.abs(dpl[..., k])[stable]
        assert rel.max() < TOL, (k, h, rel.max())
    ent = [(int(rng.integers(0, 64)), int(rng.integers(0, 64)), int(rng.integers(0, 3))) for _ in range(12)]
    for which, dimg in ((1, d1), (2, d2)):
        res = _image_fd(oracle, p, L, R, pl, g, which, ent)
        checked = [(fd, dimg[e]) for (st, fd), e in zip(res, ent) if st and dimg[e] != 0.0]
        assert len(checked) >= 8, which
        for fd, ad in checked:
            assert abs(fd - ad) <= TOL * abs(ad), (which, fd, ad)
    assert np.all(dpl[..., 3] == 0) and np.all(d1[..., 3] == 0) and np.all(d2[..., 3] == 0)


def _gpu_adjoint(L, R, pl, g, preset, lr=1):
    import torch
    from cvt_gb300.stereo import PMHuberStereo
    st = PMHuberStereo(0)
    st.set_params(default_params(preset))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    out = st.cost_adjoint(t(L), t(R), t(pl), lr, dcost=t(g))
    return [None if v is None else v.cpu().numpy().astype(np.float64) for v in out]


KINK_EPS = 3e-7     # 2.5x the FP32 error of the gradient images (1.2e-7)


def _close(got, want, amb=None):
    """Every entry that no tap within KINK_EPS of a kink reaches (amb False):
    |got - want| <= 1e-3 |want| + 1e-5 max|want|.  All entries together:
    norm-wise relative error below 5e-3 (FP32 takes the other slope where a
    tap sits within its rounding of a kink)."""
    scale = np.abs(want).max()
    m = np.ones(want.shape[:2], bool) if amb is None else ~amb
    ok = np.abs(got - want)[m] <= TOL * np.abs(want)[m] + 1e-5 * scale
    nrm = np.linalg.norm(got - want) / np.linalg.norm(want)
    return bool(ok.all()) and nrm < 5e-3, (int((~ok).sum()), nrm)


@pytest.mark.gpu
@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE])
@pytest.mark.parametrize("lr", [1, 0])
def test_gpu_adjoint_matches_fp64_adjoint(oracle, cuda, preset, lr):
    p = default_params(preset)
    L, R, pl, g, _ = _case()
    if lr == 0:
        pl = pl.copy()
        pl[..., 2] = -pl[..., 2]            # right view: x_other = x + d with d <= 0 keeps samples inside
    C64, dpl64, d164, d264, amb = oracle.cost_adjoint_f64(p, L, R, pl, g, lr=lr, kink_eps=KINK_EPS)
    C, dpl, d1, d2 = _gpu_adjoint(L, R, pl, g, preset, lr)
    _, edge, _ = oracle.cost_planes_f64(p, L, R, pl, lr=lr)
    ok = (C64 < 1e4) & ~edge
    assert np.abs(C - C64)[ok].max() <= 1e-5 * np.abs(C64[ok]).max()
    assert np.array_equal(C >= 1e4, C64 >= 1e4)
    assert amb[0].mean() < 0.1                       # most plane gradients are unambiguous
    for got, want, m in ((dpl[..., :3], dpl64[..., :3], amb[0]), (d1[..., :3], d164[..., :3], amb[1]),
                         (d2[..., :3], d264[..., :3], amb[2])):
        good, info = _close(got, want, m)
        assert good, info
    assert np.all(dpl[..., 3] == 0) and np.all(d1[..., 3] == 0) and np.all(d2[..., 3] == 0)


@pytest.mark.gpu
def test_gpu_adjoint_matches_fp64_finite_differences(oracle, cuda):
    p = default_params(PRESET_BASELINE)
    L, R, pl, g, rng = _case()
    _, dpl, d1, d2 = _gpu_adjoint(L, R, pl, g, PRESET_BASELINE)
    for k, h in ((2, 1e-3), (0, 1e-5), (1, 1e-5), (2, 1e-5)):
        fd, stable = _plane_fd(oracle, p, L, R, pl, k, h)
        want = (g * fd)[stable]
        rel = np.abs(dpl[..., k][stable] - want) / np.abs(want)
        assert rel.max() < TOL and np.median(rel) < 1e-5, (k, h, rel.max())
    ent = [(int(rng.integers(0, 64)), int(rng.integers(0, 64)), int(rng.integers(0, 3))) for _ in range(12)]
    for which, dimg in ((1, d1), (2, d2)):
        res = _image_fd(oracle, p, L, R, pl, g, which, ent)
        checked = [(fd, dimg[e]) for (st, fd), e in zip(res, ent) if st and fd != 0.0]
        assert len(checked) >= 8
        for fd, ad in checked:
            assert abs(fd - ad) <= TOL * abs(fd), (which, fd, ad)


@pytest.mark.gpu
def test_autograd_function_matches_c_abi(oracle, cuda):
    import torch
    from cvt_gb300.stereo import PMHuberStereo
    from cvt_gb300.autograd import asw_cost
    L, R, pl, g, _ = _case(n=40)
    st = PMHuberStereo(0)
    st.set_params(default_params(PRESET_BASELINE))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    i1, i2, pp, gg = t(L).requires_grad_(), t(R).requires_grad_(), t(pl).requires_grad_(), t(g)
    cost = asw_cost(st, i1, i2, pp, 1)
    (cost * gg).sum().backward()
    C, dpl, d1, d2 = st.cost_adjoint(t(L), t(R), t(pl), 1, dcost=gg)
    assert torch.equal(cost.detach(), C)
    assert torch.equal(pp.grad, dpl)
    # image gradients come from float atomics: equal up to summation order
    for a, b in ((i1.grad, d1), (i2.grad, d2)):
        assert torch.allclose(a, b, rtol=1e-4, atol=1e-6 * float(b.abs().max()))
    _, dpl64, _, _, amb = oracle.cost_adjoint_f64(default_params(PRESET_BASELINE), L, R, pl, g, kink_eps=KINK_EPS)
    good, info = _close(pp.grad.cpu().numpy()[..., :3].astype(np.float64), dpl64[..., :3], amb[0])
    assert good, info


@pytest.mark.gpu
def test_gpu_adjoint_rejects_gradients_without_dcost(cuda):
    import ctypes
    import torch
    from cvt_gb300 import _lib
    from cvt_gb300.stereo import PMHuberStereo
    st = PMHuberStereo(0)
    img = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    out = torch.empty((8, 8), dtype=torch.float32, device="cuda")
    rc = _lib.lib().cvtpm_cost_adjoint(st._h, img.data_ptr(), img.data_ptr(), 8, 8, 8 * 16, img.data_ptr(), 1,
                                       None, out.data_ptr(), img.data_ptr(), None, None, None)
    assert rc == 1                                   # CVTPM_ERR_INVALID_ARGUMENT
