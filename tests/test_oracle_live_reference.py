"""The oracle against the reference's own code run live on fresh seeded
inputs: cvt/cl/kernel/{pmhstereo,RNG,PDHuberWeighted,fill}.cl and
cvt/vision/PMHuberStereo.cpp compiled for the CPU through the OpenCL-C
emulation (oracle/ref_emu, built by build() where the reference sources are
present).  The golden fixtures pin the oracle on fixed inputs; these tests
draw new sizes, windows, disparity ranges, iteration counts and plane fields
per seed.  Skipped where the emulated reference was not built."""
import ctypes
import os

import numpy as np
import pytest

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_REFERENCE

from bitcmp import bit_diff

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "libpmref.so")


@pytest.fixture(scope="module")
def R():
    if not os.path.exists(REF):
        pytest.skip("the emulated reference (oracle/_ref/libpmref.so) is not built here")
    L = ctypes.CDLL(REF)
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i, f, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    L.ref_cost_field.argtypes = [f32, f32, i, i, f32, i, f32]
    L.ref_depthmap.argtypes = [f32, f32, i, i, i, f, i, f, f32, vp, vp]
    L.ref_depthmap_inpaint.argtypes = [f32, f32, i, i, i, f, i, f32, vp]
    L.ref_pdrof.argtypes = [f32, f32, f32, i, i, f, i]
    L.ref_weight.argtypes = [f32, i, i, f32]
    return L


def assert_bits(got, want, what):
    got, want = np.ascontiguousarray(got), np.ascontiguousarray(want)
    assert got.shape == want.shape, what
    d = bit_diff(got, want)
    assert not d.any(), f"{what}: {int(d.sum())} of {d.size} values differ"


@pytest.mark.parametrize("seed", [401, 402, 403])
def test_cost_field_live(oracle, R, seed):
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(20, 60)), int(rng.integers(12, 40))
    P = int(rng.choice([2, 4, 7, 11]))
    dmax = float(rng.choice([6.0, 10.0, 16.0]))
    sc = scenes.make_scene(W, H, 3, dmax, seed=seed)
    st = np.zeros((H, W, 4), np.float32)
    pf = sc.plane_field()
    st[..., 0] = 1.0 - pf[..., 0] + rng.normal(0, 0.05, (H, W)).astype(np.float32)
    st[..., 1] = -pf[..., 1] + rng.normal(0, 0.05, (H, W)).astype(np.float32)
    st[..., 2] = -pf[..., 2] + rng.normal(0, 2.0, (H, W)).astype(np.float32)
    want = np.empty((H, W), np.float32)
    R.ref_cost_field(sc.left, sc.right, W, H, st, P, want)
    p = default_params(PRESET_REFERENCE, patchsize=P)
    assert_bits(oracle.cost_field(p, sc.left, sc.right, st), want, f"cost {W}x{H} P={P}")


@pytest.mark.parametrize("seed", [501, 502, 503])
def test_depthmap_live(oracle, R, seed):
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(24, 52)), int(rng.integers(14, 34))
    P = int(rng.choice([3, 5, 8]))
    dmax = float(rng.choice([6.0, 9.0, 12.0]))
    iters = int(rng.integers(2, 7))
    sc = scenes.make_scene(W, H, 3, dmax, seed=seed)
    d = np.empty((H, W), np.float32)
    nm = np.empty((H, W, 4), np.float32)
    s2 = np.empty((2, H, W, 4), np.float32)
    rc = R.ref_depthmap(sc.left, sc.right, W, H, P, dmax, iters, -1.0, d, nm.ctypes.data, s2.ctypes.data)
    assert rc == 0, rc
    p = default_params(PRESET_REFERENCE, patchsize=P, depthmax=dmax, iterations=iters)
    dmap, ex = oracle.depthmap(p, sc.left, sc.right, normalmap=True, trace=True)
    what = f"{W}x{H} P={P} dmax={dmax} iterations={iters}"
    assert_bits(ex["states"], s2, "states " + what)
    assert_bits(dmap, d, "dmap " + what)
    assert_bits(ex["normalmap"], nm, "normalmap " + what)


@pytest.mark.parametrize("seed", [601, 602])
def test_depthmap_inpaint_live(oracle, R, seed):
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(24, 48)), int(rng.integers(14, 30))
    P = int(rng.choice([3, 5, 7]))
    dmax = float(rng.choice([6.0, 9.0, 12.0]))
    iters = int(rng.integers(2, 7))
    sc = scenes.make_scene(W, H, 3, dmax, seed=seed)
    d = np.empty((H, W), np.float32)
    s2 = np.empty((2, H, W, 4), np.float32)
    rc = R.ref_depthmap_inpaint(sc.left, sc.right, W, H, P, dmax, iters, d, s2.ctypes.data)
    assert rc == 0, rc
    p = default_params(PRESET_REFERENCE, patchsize=P, depthmax=dmax, iterations=iters)
    dmap, ex = oracle.depthmap_inpaint(p, sc.left, sc.right, trace=True)
    what = f"{W}x{H} P={P} dmax={dmax} iterations={iters}"
    assert_bits(ex["states"], s2, "states " + what)
    assert_bits(dmap, d, "dmap " + what)


@pytest.mark.parametrize("seed,steps,lam", [(701, 9, 5.0), (702, 30, 12.5)])
def test_pdrof_live(oracle, R, seed, steps, lam):
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(16, 50)), int(rng.integers(10, 40))
    img = scenes.make_scene(W, H, 2, 8.0, seed=seed).left
    w = np.empty((H, W), np.float32)
    R.ref_weight(img, W, H, w)
    fin = np.zeros((H, W, 4), np.float32)
    fin[..., :3] = rng.normal(0, 0.3, (H, W, 3))
    fin[..., 3] = 1.0
    u0 = np.zeros((H, W, 4), np.float32)
    u0[..., :3] = rng.normal(0, 0.3, (H, W, 3))
    want = u0.copy()
    R.ref_pdrof(want, fin, w, W, H, lam, steps)
    got = oracle.pd_apply(u0.copy(), fin, w, lam, steps)
    assert_bits(got, want, f"PDROF {W}x{H} {steps} steps")
