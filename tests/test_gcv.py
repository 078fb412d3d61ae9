"""The comparison baseline on the host (no GPU): the golden fixtures of
cvt::StereoGCVFilter are what the emulated reference produces now (rerun live
where the reference sources are present), and the maps make sense against
the scenes' ground truth."""
import ctypes
import os

import numpy as np
import pytest

from cvt_gb300 import _lib, scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "gcv_reference_golden.npz")


def test_golden_rerun_live():
    from oracle.ref_emu import gcv
    if not gcv.available():
        pytest.skip("reference sources absent")
    G = np.load(GOLDEN)
    dmin, dmax, dt = (float(v) for v in G["dm_frac_args"])
    d = gcv.depthmap(G["dm_frac_cam0"], G["dm_frac_cam1"], dmin, dmax, dt)
    assert d.tobytes() == G["dm_frac_d0"].tobytes()


def test_golden_maps_are_disparities():
    """The apply case on its scene: the left view (cam1) within 1 px of the
    ground truth on most non-occluded pixels."""
    G = np.load(GOLDEN)
    sc = scenes.make_scene(48, 32, 3, 8.0, seed=51)
    assert np.array_equal(sc.left, G["apply_a_cam1"])
    d = G["apply_a_d0"] * 8.0
    m = ~sc.occluded
    assert (np.abs(d - sc.disp_left)[m] <= 1.0).mean() > 0.8


def test_argument_checks():
    L = _lib.lib()
    assert L.cvtpm_gcv_depthmap(None, 0, None, None, 8, 8, 128, 0.0, 4.0, 1.0, None) == 1
    assert L.cvtpm_gcv_depthmap(16, 32, 16, 16, 1, 8, 16, 0.0, 4.0, 1.0, None) == 2
    assert L.cvtpm_gcv_depthmap(16, 32, 16, 16, 8, 8, 128, 0.0, 4.0, 0.0, None) == 1   # dt = 0
    assert "dt" in L.cvtpm_last_error(None).decode()


def test_batch_plan():
    from cvt_gb300 import gcv
    p = gcv.plan(1242, 375, 0.0, 128.0, 1.0)
    assert p["steps"] == 128 and p["batch"] == 128
    assert p["scratch_bytes"] == 1242 * 375 * (22 + 10 * 128) * 4
    assert p["launches"] == 14 + 9 + 1
    try:
        gcv.set_batch(5)
        p = gcv.plan(1242, 375, 0.0, 128.0, 1.0)
        assert p["batch"] == 5 and p["launches"] == 14 + 9 * 26 + 1
        assert gcv.plan(40, 30, 3.0, 1.0, 1.0)["batch"] == 2          # never more than the steps
        assert gcv.plan(40, 30, 0.0, 1.0, 0.25)["steps"] == 4
    finally:
        gcv.set_batch(0)
    assert gcv.plan(7680, 4320, 0.0, 256.0, 1.0)["batch"] == (4 << 30) // (10 * 4 * 7680 * 4320)
    L = _lib.lib()
    assert L.cvtpm_gcv_set_batch(-1) == 1 and L.cvtpm_gcv_set_batch(257) == 1
    assert L.cvtpm_gcv_plan(1, 8, 0.0, 4.0, 1.0, None, None, None, None) == 2


@pytest.mark.parametrize("name", ["apply_a", "apply_b"])
def test_oracle_apply_matches_golden(oracle, name):
    """the oracle's restatement (oracle/pm_oracle.cpp) against the golden
    outputs of the reference's own kernels"""
    G = np.load(GOLDEN)
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    out, d0, d1 = oracle.gcv_apply(G[f"{name}_cam0"], G[f"{name}_cam1"], dmin, dmax, dt)
    assert d0.tobytes() == G[f"{name}_d0"].tobytes()
    assert d1.tobytes() == G[f"{name}_d1"].tobytes()
    assert np.array_equal(out, G[f"{name}_out"])


@pytest.mark.parametrize("name", ["dm_frac", "dm_desc"])
def test_oracle_depthmap_matches_golden(oracle, name):
    G = np.load(GOLDEN)
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    d = oracle.gcv_depthmap(G[f"{name}_cam0"], G[f"{name}_cam1"], dmin, dmax, dt)
    assert d.tobytes() == G[f"{name}_d0"].tobytes()


def test_oracle_matches_reference_kernels_live(oracle):
    """random sizes on and off the 16-pixel blocks, random steps, against the
    reference's kernels run through the OpenCL emulation"""
    from oracle.ref_emu import gcv
    if not gcv.available():
        pytest.skip("reference sources absent")
    rng = np.random.default_rng(77)
    for W, H, dmin, dmax, dt in ((33, 17, 0.0, 6.0, 1.0), (16, 32, 1.5, 5.0, 0.5), (41, 23, 7.0, 2.0, 1.25)):
        sc = scenes.make_scene(W, H, 2, 6.0, seed=int(rng.integers(1000)))
        want = gcv.depthmap(sc.right, sc.left, dmin, dmax, dt)
        got = oracle.gcv_depthmap(sc.right, sc.left, dmin, dmax, dt)
        assert got.tobytes() == want.tobytes(), (W, H)
