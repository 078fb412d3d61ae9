"""TSDF fusion on the host (no GPU): the oracle's restatement of the
TSDFVolume kernels against the golden outputs of the reference's own kernels
(tests/golden/make_tsdf_golden.py) and, where the reference sources are
present, against them live; the library's projection product against the
reference's Matrix4 product."""
import ctypes
import os

import numpy as np
import pytest

from cvt_gb300 import _lib, tsdf

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "tsdf_reference_golden.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def test_oracle_kernels_match_golden(oracle, G):
    D, H, W = G["vol_after0"].shape[:3]
    assert same_bits(oracle.tsdf_clear(W, H, D, 0.5), G["clear_w"])
    vol = oracle.tsdf_clear(W, H, D, 0.0)
    for i in range(2):
        oracle.tsdf_add(vol, G[f"depth{i}"], 1.0, G[f"T{i}"], float(G["trunc"]))
        assert same_bits(vol, G[f"vol_after{i}"]), i
    ih, iw = G["raycast_neg"].shape
    assert same_bits(oracle.tsdf_raycast(vol, iw, ih, G["Ti2"], G["T2"], -1.0), G["raycast_neg"])
    assert same_bits(oracle.tsdf_raycast(vol, iw, ih, G["Ti2"], G["T2"], 1.0), G["raycast_pos"])
    assert not G["raycast_pos"].any()          # the reference reports -z * scale, clamped at 0
    for axis, idx in ((0, 13), (1, 9), (2, 11)):
        assert same_bits(oracle.tsdf_slice(vol, axis, idx), G[f"slice{axis}"]), axis


def test_oracle_matrices_and_library_projection(oracle, G):
    K4 = np.eye(4, dtype=np.float32)
    K4[:3, :3] = G["K"]
    for i in range(3):
        T, _ = oracle.tsdf_matrices(G[f"proj{i}"], G["g2w"])
        assert same_bits(T, G[f"T{i}"]), i
        assert same_bits(tsdf.projection(G["K"], G[f"E{i}"]), G[f"proj{i}"]), i
        # the inverse: a restatement of Matrix.cpp (not compiled: it needs Eigen); it inverts
        assert np.allclose(G[f"Ti{i}"] @ G[f"T{i}"], np.eye(4), atol=1e-4)


def test_oracle_matches_reference_kernels_live(oracle):
    from oracle.ref_emu import tsdf as ref
    if not ref.available():
        pytest.skip("reference sources absent")
    rng = np.random.default_rng(99)
    W, H, D = 13, 11, 9
    g2w = np.eye(4, dtype=np.float32)
    g2w[:3, :3] *= 0.1
    g2w[:3, 3] = [-0.6, -0.5, 0.5]
    K4 = np.eye(4, dtype=np.float32)
    K4[:3, :3] = [[20, 0, 10.5], [0, 20, 8.5], [0, 0, 1]]
    for trial in range(4):
        E = np.eye(4, dtype=np.float32)
        E[:3, 3] = rng.normal(0, 0.05, 3)
        proj = ref.mat4_mul(K4, E)
        T, Ti = oracle.tsdf_matrices(proj, g2w)
        assert same_bits(T, ref.mat4_mul(proj, g2w)), trial
        dm = (0.9 + 0.3 * rng.random((18, 22))).astype(np.float32)
        dm[rng.random(dm.shape) < 0.1] = 0.0
        a, b = oracle.tsdf_clear(W, H, D, 0.0), ref.tsdf_clear(W, H, D, 0.0)
        for k in range(3):
            oracle.tsdf_add(a, dm * (1 + 0.02 * k), 1.0, T, 0.15)
            ref.tsdf_add(b, dm * (1 + 0.02 * k), 1.0, T, 0.15)
        assert same_bits(a, b), trial
        for s in (-1.0, 2.0):
            assert same_bits(oracle.tsdf_raycast(a, 22, 18, Ti, T, s), ref.tsdf_raycast(b, 22, 18, Ti, T, s)), trial
        for axis in range(3):
            assert same_bits(oracle.tsdf_slice(a, axis, 3), ref.tsdf_slice(b, axis, 3))


def test_argument_checks():
    L = _lib.lib()
    g = (ctypes.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(16))
    h = ctypes.c_void_p()
    assert L.cvtpm_tsdf_create(ctypes.byref(h), 0, g, 1, 8, 8, 0.1) == 2          # each dimension >= 2
    assert L.cvtpm_tsdf_create(ctypes.byref(h), 0, g, 8, 8, 8, 0.0) == 1          # truncation > 0
    assert L.cvtpm_tsdf_create(None, 0, g, 8, 8, 8, 0.1) == 1
    assert L.cvtpm_tsdf_clear(None, 0.0, None) == 1
    assert "NULL" in L.cvtpm_last_error(None).decode()


def _edge_disparities():
    rng = np.random.default_rng(3)
    d = rng.uniform(-0.1, 1.1, (37, 53)).astype(np.float32)
    d.flat[:8] = [0.0, -0.0, np.nan, np.inf, -np.inf, 1e-30, 0.01 / 64, np.nextafter(np.float32(0.01 / 64), 1)]
    return d


def test_oracle_disparity_to_depth():
    """Vision::disparityToDepthmap restated: float32 products and IEEE
    division, 0 at or below the threshold (NaN included)"""
    from oracle import oracle
    d = _edge_disparities()
    got = oracle.disparity_to_depth(d, 64.0, 525.0, 0.12, 0.01)
    fb = np.float32(525.0) * np.float32(0.12)
    s = d * np.float32(64.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        want = np.where(s > np.float32(0.01), fb / s, np.float32(0.0)).astype(np.float32)
    assert same_bits(got, want)
