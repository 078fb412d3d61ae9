"""Stereo rectification on the host (no GPU).

The oracle's restatement of StereoCameraCalibration::undistortRectify and
IWarp::apply is pinned against the golden fixtures produced by the
reference's own code (tests/golden/make_rect_golden.py) and, where the
reference sources are present, against that code live on random rigs and
maps.  The library's host half (the rectified calibration) must give the
same bits.
"""
import ctypes
import os

import numpy as np
import pytest

from cvt_gb300 import _lib, imageio, rectify

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rect_reference_golden.npz")
CASES = ("horizontal", "vertical", "large_rotation", "baseline_left")
WARPS = ("gray_float", "rgba_float", "gray_u8", "rgba_u8")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def cams(G):
    return tuple({k: G[f"{c}_{k}"] for k in ("K", "radial", "tangential")} for c in ("cam0", "cam1"))


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("case", CASES)
def test_oracle_rectification_matches_golden(oracle, G, case):
    c0, c1 = cams(G)
    r = oracle.stereo_rectify(c0, c1, G[f"rect_{case}_extrinsics"], int(G[f"rect_{case}_vertical"]), 64, 48)
    for k, v in r.items():
        assert same_bits(v, G[f"rect_{case}_{k}"]), k


@pytest.mark.parametrize("name", WARPS)
def test_oracle_warp_matches_golden(oracle, G, name):
    d = oracle.warp(int(G[f"warp_{name}_fmt"]), G[f"warp_{name}_src"], G[f"warp_{name}_map"])
    assert same_bits(d, G[f"warp_{name}_dst"])


@pytest.mark.parametrize("case", CASES)
def test_library_rectified_calibration_matches_golden(G, case):
    c0, c1 = cams(G)
    r = rectify.rectification(c0, c1, G[f"rect_{case}_extrinsics"], bool(G[f"rect_{case}_vertical"]))
    assert same_bits(r["first"]["K"], G[f"rect_{case}_K0"])
    assert same_bits(r["second"]["K"], G[f"rect_{case}_K1"])
    assert same_bits(r["extrinsics"], G[f"rect_{case}_E"])
    assert same_bits(r["R0"], G[f"rect_{case}_R0"]) and same_bits(r["R1"], G[f"rect_{case}_R1"])
    assert not r["first"]["radial"].any() and not r["second"]["tangential"].any()


def _random_rig(rng):
    def rot(axis, angle):
        a = axis / np.linalg.norm(axis)
        k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * k @ k

    def cam():
        f = rng.uniform(300, 900)
        return {"K": np.array([[f, 0, rng.uniform(200, 400)], [0, f * rng.uniform(0.98, 1.02), rng.uniform(150, 250)],
                               [0, 0, 1]], np.float32),
                "radial": rng.normal(0, [0.2, 0.05, 0.01]).astype(np.float32),
                "tangential": rng.normal(0, 0.002, 2).astype(np.float32)}
    E = np.eye(4)
    E[:3, :3] = rot(rng.normal(size=3), rng.choice([rng.uniform(-0.2, 0.2), rng.uniform(2.1, 3.0)]))
    E[:3, 3] = rng.normal(0, 0.1, 3)
    return cam(), cam(), E.astype(np.float32)


def test_oracle_matches_reference_code_live(oracle):
    from oracle.ref_emu import rect
    if not rect.available():
        pytest.skip("reference sources absent")
    rng = np.random.default_rng(1234)
    for trial in range(12):
        c0, c1, E = _random_rig(rng)
        vertical = trial % 3 == 0
        a = oracle.stereo_rectify(c0, c1, E, vertical, 40, 30)
        b = rect.stereo_rectify(c0, c1, E, vertical, 40, 30)
        for k in a:
            assert same_bits(a[k], b[k]), (trial, k)
    for fmt, shape, dt in ((4, (31, 45), np.float32), (16, (31, 45, 4), np.float32), (1, (31, 45), np.uint8),
                           (13, (31, 45, 4), np.uint8)):
        src = (rng.random(shape, dtype=np.float32) if dt == np.float32
               else rng.integers(0, 256, shape, dtype=np.uint8))
        m = np.stack([rng.uniform(-3, 48, (20, 33)), rng.uniform(-3, 34, (20, 33))], -1).astype(np.float32)
        m[0, :4] = [[-0.0, 2.0], [-4.0, 1.0], [44.0, 30.0], [44.9, 30.9]]
        assert same_bits(oracle.warp(fmt, src, m), rect.warp(fmt, src, m)), fmt


def test_argument_checks():
    L = _lib.lib()
    c = rectify._camera({"K": np.eye(3)})
    E = (ctypes.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(16))
    out = _lib.CvtpmRectification()
    assert L.cvtpm_stereo_rectify(None, ctypes.byref(c), E, 0, ctypes.byref(out), 0, 0, None, None, 0, None) == 1
    bad = rectify._camera({"K": np.full((3, 3), np.nan)})
    assert L.cvtpm_stereo_rectify(ctypes.byref(bad), ctypes.byref(c), E, 0, ctypes.byref(out), 0, 0, None, None, 0,
                                  None) == 1
    # one map without the other, and a pitch below width * 8: refused before any device work
    assert L.cvtpm_stereo_rectify(ctypes.byref(c), ctypes.byref(c), E, 0, ctypes.byref(out), 8, 8, 16, None, 64,
                                  None) == 1
    assert L.cvtpm_stereo_rectify(ctypes.byref(c), ctypes.byref(c), E, 0, ctypes.byref(out), 8, 8, 16, 16, 32,
                                  None) == 1
    # IWarp::apply supports GRAY/RGBA/BGRA float and uint8 only
    img = _lib.CvtpmImage(imageio.GRAY_UINT16, 8, 8, 16, 256)
    assert L.cvtpm_warp_apply(ctypes.byref(img), ctypes.byref(img), 256, 64, None) == 7
    assert "unsupported" in L.cvtpm_last_error(None).decode()
