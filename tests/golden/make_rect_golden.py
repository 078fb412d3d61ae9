"""Generate tests/golden/rect_reference_golden.npz from the reference itself.

The reference's StereoCameraCalibration (cvt/vision/StereoCameraCalibration.h,
with cvt/math underneath) and SIMD::warpBilinear* (cvt/util/SIMD.cpp) are
compiled from their sources by oracle/ref_emu/build_ref.py (build_rect) and
run on seeded calibrations and images.  The fixtures hold the inputs and the
reference's outputs:

  rect_<case>   StereoCameraCalibration(first, second, extrinsics)
                .undistortRectify on 64 x 48 maps: both maps, the rectified
                intrinsics and extrinsics, the rectifying rotations.  Cases:
                a horizontal rig, the same with `vertical`, a rig whose
                relative rotation exceeds 120 degrees (the quaternion's
                trace <= 0 branch) and a rig with its baseline to the left.
  warp_<fmt>    IWarp::apply of a 60 x 40 image in GRAY_FLOAT, RGBA_FLOAT,
                GRAY_UINT8 and RGBA_UINT8 through a map mixing rectification
                coordinates, noise, the border band and edge values (-0, -1,
                negative integers, beyond the image, NaN).

Run in the container that holds the reference:
    python tests/golden/make_rect_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_emu import rect  # noqa: E402

OUT = os.path.join(HERE, "rect_reference_golden.npz")
W, H = 64, 48


def rotation(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * k @ k


def extrinsics(axis, angle, t):
    E = np.eye(4)
    E[:3, :3] = rotation(axis, angle)
    E[:3, 3] = t
    return E.astype(np.float32)


CAM0 = {"K": np.array([[52.0, 0, 32.2], [0, 51.8, 24.1], [0, 0, 1]], np.float32),
        "radial": np.array([-0.21, 0.05, 0.001], np.float32), "tangential": np.array([0.0012, -0.0008], np.float32)}
CAM1 = {"K": np.array([[51.5, 0, 31.8], [0, 51.6, 23.8], [0, 0, 1]], np.float32),
        "radial": np.array([-0.19, 0.04, 0.0], np.float32), "tangential": np.array([-0.0005, 0.0007], np.float32)}

# (name, extrinsics, vertical)
CASES = [
    ("horizontal", extrinsics([0.1, 1.0, 0.05], 0.03, [-0.12, 0.004, 0.002]), 0),
    ("vertical", extrinsics([1.0, 0.1, 0.05], 0.02, [0.003, -0.11, 0.001]), 1),
    ("large_rotation", extrinsics([0.2, 1.0, 0.3], 2.3, [-0.1, 0.02, 0.01]), 0),
    ("baseline_left", extrinsics([0.05, 1.0, 0.02], -0.05, [0.15, -0.01, 0.003]), 0),
]

FORMATS = [("gray_float", 4), ("rgba_float", 12), ("gray_u8", 1), ("rgba_u8", 9)]


def warp_map(base, seed):
    rng = np.random.default_rng(seed)
    m = (0.9 * base + rng.normal(0.0, 6.0, base.shape)).astype(np.float32)
    edge = np.array([[-0.0, 5.5], [-1.0, 3.25], [-2.0, 7.0], [-0.5, -0.75], [59.5, 39.25], [59.0, 10.0],
                     [60.0, 12.0], [70.0, 20.0], [12.0, -1.0], [13.5, 39.99], [np.nan, 4.0], [1e12, 2.0]],
                    np.float32)
    m[0, :len(edge)] = edge
    return m


def main():
    if not rect.available():
        raise SystemExit("the reference sources are not present; cannot generate fixtures")
    out = {}
    for name, E, vertical in CASES:
        r = rect.stereo_rectify(CAM0, CAM1, E, vertical, W, H)
        out[f"rect_{name}_extrinsics"] = E      # input; the rectified extrinsics are rect_<case>_E
        out[f"rect_{name}_vertical"] = np.int32(vertical)
        for k, v in r.items():
            out[f"rect_{name}_{k}"] = v
    for c, cam in (("cam0", CAM0), ("cam1", CAM1)):
        for k, v in cam.items():
            out[f"{c}_{k}"] = v
    base = out["rect_horizontal_map0"]
    rng = np.random.default_rng(7)
    for name, fmt in FORMATS:
        if fmt in (4, 12):
            src = rng.random((40, 60) + ((4,) if fmt == 12 else ()), dtype=np.float32)
        else:
            src = rng.integers(0, 256, (40, 60) + ((4,) if fmt == 9 else ()), dtype=np.uint8)
        m = warp_map(base, fmt)
        out[f"warp_{name}_src"] = src
        out[f"warp_{name}_map"] = m
        out[f"warp_{name}_fmt"] = np.int32(fmt)
        out[f"warp_{name}_dst"] = rect.warp(fmt, src, m)
    np.savez_compressed(OUT, **out)
    print(OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
