"""Generate tests/golden/gcv_reference_golden.npz from the reference itself.

cvt::StereoGCVFilter's kernels (cvt/cl/kernel/stereogcv, prefixsum,
boxfilter, guidedfilter, gradx, fill) run through the OpenCL emulation in
oracle/ref_emu with the launch sequence of StereoGCVFilter::depthmap / apply
(oracle/ref_emu/ref_harness.cpp).  Cases: apply() on a 48 x 32 pair (sizes
multiples of the 16-pixel scan blocks: the block fix-up's edge rows run) and
a 37 x 29 pair (ragged blocks); depthmap() with a fractional step and with a
descending range (dmin > dmax: the reference flips dt).  Inputs are the
seeded synthetic scenes of cvt_gb300/scenes.py with the right image as cam0
and the left as cam1 (the map then belongs to the left view).

Run in the container that holds the reference:
    python tests/golden/make_gcv_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cvt_gb300 import scenes  # noqa: E402
from oracle.ref_emu import gcv  # noqa: E402

OUT = os.path.join(HERE, "gcv_reference_golden.npz")

# (name, kind, W, H, planes, scene dmax, seed, dmin, dmax, dt)
CASES = [
    ("apply_a", "apply", 48, 32, 3, 8.0, 51, 0.0, 8.0, 1.0),
    ("apply_b", "apply", 37, 29, 2, 6.0, 52, 0.0, 6.0, 1.0),
    ("dm_frac", "depthmap", 40, 24, 2, 6.0, 53, 0.0, 6.0, 0.75),
    ("dm_desc", "depthmap", 53, 31, 3, 7.0, 54, 7.0, 0.0, 1.0),
]


def main():
    if not gcv.available():
        raise SystemExit("the reference sources are not present; cannot generate fixtures")
    out = {}
    for name, kind, W, H, planes, sdmax, seed, dmin, dmax, dt in CASES:
        sc = scenes.make_scene(W, H, planes, sdmax, seed=seed)
        cam0, cam1 = sc.right, sc.left
        out[f"{name}_cam0"], out[f"{name}_cam1"] = cam0, cam1
        out[f"{name}_args"] = np.array([dmin, dmax, dt], np.float32)
        if kind == "apply":
            o, d0, d1 = gcv.apply(cam0, cam1, dmin, dmax, dt)
            out[f"{name}_out"], out[f"{name}_d0"], out[f"{name}_d1"] = o, d0, d1
        else:
            out[f"{name}_d0"] = gcv.depthmap(cam0, cam1, dmin, dmax, dt)
        print(name, "done", flush=True)
    np.savez_compressed(OUT, **out)
    print(OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
