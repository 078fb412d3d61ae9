"""Generate tests/golden/png_reference_golden.npz from the reference itself.

The PNG saver (plugins/isaver/PNG/PNGSaver.cpp) converts float images to
8 bits with Image::convert before writing them; the conversions are
SIMD::Conv_GRAYf_to_GRAYu8 (the float-to-sRGB table), SIMD::Conv_f_to_u8
and SIMD::Conv_XXXAf_to_XXXAu8 (cvt/util/SIMD.cpp), compiled from the
reference's sources by oracle/ref_emu/build_ref.py (build_rect).  The
fixture holds a float sweep (every table step, both sides of each step
boundary, values below 0 and above 1, random values) and the three
conversions' outputs:

  x            float32 samples (a multiple of 4)
  gray         Conv_GRAYf_to_GRAYu8(x)
  grayalpha    Conv_f_to_u8(x)
  rgba         Conv_XXXAf_to_XXXAu8(x) (x read as RGBA pixels)

Run in the container that holds the reference:
    python tests/golden/make_png_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_emu import rect  # noqa: E402

OUT = os.path.join(HERE, "png_reference_golden.npz")


def samples() -> np.ndarray:
    i = np.arange(-8, 8200, dtype=np.float64)
    steps = (i / 8192.0).astype(np.float32)
    below = np.nextafter(steps, np.float32(-np.inf))
    mid = ((i + 0.5) / 8192.0).astype(np.float32)
    k = np.arange(-2, 260, dtype=np.float64)
    lin = ((k - 0.5) / 255.0).astype(np.float32)
    lin2 = np.nextafter(lin, np.float32(np.inf))
    rng = np.random.default_rng(7)
    rnd = rng.uniform(-0.2, 1.2, 4096).astype(np.float32)
    special = np.array([0.0, -0.0, 1.0, np.nextafter(np.float32(1), np.float32(0)), 1.5, -1.5, 1e-30, -1e-30,
                        2.0, 100.0, -100.0], np.float32)
    x = np.concatenate([steps, below, mid, lin, lin2, rnd, special])
    pad = (-x.size) % 4
    return np.concatenate([x, np.zeros(pad, np.float32)])


def main():
    if not rect.available():
        raise SystemExit("reference sources absent")
    x = samples()
    np.savez_compressed(OUT, x=x, gray=rect.conv_f_u8(0, x), grayalpha=rect.conv_f_u8(1, x),
                        rgba=rect.conv_f_u8(2, x))
    print("wrote", OUT, x.size, "samples")


if __name__ == "__main__":
    main()
