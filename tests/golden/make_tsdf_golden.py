"""Generate tests/golden/tsdf_reference_golden.npz from the reference itself.

The kernels of cvt/cl/kernel/TSDFVolume/TSDFVolume.cl run through the OpenCL
emulation in oracle/ref_emu (build_ref.py) with the launch sizes of
cvt/vision/TSDFVolume.cpp; the projections are formed with the reference's
Matrix4 product (cvt/math/Matrix4.h, through build_ref.build_rect).  The
inverse for the ray cast (Matrix.cpp, which needs Eigen) is the oracle's
restatement.  Scene: a 32 x 28 x 24 grid of 5 cm voxels, a sphere in front
of a tilted plane, depth maps rendered analytically from two poses (64 x 48,
focal 45 px), integrated in order, then ray cast from a third pose with
scale -1 (depth) and +1 (the reference's sign: all zero), and the three
slice kernels at one plane each.

Run in the container that holds the reference:
    python tests/golden/make_tsdf_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from oracle.ref_emu import tsdf as ref  # noqa: E402

OUT = os.path.join(HERE, "tsdf_reference_golden.npz")
W, H, D = 32, 28, 24
IW, IH = 64, 48
TRUNC = 0.12


def pose(angle_y, t):
    c, s = np.cos(angle_y), np.sin(angle_y)
    E = np.eye(4)
    E[:3, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
    E[:3, 3] = t
    return E.astype(np.float32)


def render(K, E):
    """Camera-space depth of the first hit of each pixel's ray with the sphere
    (centre (0.05, 0, 1.0), radius 0.22) or the plane z = 1.25 + 0.2 x."""
    Ki = np.linalg.inv(K.astype(np.float64))
    Ei = np.linalg.inv(E.astype(np.float64))
    v, u = np.mgrid[0:IH, 0:IW].astype(np.float64)
    rays_c = np.stack([u, v, np.ones_like(u)], -1) @ Ki.T         # z = 1 in the camera
    o = Ei[:3, 3]
    dirs = rays_c @ Ei[:3, :3].T
    best = np.full((IH, IW), np.inf)
    c, r = np.array([0.05, 0.0, 1.0]), 0.22
    oc = o - c
    b = dirs @ oc
    a = (dirs * dirs).sum(-1)
    disc = b * b - a * ((oc * oc).sum() - r * r)
    t = (-b - np.sqrt(np.maximum(disc, 0))) / a
    best = np.where((disc > 0) & (t > 0), t, best)
    # plane z - 0.2 x = 1.25
    n = np.array([-0.2, 0.0, 1.0])
    tp = (1.25 - o @ n) / (dirs @ n)
    best = np.where((tp > 0) & (tp < best), tp, best)
    depth = np.where(np.isfinite(best), best, 0.0)                 # t is the camera z (rays have z = 1)
    return depth.astype(np.float32)


def main():
    if not ref.available():
        raise SystemExit("the reference sources are not present; cannot generate fixtures")
    g2w = np.eye(4, dtype=np.float32)
    g2w[:3, :3] *= 0.05
    g2w[:3, 3] = [-0.75, -0.7, 0.6]
    K = np.array([[45.0, 0, 31.5], [0, 45.0, 23.5], [0, 0, 1]], np.float32)
    K4 = np.eye(4, dtype=np.float32)
    K4[:3, :3] = K
    poses = [pose(0.0, [0, 0, 0]), pose(0.12, [-0.1, 0.02, 0.03]), pose(-0.08, [0.06, -0.01, 0.0])]
    out = {"g2w": g2w, "K": K, "trunc": np.float32(TRUNC)}
    vol = ref.tsdf_clear(W, H, D, 0.0)
    for i, E in enumerate(poses):
        proj = ref.mat4_mul(K4, E)                                  # K.toMatrix4() * E
        T = ref.mat4_mul(proj, g2w)                                 # proj * g2w
        _, Ti = orc.tsdf_matrices(proj, g2w)
        out[f"E{i}"], out[f"proj{i}"], out[f"T{i}"], out[f"Ti{i}"] = E, proj, T, Ti
        if i < 2:
            dm = render(K, E)
            out[f"depth{i}"] = dm
            ref.tsdf_add(vol, dm, 1.0, T, TRUNC)
            out[f"vol_after{i}"] = vol.copy()
    out["raycast_neg"] = ref.tsdf_raycast(vol, IW, IH, out["Ti2"], out["T2"], -1.0)
    out["raycast_pos"] = ref.tsdf_raycast(vol, IW, IH, out["Ti2"], out["T2"], 1.0)
    for axis, idx in ((0, 13), (1, 9), (2, 11)):
        out[f"slice{axis}"] = ref.tsdf_slice(vol, axis, idx)
    out["clear_w"] = ref.tsdf_clear(W, H, D, 0.5)
    np.savez_compressed(OUT, **out)
    print(OUT, len(out), "arrays; surface pixels:", int((out["raycast_neg"] > 0).sum()), "of", IW * IH,
          "; updated voxels:", int((vol[..., 1] > 0).sum()))


if __name__ == "__main__":
    main()
