"""Generate tests/golden/pm_reference_golden.npz from the reference itself.

The reference's own sources — cvt/cl/kernel/{pmhstereo,RNG,PDHuberWeighted,fill}.cl
and cvt/vision/PMHuberStereo.cpp with cvt/gfx/PDROF.h — are compiled for the
CPU through the OpenCL-C emulation in oracle/ref_emu (build_ref.py) and run
on small seeded synthetic pairs.  The fixtures record the inputs and the
reference's outputs:

  kernels  gradxy, weight (pmhstereo.cl:737-831), the aggregated cost of a
           fixed plane field (:170-228), init of both views (:230-248),
           PDROF::apply (PDROF.h:50-96) for 250 and 7 steps
  runs     PMHuberStereo::depthMap (PMHuberStereo.cpp:64-291): final states of
           both views, disparity map and normal map
  inpaint  pmhstereo_occmap / pmhstereo_normal_depth (pmhstereo.cl:663-712),
           PDROFInpaint::apply (PDROFInpaint.h:50-98) for 100 and 7 steps, and
           PMHuberStereo::depthMapInpaint (PMHuberStereo.cpp:293-506) runs with
           odd and even iteration counts

Run in the container that holds the reference:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cvt_gb300 import scenes  # noqa: E402
from oracle.ref_emu import build_ref  # noqa: E402

OUT = os.path.join(HERE, "pm_reference_golden.npz")

# (name, W, H, planes, dmax, seed, patchsize, iterations)
RUNS = [
    ("run_a", 56, 40, 3, 12.0, 101, 9, 3),
    ("run_b", 44, 32, 3, 10.0, 102, 17, 7),
    ("run_c", 37, 23, 2, 8.0, 103, 5, 2),
]


# (name, W, H, planes, dmax, seed, patchsize, iterations)
INPAINT_RUNS = [
    ("inp_a", 56, 40, 3, 12.0, 201, 9, 3),
    ("inp_b", 44, 32, 3, 10.0, 202, 7, 6),
]


def load():
    lib = build_ref.build()
    if lib is None:
        raise SystemExit("the reference sources are not present; cannot generate fixtures")
    R = ctypes.CDLL(lib)
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i, f, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    R.ref_gradxy.argtypes = [f32, i, i, f32]
    R.ref_weight.argtypes = [f32, i, i, f32]
    R.ref_cost_field.argtypes = [f32, f32, i, i, f32, i, f32]
    R.ref_init.argtypes = [f32, f32, i, i, i, f, i, f32]
    R.ref_pdrof.argtypes = [f32, f32, f32, i, i, f, i]
    R.ref_depthmap.argtypes = [f32, f32, i, i, i, f, i, f, f32, vp, vp]
    R.ref_depthmap_inpaint.argtypes = [f32, f32, i, i, i, f, i, f32, vp]
    R.ref_occmap.argtypes = [f32, f32, i, i, f, i, f32]
    R.ref_normal_depth.argtypes = [f32, i, i, f, i, f32]
    R.ref_pdrof_inpaint.argtypes = [f32, f32, f32, f32, i, i, f, i]
    return R


def main():
    R = load()
    out = {}
    # ---- kernels on one pair
    sc = scenes.make_scene(61, 43, 4, 14.0, seed=100)
    W, H = sc.width, sc.height
    out["k_left"], out["k_right"] = sc.left, sc.right
    g = np.empty((H, W, 4), np.float32)
    R.ref_gradxy(sc.left, W, H, g)
    out["k_gradxy_left"] = g.copy()
    wl = np.empty((H, W), np.float32)
    R.ref_weight(sc.left, W, H, wl)
    out["k_weight_left"] = wl
    rng = np.random.default_rng(7)
    st = np.zeros((H, W, 4), np.float32)
    pf = sc.plane_field()
    st[..., 0] = 1.0 - pf[..., 0] + rng.normal(0, 0.01, (H, W)).astype(np.float32)
    st[..., 1] = -pf[..., 1] + rng.normal(0, 0.01, (H, W)).astype(np.float32)
    st[..., 2] = -pf[..., 2] + rng.normal(0, 1.0, (H, W)).astype(np.float32)
    out["k_states"] = st
    for P in (17, 6):
        c = np.empty((H, W), np.float32)
        R.ref_cost_field(sc.left, sc.right, W, H, st, P, c)
        out[f"k_cost_p{P}"] = c
    for lr in (1, 0):
        a, b = (sc.left, sc.right) if lr else (sc.right, sc.left)
        o = np.empty((H, W, 4), np.float32)
        R.ref_init(a, b, W, H, 17, 14.0, lr, o)
        out[f"k_init_lr{lr}"] = o
    fin = np.zeros((H, W, 4), np.float32)
    fin[..., :3] = rng.normal(0, 0.3, (H, W, 3))
    fin[..., 3] = 1.0
    u0 = np.zeros((H, W, 4), np.float32)
    u0[..., :3] = rng.normal(0, 0.3, (H, W, 3))
    out["k_pd_input"], out["k_pd_warm"] = fin, u0
    for it, lam in ((250, 5.0), (7, 17.5)):
        u = u0.copy()
        R.ref_pdrof(u, fin, wl, W, H, lam, it)
        out[f"k_pd_{it}"] = u
    # ---- inpaint kernels: the init states of both views, a random mask
    sl, sr = out["k_init_lr1"], out["k_init_lr0"]
    for lr, (a, b) in ((1, (sl, sr)), (0, (sr, sl))):
        o = np.empty((H, W, 4), np.float32)
        R.ref_occmap(a, b, W, H, 0.5, lr, o)
        out[f"k_occmap_lr{lr}"] = o
        nd = np.empty((H, W, 4), np.float32)
        R.ref_normal_depth(a, W, H, 14.0, lr, nd)
        out[f"k_normal_depth_lr{lr}"] = nd
    mask = np.zeros((H, W, 4), np.float32)
    mask[..., :3] = (rng.random((H, W)) < 0.7)[..., None]
    mask[..., 3] = 1.0
    out["k_pdi_mask"] = mask
    for it, lam in ((100, 5.0), (7, 17.5)):
        u = u0.copy()
        R.ref_pdrof_inpaint(u, fin, wl, mask, W, H, lam, it)
        out[f"k_pdi_{it}"] = u
    for name, W2, H2, planes, dmax, seed, P, iters in INPAINT_RUNS:
        sc2 = scenes.make_scene(W2, H2, planes, dmax, seed=seed)
        d = np.empty((H2, W2), np.float32)
        s2 = np.empty((2, H2, W2, 4), np.float32)
        rc = R.ref_depthmap_inpaint(sc2.left, sc2.right, W2, H2, P, dmax, iters, d, s2.ctypes.data)
        assert rc == 0, rc
        out[f"{name}_left"], out[f"{name}_right"] = sc2.left, sc2.right
        out[f"{name}_cfg"] = np.array([W2, H2, P, iters, dmax], np.float64)
        out[f"{name}_dmap"], out[f"{name}_states"] = d, s2
        print(f"{name}: {W2}x{H2} P={P} iterations={iters} done", file=sys.stderr)
    # ---- full runs
    for name, W, H, planes, dmax, seed, P, iters in RUNS:
        sc = scenes.make_scene(W, H, planes, dmax, seed=seed)
        d = np.empty((H, W), np.float32)
        nm = np.empty((H, W, 4), np.float32)
        s2 = np.empty((2, H, W, 4), np.float32)
        rc = R.ref_depthmap(sc.left, sc.right, W, H, P, dmax, iters, -1.0, d, nm.ctypes.data, s2.ctypes.data)
        assert rc == 0, rc
        out[f"{name}_left"], out[f"{name}_right"] = sc.left, sc.right
        out[f"{name}_cfg"] = np.array([W, H, P, iters, dmax], np.float64)
        out[f"{name}_dmap"], out[f"{name}_normalmap"], out[f"{name}_states"] = d, nm, s2
        print(f"{name}: {W}x{H} P={P} iterations={iters} done", file=sys.stderr)
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
