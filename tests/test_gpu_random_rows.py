"""Seeded random configurations of the rows beside the plain depthMap, on
the GPU against the oracle, bit for bit: depthMapInpaint (presets,
arithmetics, RNGs, windows, PD steps), StereoGCVFilter::apply (sizes from
2 x 2, ascending, descending and fractional disparity steps, batch sizes),
TSDF integration and ray cast (volume shapes, grid-to-world maps, poses,
truncations, empty depth pixels) and IWarp::apply's four samplers (maps
reaching outside the source, NaN entries)."""
import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import gcv, imageio, rectify, scenes, tsdf
from cvt_gb300 import params as P

pytestmark = pytest.mark.gpu


def test_inpaint_random(cuda, oracle):
    from cvt_gb300.stereo import PMHuberStereo
    rng = np.random.default_rng(31)
    st = PMHuberStereo(0)
    for case in range(8):
        W, H = int(rng.integers(8, 70)), int(rng.integers(4, 50))
        dmax, patch, iters = float(rng.choice([6.0, 12.0, 20.0])), int(rng.integers(1, 12)), int(rng.integers(1, 4))
        p = P.default_params([P.PRESET_REFERENCE, P.PRESET_BASELINE][int(rng.integers(2))],
                             arith=[P.ARITH_EXACT, P.ARITH_FAST][int(rng.integers(2))],
                             rng=[P.RNG_MWC64X, P.RNG_PHILOX][int(rng.integers(2))], patchsize=patch,
                             depthmax=dmax, iterations=iters, pd_iterations=int(rng.integers(1, 30)),
                             seed=int(rng.integers(1 << 30)))
        sc = scenes.make_scene(W, H, 2, dmax, seed=int(rng.integers(1 << 20)))
        st.set_params(p)
        dm = torch.empty(0, device="cuda")
        st.depthMapInpaint(dm, torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), patch, dmax,
                           iters, 4)
        torch.cuda.synchronize()
        want, _ = oracle.depthmap_inpaint(p, sc.left, sc.right)
        assert not bit_diff(dm.cpu().numpy(), want).any(), (case, W, H)


def test_gcv_random(cuda, oracle):
    rng = np.random.default_rng(32)
    try:
        for case in range(8):
            W, H = int(rng.integers(2, 70)), int(rng.integers(2, 50))
            dmin, dmax = float(rng.choice([0.0, 1.0, 3.5, 9.0])), float(rng.choice([0.0, 4.0, 7.25, 12.0]))
            if dmin == dmax:
                dmax += 2.0
            dt = float(rng.choice([0.5, 1.0, 1.25]))
            sc = scenes.make_scene(W, H, 2, 12.0, seed=int(rng.integers(1 << 20)))
            gcv.set_batch(int(rng.choice([0, 1, 3, 5])))
            got = gcv.StereoGCVFilter().apply(torch.from_numpy(sc.right).cuda(), torch.from_numpy(sc.left).cuda(),
                                              dmin, dmax, dt)
            out, d0, d1 = (t.cpu().numpy() for t in got)
            wo, w0, w1 = oracle.gcv_apply(sc.right, sc.left, dmin, dmax, dt)
            assert not bit_diff(d0, w0).any() and not bit_diff(d1, w1).any(), (case, W, H, dmin, dmax, dt)
            assert np.array_equal(out, wo), (case, W, H)
    finally:
        gcv.set_batch(0)


def test_tsdf_random(cuda, oracle):
    rng = np.random.default_rng(33)
    for case in range(6):
        Wv, Hv, Dv = (int(v) for v in rng.integers(2, 30, 3))
        g2w = np.eye(4, dtype=np.float32)
        g2w[:3, :3] *= rng.uniform(0.02, 0.1)
        g2w[:3, 3] = rng.uniform(-1, 1, 3)
        K = np.array([[rng.uniform(20, 60), 0, 16], [0, rng.uniform(20, 60), 12], [0, 0, 1]], np.float32)
        E = np.eye(4, dtype=np.float32)
        E[:3, 3] = rng.normal(0, 0.1, 3)
        dmap = rng.uniform(0.3, 3.0, (24, 32)).astype(np.float32)
        dmap[rng.random(dmap.shape) < 0.1] = 0.0
        trunc = float(rng.uniform(0.05, 0.4))
        v = tsdf.TSDFVolume(g2w, Wv, Hv, Dv, trunc)
        v.clear()
        v.addDepthMap(K, E, torch.from_numpy(dmap).cuda(), 1.0)
        d = v.rayCastDepthMap(K, E, 32, 24, -1.0)
        torch.cuda.synchronize()
        T, Ti = oracle.tsdf_matrices(tsdf.projection(K, E), g2w)
        want = oracle.tsdf_add(oracle.tsdf_clear(Wv, Hv, Dv), dmap, 1.0, T, trunc)
        assert not bit_diff(v.volume().cpu().numpy(), want).any(), case
        assert not bit_diff(d.cpu().numpy(), oracle.tsdf_raycast(want, 32, 24, Ti, T, -1.0)).any(), case


def test_warp_random(cuda, oracle):
    rng = np.random.default_rng(34)
    for case in range(6):
        sw, sh = int(rng.integers(2, 60)), int(rng.integers(2, 40))
        W, H = int(rng.integers(1, 50)), int(rng.integers(1, 40))
        m = np.stack([rng.uniform(-3, sw + 3, (H, W)), rng.uniform(-3, sh + 3, (H, W))], -1).astype(np.float32)
        m[rng.random((H, W)) < 0.05] = np.nan
        for fmt in (imageio.GRAY_FLOAT, imageio.RGBA_FLOAT, imageio.GRAY_UINT8, imageio.RGBA_UINT8):
            c, dt = imageio.fmt_info(fmt)
            shape = (sh, sw) + ((c,) if c > 1 else ())
            src = rng.random(shape, dtype=np.float32) if dt == np.float32 else rng.integers(0, 256, shape, dtype=np.uint8)
            got = rectify.warp_apply(torch.from_numpy(src).cuda(), fmt, torch.from_numpy(m).cuda())
            torch.cuda.synchronize()
            assert not bit_diff(got.cpu().numpy(), oracle.warp(fmt, src, m)).any(), (case, fmt)
