"""Stereo rectification on the GPU: the undistort-rectify warp maps and
IWarp::apply's four samplers against the oracle (live, same host) and the
reference's golden outputs, and a rectified pair through depthMap."""
import os

import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import imageio, rectify, scenes
from cvt_gb300.params import default_params, PRESET_REFERENCE

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "rect_reference_golden.npz")
CASES = ("horizontal", "vertical", "large_rotation", "baseline_left")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def cams(G):
    return tuple({k: G[f"{c}_{k}"] for k in ("K", "radial", "tangential")} for c in ("cam0", "cam1"))


@pytest.mark.parametrize("case", CASES)
def test_maps_match_oracle_and_reference(cuda, oracle, G, case):
    c0, c1 = cams(G)
    E, vertical = G[f"rect_{case}_extrinsics"], bool(G[f"rect_{case}_vertical"])
    r = rectify.StereoRectification(c0, c1, E, 64, 48, vertical)
    torch.cuda.synchronize()
    m0, m1 = r.maps[0].cpu().numpy(), r.maps[1].cpu().numpy()
    want = oracle.stereo_rectify(c0, c1, E, vertical, 64, 48)       # this host's C library
    assert not bit_diff(m0, want["map0"]).any() and not bit_diff(m1, want["map1"]).any()
    # the reference's maps were made on another host: its sinf/cosf/acosf may
    # round the rectifying rotation differently by an ulp; the maps then stay
    # within a relative 1e-5
    for got, ref in ((m0, G[f"rect_{case}_map0"]), (m1, G[f"rect_{case}_map1"])):
        fin = np.isfinite(ref)
        assert (np.isfinite(got) == fin).all()
        assert np.allclose(got[fin], ref[fin], rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("name", ["gray_float", "rgba_float", "gray_u8", "rgba_u8"])
def test_warp_matches_reference(cuda, G, name):
    fmt = int(G[f"warp_{name}_fmt"])
    src = torch.from_numpy(G[f"warp_{name}_src"]).cuda()
    m = torch.from_numpy(G[f"warp_{name}_map"]).cuda()
    got = rectify.warp_apply(src, fmt, m).cpu().numpy()
    assert not bit_diff(got, G[f"warp_{name}_dst"]).any()


@pytest.mark.parametrize("fmt", [imageio.BGRA_FLOAT, imageio.BGRA_UINT8, imageio.GRAY_FLOAT, imageio.GRAY_UINT8])
def test_warp_matches_oracle_padded(cuda, oracle, fmt):
    rng = np.random.default_rng(fmt)
    c, dt = imageio.fmt_info(fmt)
    shape = (53, 77) + ((c,) if c > 1 else ())
    src = rng.random(shape, dtype=np.float32) if dt == np.float32 else rng.integers(0, 256, shape, dtype=np.uint8)
    m = np.stack([rng.uniform(-2, 79, (41, 66)), rng.uniform(-2, 55, (41, 66))], -1).astype(np.float32)
    m[0, :5] = [[-0.0, 1.0], [-1.0, -1.0], [76.0, 52.0], [76.5, 52.5], [np.inf, 3.0]]
    # the source with padded rows
    t = torch.zeros((53, 100) + shape[2:], dtype=torch.float32 if dt == np.float32 else torch.uint8, device="cuda")
    t[:, :77] = torch.from_numpy(src).cuda()
    got = rectify.warp_apply(t[:, :77], fmt, torch.from_numpy(m).cuda()).cpu().numpy()
    assert not bit_diff(got, oracle.warp(fmt, src, m)).any()


def test_rectified_pair_through_depthmap(cuda, oracle):
    """A uint8 pair rectified on the GPU and run through depthMap gives the
    oracle's disparities on the oracle's rectification of the same pair."""
    from cvt_gb300.stereo import PMHuberStereo
    sc = scenes.make_scene(72, 48, 3, 10.0, seed=31)
    lu8 = np.ascontiguousarray(np.round(sc.left * 255).astype(np.uint8))
    ru8 = np.ascontiguousarray(np.round(sc.right * 255).astype(np.uint8))
    K = np.array([[60.0, 0, 35.5], [0, 60.0, 23.5], [0, 0, 1]], np.float32)
    c0 = {"K": K, "radial": np.array([-0.02, 0.0, 0.0], np.float32), "tangential": np.zeros(2, np.float32)}
    c1 = {"K": K, "radial": np.array([-0.015, 0.0, 0.0], np.float32), "tangential": np.zeros(2, np.float32)}
    E = np.eye(4, dtype=np.float32)
    E[0, 1], E[1, 0] = -0.004, 0.004
    E[0, 3] = -0.1
    r = rectify.StereoRectification(c0, c1, E, 72, 48)
    lr = r.undistortLeft(torch.from_numpy(lu8).cuda(), imageio.RGBA_UINT8)
    rr = r.undistortRight(torch.from_numpy(ru8).cuda(), imageio.RGBA_UINT8)
    p = default_params(PRESET_REFERENCE, patchsize=5, depthmax=10.0, iterations=2)
    st = PMHuberStereo(0, p)
    d = st.depthMapImage(None, lr, imageio.RGBA_UINT8, rr, imageio.RGBA_UINT8, 5, 10.0, 2, 4)
    torch.cuda.synchronize()
    want_r = oracle.stereo_rectify(c0, c1, E, 0, 72, 48)
    ol = oracle.warp(imageio.RGBA_UINT8, lu8, want_r["map0"])
    orr = oracle.warp(imageio.RGBA_UINT8, ru8, want_r["map1"])
    assert not bit_diff(lr.cpu().numpy(), ol).any() and not bit_diff(rr.cpu().numpy(), orr).any()
    want, _ = oracle.depthmap(p, oracle.image_to_rgbaf(ol, imageio.RGBA_UINT8),
                              oracle.image_to_rgbaf(orr, imageio.RGBA_UINT8))
    assert not bit_diff(d.cpu().numpy(), want).any()
