"""TSDF fusion on the GPU through libcvtpm.so, against the golden outputs of
the reference's own kernels: integration of two depth maps, ray casts with
both signs of scale, the slice kernels, clear, saveRaw; and a ray cast from
a camera too far away for its march to advance (bounded, zero)."""
import os

import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import tsdf

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "tsdf_reference_golden.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def _vol(G):
    D, H, W = G["vol_after0"].shape[:3]
    return tsdf.TSDFVolume(G["g2w"], W, H, D, float(G["trunc"]))


def test_fusion_matches_reference(cuda, G):
    v = _vol(G)
    v.clear(0.5)
    assert not bit_diff(v.volume().cpu().numpy(), G["clear_w"]).any()
    v.clear()
    for i in range(2):
        v.addDepthMap(G["K"], G[f"E{i}"], torch.from_numpy(G[f"depth{i}"]).cuda(), 1.0)
        torch.cuda.synchronize()
        assert not bit_diff(v.volume().cpu().numpy(), G[f"vol_after{i}"]).any(), i
    ih, iw = G["raycast_neg"].shape
    for scale, key in ((-1.0, "raycast_neg"), (1.0, "raycast_pos")):
        d = v.rayCastDepthMap(G["K"], G["E2"], iw, ih, scale)
        torch.cuda.synchronize()
        assert not bit_diff(d.cpu().numpy(), G[key]).any(), key
    for axis, idx in ((0, 13), (1, 9), (2, 11)):
        assert not bit_diff(v.slice(axis, idx).cpu().numpy(), G[f"slice{axis}"]).any(), axis


def test_projection_overload_and_save_raw(cuda, G, tmp_path):
    v = _vol(G)
    v.clear()
    v.addDepthMap(G["proj0"], torch.from_numpy(G["depth0"]).cuda(), scale=1.0)   # addDepthMap(proj, dmap, scale)
    torch.cuda.synchronize()
    want = G["vol_after0"]
    assert not bit_diff(v.volume().cpu().numpy(), want).any()
    v.saveRaw(tmp_path / "w.raw", True)
    v.saveRaw(tmp_path / "t.raw", False)
    assert (tmp_path / "w.raw").read_bytes() == want.tobytes()
    assert (tmp_path / "t.raw").read_bytes() == np.ascontiguousarray(want[..., 0]).tobytes()


def test_far_camera_raycast_is_bounded(cuda, G, oracle):
    """A camera 5e7 m (1e9 voxels) away on the volume's diagonal, looking
    along (1, 1, 1): the ray through the principal point enters the volume,
    but lambda + step rounds to lambda at that distance, so the reference's
    float march would not end.  Here every ray stops after its step bound;
    the result equals the oracle's, which has the same bound."""
    v = _vol(G)
    v.clear()
    v.addDepthMap(G["K"], G["E0"], torch.from_numpy(G["depth0"]).cuda(), 1.0)
    z = np.array([1.0, 1.0, 1.0]) / np.sqrt(3.0)
    x = np.array([1.0, -1.0, 0.0]) / np.sqrt(2.0)
    R = np.stack([x, np.cross(z, x), z])
    centre = np.array([0.05, 0.0, 1.2])
    C = centre - 5e7 * z
    E = np.eye(4)
    E[:3, :3] = R
    E[:3, 3] = -R @ C
    K = np.array([[45.0, 0, 8.0], [0, 45.0, 6.0], [0, 0, 1]], np.float32)   # pixel (8, 6) on the axis
    d = v.rayCastDepthMap(K, E.astype(np.float32), 16, 12, -1.0)
    torch.cuda.synchronize()
    proj = tsdf.projection(K, E.astype(np.float32))
    T, Ti = oracle.tsdf_matrices(proj, G["g2w"])
    want = oracle.tsdf_raycast(v.volume().cpu().numpy(), 16, 12, Ti, T, -1.0)
    assert not bit_diff(d.cpu().numpy(), want).any()


def test_disparity_to_depth_matches_oracle(cuda, oracle):
    from cvt_gb300 import vision
    rng = np.random.default_rng(3)
    d = rng.uniform(-0.1, 1.1, (37, 53)).astype(np.float32)
    d.flat[:8] = [0.0, -0.0, np.nan, np.inf, -np.inf, 1e-30, 0.01 / 64, np.nextafter(np.float32(0.01 / 64), 1)]
    for args in ((64.0, 525.0, 0.12, 0.01), (1.0, 700.5, 0.54, 0.0), (128.0, 1.0, -0.3, 0.5)):
        got = vision.disparityToDepthmap(torch.from_numpy(d).cuda(), *args)
        torch.cuda.synchronize()
        assert not bit_diff(got.cpu().numpy(), oracle.disparity_to_depth(d, *args)).any(), args
    # a pitched view of a wider buffer
    wide = torch.zeros((37, 64), device="cuda")
    wide[:, :53] = torch.from_numpy(d).cuda()
    got = vision.disparityToDepthmap(wide[:, :53], 64.0, 525.0, 0.12)
    assert not bit_diff(got.cpu().numpy(), oracle.disparity_to_depth(d, 64.0, 525.0, 0.12)).any()


def test_stereo_to_tsdf_chain_matches_oracle(cuda, oracle):
    """The output side end to end: PatchMatch depthMap of a rectified pair ->
    disparityToDepthmap -> TSDFVolume::addDepthMap, on the GPU and in the
    oracle, volumes bit for bit."""
    from cvt_gb300 import scenes, vision
    from cvt_gb300.params import default_params, PRESET_REFERENCE
    from cvt_gb300.stereo import PMHuberStereo
    W, H, dmax = 64, 48, 12.0
    sc = scenes.make_scene(W, H, 3, dmax, seed=21)
    p = default_params(PRESET_REFERENCE, patchsize=5, depthmax=dmax, iterations=2, pd_iterations=20)
    st = PMHuberStereo(0)
    st.set_params(p)
    dm = torch.empty(0, device="cuda")
    st.depthMap(dm, torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), p.patchsize, dmax,
                p.iterations, 4)
    want_dm, _ = oracle.depthmap(p, sc.left, sc.right)
    assert not bit_diff(dm.cpu().numpy(), want_dm).any()
    f, B = 60.0, 0.1
    depth = vision.disparityToDepthmap(dm, dmax, f, B)
    want_depth = oracle.disparity_to_depth(want_dm, dmax, f, B)
    assert not bit_diff(depth.cpu().numpy(), want_depth).any()
    K = np.array([[f, 0, W / 2 - 0.5], [0, f, H / 2 - 0.5], [0, 0, 1]], np.float32)
    E = np.eye(4, dtype=np.float32)
    g2w = np.eye(4, dtype=np.float32)
    g2w[:3, :3] *= 0.05
    g2w[:3, 3] = [-0.8, -0.6, 0.3]
    v = tsdf.TSDFVolume(g2w, 32, 24, 40, 0.1)
    v.clear()
    v.addDepthMap(K, E, depth, 1.0)
    torch.cuda.synchronize()
    T, _ = oracle.tsdf_matrices(tsdf.projection(K, E), g2w)
    want = oracle.tsdf_add(oracle.tsdf_clear(32, 24, 40), want_depth, 1.0, T, 0.1)
    got = v.volume().cpu().numpy()
    assert not bit_diff(got, want).any()
    assert (got[..., 1] > 0).sum() > 100        # the surface band is populated
