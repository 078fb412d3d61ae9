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
