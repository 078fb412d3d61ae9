"""cvtpm_polish_planes: Levenberg-Marquardt polishing of a plane field on
its aggregated cost (gradient from the adjoint, Gauss-Newton curvature of the
truncated-L1 terms).  A step is kept only when the cost decreases.

Scene: 320x180, 6 slanted planes, dmax 40; planes from a 5-iteration FAST
depthMap (left view)."""
import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_BASELINE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def field(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    sc = scenes.make_scene(320, 180, 6, 40.0, seed=11)
    p = default_params(PRESET_BASELINE, patchsize=17, depthmax=40.0, iterations=5, maxdispdiff=1.0)
    st = PMHuberStereo(0, p)
    L, R = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    tr = {}
    st.depthMap(None, L, R, 17, 40.0, 5, 4, trace=tr)
    s = tr["states"][0]
    planes = torch.zeros_like(s)
    planes[..., 0], planes[..., 1], planes[..., 2] = 1 - s[..., 0], -s[..., 1], -s[..., 2]
    c0, _, _, _ = st.cost_adjoint(L, R, planes.contiguous(), 1)
    return st, sc, L, R, planes.contiguous(), c0, tr["valid"].bool()


def _disp(planes):
    H, W = planes.shape[:2]
    yy, xx = torch.meshgrid(torch.arange(H, device="cuda"), torch.arange(W, device="cuda"), indexing="ij")
    return planes[..., 0] * xx + planes[..., 1] * yy + planes[..., 2]


def test_zero_steps_is_identity(field):
    st, sc, L, R, planes, c0, _ = field
    pp = planes.clone()
    c = st.polish_planes(L, R, pp, 1, 0)
    torch.cuda.synchronize()
    assert torch.equal(pp, planes)
    assert torch.equal(c, c0)                  # the same cost arithmetic as the adjoint's forward


def test_polish_never_increases_cost_and_reduces_error(field):
    st, sc, L, R, planes, c0, valid = field
    pp = planes.clone()
    c1 = st.polish_planes(L, R, pp, 1, 4)
    torch.cuda.synchronize()
    ok = c0 < 1e4
    assert int(((c1 > c0) & ok).sum()) == 0
    assert float((c1 < c0)[ok].float().mean()) > 0.9
    assert float(c1[ok].mean()) < float(c0[ok].mean())
    gt = torch.from_numpy(sc.disp_left).cuda()
    m = valid & ~torch.from_numpy(sc.occluded).cuda()
    e0 = (_disp(planes) - gt).abs()[m].mean()
    e1 = (_disp(pp) - gt).abs()[m].mean()
    assert float(e1) < float(e0)


def test_polished_cost_lower_in_fp64(field, oracle):
    """The decrease is real, not FP32 rounding: the FP64 cost of the polished
    planes is below that of the original ones on >= 95 % of the improved
    pixels (a tiny decrease can sit within FP32 error)."""
    st, sc, L, R, planes, c0, _ = field
    pp = planes.clone()
    c1 = st.polish_planes(L, R, pp, 1, 4)
    torch.cuda.synchronize()
    p = default_params(PRESET_BASELINE, patchsize=17, depthmax=40.0)
    f0, _, _ = oracle.cost_planes_f64(p, sc.left, sc.right, planes.cpu().numpy().astype(np.float64))
    f1, _, _ = oracle.cost_planes_f64(p, sc.left, sc.right, pp.cpu().numpy().astype(np.float64))
    improved = ((c1 < c0) & (c0 < 1e4)).cpu().numpy() & (f0 < 1e4)
    assert float((f1[improved] < f0[improved]).mean()) >= 0.95
