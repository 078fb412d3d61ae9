"""cvtpm_depthmap_resumable: a depthMap run split into a call that stops
before some iteration and saves the state there, and a call that resumes
from that state, gives the bits of the uninterrupted run (disparity map,
final states, winners, validity), whatever the split point: before the first
iteration, before and after the theta ramp starts, at the end.  The saved
state is checked against the oracle at one split point too."""
import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_BASELINE, PRESET_REFERENCE, ARITH_EXACT, RNG_MWC64X, SCHEDULE_REDBLACK

pytestmark = pytest.mark.gpu


def _same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape and not bit_diff(a, b).any(), what


@pytest.mark.parametrize("mode", ["fast-philox", "exact-mwc64x", "redblack"])
def test_split_run_matches_the_whole_run(cuda, mode):
    from cvt_gb300.stereo import PMHuberStereo
    kw = dict(patchsize=5, depthmax=12.0, iterations=8, pd_iterations=10)
    if mode == "exact-mwc64x":
        p = default_params(PRESET_REFERENCE, arith=ARITH_EXACT, rng=RNG_MWC64X, **kw)
    elif mode == "redblack":
        p = default_params(PRESET_BASELINE, schedule=SCHEDULE_REDBLACK, **kw)
    else:
        p = default_params(PRESET_BASELINE, **kw)
    sc = scenes.make_scene(72, 40, 3, 12.0, seed=61)
    L, R = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    st = PMHuberStereo(0, p)
    tw = {}
    whole = st.depthMap(None, L, R, 5, 12.0, 8, 4, trace=tw)
    torch.cuda.synchronize()
    for split in (0, 3, 6, 8):
        d0, chk = st.depthMapResumable(None, L, R, 5, 12.0, 8, stop=split, save=True)
        assert chk["iteration"] == split and (d0 is None) == (split < 8)
        tr = {}
        d1, _ = st.depthMapResumable(None, L, R, 5, 12.0, 8, resume=chk, trace=tr)
        torch.cuda.synchronize()
        _same(d1.cpu(), whole.cpu(), f"dmap, split {split}")
        for k in ("states", "winners", "valid"):
            if split < 8 or k != "winners":         # a resume at the end runs no pass: no winners
                _same(tr[k].cpu(), tw[k].cpu(), f"{k}, split {split}")


def test_saved_state_matches_the_oracle_run(cuda, oracle):
    """the state an 8-iteration run saves before iteration 5 is the oracle's
    final state of a 5-iteration run: theta stays 0 through iteration 5 of
    an 8-iteration run, so both runs' first 5 iterations are the same"""
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(PRESET_BASELINE, patchsize=5, depthmax=12.0, iterations=8, pd_iterations=10)
    sc = scenes.make_scene(64, 36, 3, 12.0, seed=62)
    L, R = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    st = PMHuberStereo(0, p)
    _, chk = st.depthMapResumable(None, L, R, 5, 12.0, 8, stop=5, save=True)
    torch.cuda.synchronize()
    _, ex = oracle.depthmap(p.replace(iterations=5), sc.left, sc.right, trace=True)
    _same(chk["states"].cpu(), ex["states"], "states after 5 iterations")


def test_bad_checkpoints_are_refused(cuda):
    from cvt_gb300 import _lib
    from cvt_gb300.stereo import PMHuberStereo
    st = PMHuberStereo(0, default_params(PRESET_BASELINE, patchsize=3, iterations=2, pd_iterations=2))
    sc = scenes.make_scene(16, 12, 2, 6.0, seed=63)
    L, R = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    bad = {"iteration": 3, "states": torch.zeros((2, 12, 16, 4), device="cuda"),
           "smooth": torch.zeros((2, 12, 16, 4), device="cuda")}
    with pytest.raises(_lib.CvtpmError):
        st.depthMapResumable(None, L, R, 3, 6.0, 2, resume=bad)
    bad["iteration"] = 2
    with pytest.raises(_lib.CvtpmError):                # stop before the resumed iteration
        st.depthMapResumable(None, L, R, 3, 6.0, 2, resume=bad, stop=1)
