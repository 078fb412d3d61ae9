"""cvtpm_depthmap_batched: many pairs of uneven size and disparity range in
one captured graph.  Every pair's disparity map must be bit-identical to the
plain per-pair cvtpm_depthmap with the same parameters, for the autotuned
lane count, on graph replays and for fixed lane counts."""
import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_BASELINE, PRESET_REFERENCE, ARITH_EXACT, RNG_MWC64X

pytestmark = pytest.mark.gpu

SIZES = [(96, 64, 16.0), (150, 70, 24.0), (64, 48, 8.0), (128, 96, 32.0), (40, 30, 6.0), (200, 80, 20.0)]


def _pairs(sizes, seed0=300):
    out = []
    for i, (w, h, dmax) in enumerate(sizes):
        sc = scenes.make_scene(w, h, 3 + i % 4, dmax, seed=seed0 + i)
        out.append((torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), dmax))
    return out


def _plain(st, pairs, p):
    res = []
    for left, right, dmax in pairs:
        d = torch.empty(left.shape[:2], device="cuda")
        st.depthMap(d, left, right, p.patchsize, dmax, p.iterations, 4)
        res.append(d.cpu().numpy())
    return res


@pytest.mark.parametrize("preset", [PRESET_BASELINE, PRESET_REFERENCE])
def test_batched_matches_plain_per_pair(cuda, preset):
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(preset, patchsize=7, iterations=3, pd_iterations=12)
    if preset == PRESET_REFERENCE:
        p = p.replace(arith=ARITH_EXACT, rng=RNG_MWC64X)
    pairs = _pairs(SIZES)
    plain = PMHuberStereo(0, p)
    want = _plain(plain, pairs, p)
    bat = PMHuberStereo(0, p)
    got = None
    for attempt in range(2):                       # capture (after tuning), then replay
        got = bat.depthMapBatched(pairs, outs=got)
        torch.cuda.synchronize()
        for i, (g, w) in enumerate(zip(got, want)):
            assert not bit_diff(g.cpu().numpy(), w).any(), f"pair {i}, call {attempt}"
    info = bat.batch_info()
    assert info["tuned"] == 1 and info["replays"] == 1
    assert info["lanes"] in (1, 2, 4, 8) and len(info["candidates"]) >= 2
    assert info["shared_windows"] == (1 if preset == PRESET_BASELINE else 0)
    assert all(c["proxy_ms"] > 0 for c in info["candidates"])


def test_batched_fixed_lanes_and_changed_batch(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(PRESET_BASELINE, patchsize=5, iterations=2, pd_iterations=6)
    pairs = _pairs(SIZES[:4], seed0=500)
    want = _plain(PMHuberStereo(0, p), pairs, p)
    bat = PMHuberStereo(0, p)
    for lanes in (3, 1):
        bat.set_batch_lanes(lanes)
        got = bat.depthMapBatched(pairs)
        torch.cuda.synchronize()
        assert bat.batch_info()["lanes"] == lanes and bat.batch_info()["tuned"] == 0
        for g, w in zip(got, want):
            assert not bit_diff(g.cpu().numpy(), w).any()
    # a different batch on the same context re-captures
    pairs2 = pairs[::-1]
    got = bat.depthMapBatched(pairs2)
    torch.cuda.synchronize()
    for g, w in zip(got, want[::-1]):
        assert not bit_diff(g.cpu().numpy(), w).any()


def test_batched_rejects_bad_pairs(cuda):
    from cvt_gb300 import _lib
    from cvt_gb300.stereo import PMHuberStereo
    st = PMHuberStereo(0)
    assert _lib.lib().cvtpm_depthmap_batched(st._h, None, 0, None) == 1
    left = torch.zeros((8, 8, 4), device="cuda")
    with pytest.raises(_lib.CvtpmError) as e:
        st.depthMapBatched([(left, left, 0.0)])
    assert e.value.status == 1 and "depthmax" in str(e.value)
