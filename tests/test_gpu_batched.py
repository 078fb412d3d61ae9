"""cvtpm_depthmap_batched: many pairs of uneven size and disparity range in
one captured graph.  Every pair's disparity map must be bit-identical to the
plain per-pair cvtpm_depthmap with the same parameters: in the default
phase-batched mode (one launch per phase for all pairs, autotuned or with
every pinned combination of launch knobs, more pairs than one launch holds,
PD step counts even, odd and zero), on graph replays, and in the lane mode
with fixed lane counts."""
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
    # the tuner timed both modes and kept the faster
    modes = info["mode_ms"]
    assert modes["phase_batched"] > 0 and modes["one_lane"] > 0
    phased = bool(np.float32(modes["phase_batched"]) < np.float32(0.97) * np.float32(modes["one_lane"]))
    assert (info["phased"], info["lanes"]) == ((1, 0) if phased else (0, 1))
    assert info["grid_mult"] in (0, 1, 2) and info["pd_rows"] in (8, 16) and info["pd_halo"] in (2, 4)
    assert len(info["candidates"]) == 11 and all(c["proxy_ms"] > 0 for c in info["candidates"])
    assert info["shared_windows"] == 1
    if phased:
        # one launch per phase for all pairs: about one plain call's launches, not one call's per pair
        plain.reset_stats()
        plain.depthMap(torch.empty(0, device="cuda"), pairs[0][0], pairs[0][1], p.patchsize, pairs[0][2], p.iterations, 4)
        torch.cuda.synchronize()
        assert 0 < info["launches"] <= 2 * plain.stats()["launches"] < len(pairs) * plain.stats()["launches"]


def test_phased_tuned_knobs_match_plain(cuda):
    """The phase-batched graph with the knobs the tuner chose, pinned on a
    second context so that the phase-batched mode runs whichever mode the
    tuner's proxy preferred."""
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(PRESET_BASELINE, patchsize=5, iterations=2, pd_iterations=6)
    pairs = _pairs(SIZES[:4], seed0=600)
    want = _plain(PMHuberStereo(0, p), pairs, p)
    bat = PMHuberStereo(0, p)
    got = bat.depthMapBatched(pairs)
    info = bat.batch_info()
    kn = (info["grid_mult"], info["pd_rows"], info["pd_halo"])
    bat2 = PMHuberStereo(0, p)
    bat2.set_batch_knobs(*kn)
    got2 = bat2.depthMapBatched(pairs)
    torch.cuda.synchronize()
    assert bat2.batch_info()["phased"] == 1
    for i, (g, g2, w) in enumerate(zip(got, got2, want)):
        assert not bit_diff(g.cpu().numpy(), w).any(), f"pair {i}"
        assert not bit_diff(g2.cpu().numpy(), w).any(), f"pair {i} (phase-batched, tuned knobs)"


@pytest.mark.parametrize("knobs", [(0, 16, 4), (1, 8, 2), (2, 8, 4), (1, 16, 2)])
@pytest.mark.parametrize("pd_iterations", [0, 7, 12])
def test_phased_knobs_match_plain(cuda, knobs, pd_iterations):
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(PRESET_BASELINE, patchsize=5, iterations=2, pd_iterations=pd_iterations)
    pairs = _pairs(SIZES[:4], seed0=700)
    want = _plain(PMHuberStereo(0, p), pairs, p)
    bat = PMHuberStereo(0, p)
    bat.set_batch_knobs(*knobs)
    got = bat.depthMapBatched(pairs)
    torch.cuda.synchronize()
    info = bat.batch_info()
    assert info["tuned"] == 0 and (info["grid_mult"], info["pd_rows"], info["pd_halo"]) == knobs
    for i, (g, w) in enumerate(zip(got, want)):
        assert not bit_diff(g.cpu().numpy(), w).any(), f"pair {i}"


def test_phased_more_pairs_than_one_launch_holds(cuda):
    """70 small pairs: every phase takes two launches (64 + 6 pairs)."""
    from cvt_gb300.stereo import PMHuberStereo
    p = default_params(PRESET_BASELINE, patchsize=3, iterations=2, pd_iterations=4)
    rng = np.random.default_rng(9)
    sizes = [(int(rng.integers(8, 40)), int(rng.integers(6, 24)), float(rng.choice([4.0, 6.0, 9.0]))) for _ in range(70)]
    pairs = _pairs(sizes, seed0=900)
    want = _plain(PMHuberStereo(0, p), pairs, p)
    bat = PMHuberStereo(0, p)
    bat.set_batch_knobs(1, 16, 4)
    got = bat.depthMapBatched(pairs)
    torch.cuda.synchronize()
    for i, (g, w) in enumerate(zip(got, want)):
        assert not bit_diff(g.cpu().numpy(), w).any(), f"pair {i}"


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
    # a different batch on the same context re-captures, in either mode
    pairs2 = pairs[::-1]
    for lanes in (1, 0):
        bat.set_batch_lanes(lanes)
        got = bat.depthMapBatched(pairs2)
        torch.cuda.synchronize()
        info = bat.batch_info()
        if lanes:
            assert info["phased"] == 0 and info["lanes"] == lanes
        else:                                       # the tuner's faster mode
            m = info["mode_ms"]
            faster = np.float32(m["phase_batched"]) < np.float32(0.97) * np.float32(m["one_lane"])
            assert info["phased"] == (1 if faster else 0)
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
