"""Disparity quality of the bench configuration against the reference's own
algorithm, on the 1242x375 synthetic scenes (16 slanted planes, dmax 128,
2 % salt, +/-5 % gain/bias; pairs 0-7, seeds 2000-2007), 8 iterations,
35x35 window, LR threshold 1 px.

The reference's algorithm is EXACT arithmetic + MWC64X, whose full runs are
bit-identical to the reference's code (test_gpu_golden.py).  The bench runs
FAST arithmetic + Philox4x32-10.  Two separate effects:

* arithmetic (same RNG stream): FAST and EXACT end within a few hundredths
  of a percentage point per pair;
* RNG stream: a different stream moves a pair's bad-1px by ~0.3 pp either
  way (a different seed of the same generator does the same), so the claim
  is on the mean over the 8 pairs.
"""
import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import (default_params, PRESET_BASELINE, PRESET_REFERENCE, ARITH_EXACT, ARITH_FAST,
                              RNG_MWC64X, RNG_PHILOX)

pytestmark = pytest.mark.gpu

PAIRS = 8
BAD1_PP = 0.1


def _bad1(ctx, preset, pairs, **kw):
    out = []
    for pair in pairs:
        sc = scenes.config_scene(2, pair)
        L, R = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
        d = torch.empty(sc.left.shape[:2], device="cuda")
        ctx.set_params(default_params(preset, patchsize=17, depthmax=128.0, iterations=8, maxdispdiff=1.0, **kw))
        ctx.depthMap(d, L, R, 17, 128.0, 8, 4)
        out.append(scenes.bad_pixel_rate(d.cpu().numpy() * 128.0, sc))
    return np.array(out)


@pytest.fixture(scope="module")
def ctx(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    return PMHuberStereo(0)


@pytest.mark.parametrize("preset", [PRESET_BASELINE, PRESET_REFERENCE])
def test_fast_arithmetic_keeps_bad1_of_reference_order(ctx, preset):
    pairs = range(4)
    ref = _bad1(ctx, preset, pairs, arith=ARITH_EXACT, rng=RNG_MWC64X)
    fast = _bad1(ctx, preset, pairs, arith=ARITH_FAST, rng=RNG_MWC64X)
    assert np.all(np.abs(fast - ref) < BAD1_PP), (fast, ref)
    assert abs(fast.mean() - ref.mean()) < 0.02, (fast.mean(), ref.mean())


def test_bench_configuration_bad1_within_0p1_of_reference(ctx):
    pairs = range(PAIRS)
    ref = _bad1(ctx, PRESET_BASELINE, pairs, arith=ARITH_EXACT, rng=RNG_MWC64X)
    bench = _bad1(ctx, PRESET_BASELINE, pairs, arith=ARITH_FAST, rng=RNG_PHILOX)
    assert abs(bench.mean() - ref.mean()) < BAD1_PP, (bench.mean(), ref.mean())
    assert 2.0 < ref.mean() < 20.0       # the scenes are neither trivial nor failed
