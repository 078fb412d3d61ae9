"""GPU parity at the timed configurations, full size, against the oracle.

The bench times depthMap on a whole 1242x375 pair (16 planes, dmax 128, 2 %
salt, +/-5 % gain/bias, 35x35 window, 8 iterations, LR threshold 1 px with
fill-in, 250 PD steps per view and iteration) and the second workload is a
whole 640x480 pair (8 planes, dmax 64, 3 iterations).  Here both run on the
GPU through the C ABI and in the oracle on the same seeded inputs, at full
size and for every iteration, so the theta > 0 iterations 6 and 7 of the
8-iteration run (PMHuberStereo.cpp:264-265) and the view candidates of every
pass meet the oracle.  Each is run in the bench's arithmetic (FAST + Philox)
and in the reference's (EXACT operation order + MWC64X streams); winners,
validity mask, final plane states of both views, disparity map and normal map
are compared bit for bit.  The oracle takes minutes per run on the host's
cores (about 0.02 Mpix-iter/s on 16 of them); its time is printed.
"""
import time

import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_BASELINE, ARITH_EXACT, ARITH_FAST, RNG_MWC64X, RNG_PHILOX

from bitcmp import bit_diff

pytestmark = pytest.mark.gpu

CONFIGS = {
    # scene config, iterations, dmax, LR threshold (px)
    "1242x375x8": (2, 8, 128.0, 1.0),
    "640x480x3": (1, 3, 64.0, 0.5),
}
MODES = {"fast-philox": (ARITH_FAST, RNG_PHILOX), "exact-mwc64x": (ARITH_EXACT, RNG_MWC64X)}


def assert_bitexact(got, want, what):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, what
    diff = bit_diff(got, want)
    assert not diff.any(), f"{what}: {int(diff.sum())} of {diff.size} differ, first at {np.argwhere(diff)[0]}"


@pytest.mark.parametrize("mode", list(MODES), ids=list(MODES))
@pytest.mark.parametrize("config", list(CONFIGS), ids=list(CONFIGS))
def test_timed_configuration_fullsize_bitexact(cuda, oracle, config, mode):
    from cvt_gb300.stereo import PMHuberStereo
    index, iters, dmax, lr_px = CONFIGS[config]
    arith, rng = MODES[mode]
    sc = scenes.config_scene(index, pair=0)
    p = default_params(PRESET_BASELINE, arith=arith, rng=rng, patchsize=17, depthmax=dmax, iterations=iters,
                       maxdispdiff=lr_px)
    st = PMHuberStereo(0, p)
    dm = torch.empty(0, device="cuda")
    nm = torch.empty(0, device="cuda")
    tr = {}
    st.depthMap(dm, torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda(), 17, dmax, iters, 4,
                -1.0, nm, trace=tr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    want, ex = oracle.depthmap(p, sc.left, sc.right, normalmap=True, trace=True)
    print(f"\n{config} {mode}: oracle {time.perf_counter() - t0:.1f} s on {oracle.max_threads()} threads")
    assert_bitexact(tr["winners"].cpu().numpy(), ex["winners"], "winners")
    assert_bitexact(tr["valid"].cpu().numpy(), ex["valid"], "valid")
    assert_bitexact(tr["states"].cpu().numpy(), ex["states"], "states")
    assert_bitexact(dm.cpu().numpy(), want, "dmap")
    assert_bitexact(nm.cpu().numpy(), ex["normalmap"], "normalmap")
    # the run is a real one: most non-occluded pixels within 1 px of the truth
    assert scenes.bad_pixel_rate(dm.cpu().numpy() * dmax, sc) < 30.0
