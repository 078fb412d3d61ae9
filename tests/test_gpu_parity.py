"""GPU parity: libcvtpm.so (through the C ABI) against the CPU oracle on the
same seeded inputs.  Integer outputs (winning hypothesis, validity mask) and
every float output are compared bit for bit: both sides use the same
arithmetic (EXACT = the reference's operation order; FAST = the fused form the
oracle mirrors)."""
import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import (default_params, PRESET_REFERENCE, PRESET_BASELINE, ARITH_EXACT, ARITH_FAST,
                              RNG_MWC64X, RNG_PHILOX)

from bitcmp import bit_diff

pytestmark = pytest.mark.gpu

MODES = [(ARITH_EXACT, RNG_MWC64X), (ARITH_FAST, RNG_PHILOX), (ARITH_EXACT, RNG_PHILOX), (ARITH_FAST, RNG_MWC64X)]
MODE_IDS = ["exact-mwc64x", "fast-philox", "exact-philox", "fast-mwc64x"]


def assert_bitexact(got, want, what):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, what
    diff = bit_diff(got, want)
    assert not diff.any(), f"{what}: {int(diff.sum())} of {diff.size} differ, first at {np.argwhere(diff)[0]}"


@pytest.fixture(scope="module")
def stereo(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    return PMHuberStereo(0)


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def plane_states(sc, rng, lr=1):
    """Ground-truth planes as reference states, perturbed, plus random and
    non-finite entries."""
    H, W = sc.labels.shape
    pf = sc.plane_field().astype(np.float64)
    a = pf[..., 0] + rng.normal(0, 0.01, (H, W))
    b = pf[..., 1] + rng.normal(0, 0.01, (H, W))
    c = pf[..., 2] + rng.normal(0, 1.0, (H, W))
    s = np.zeros((H, W, 4), np.float32)
    s[..., 0], s[..., 1], s[..., 2] = 1.0 - a, -b, -c        # x' = x - d
    m = rng.random((H, W)) < 0.05
    s[m, 0] = rng.uniform(-1, 3, m.sum())
    s[m, 2] = rng.uniform(-100, 100, m.sum())
    s[0, 0, 0] = np.inf
    s[0, 1, 2] = np.nan
    return s


@pytest.mark.parametrize("arith", [ARITH_EXACT, ARITH_FAST], ids=["exact", "fast"])
@pytest.mark.parametrize("preset", [PRESET_REFERENCE, PRESET_BASELINE], ids=["ref", "baseline"])
def test_cost_field_bitexact(stereo, oracle, arith, preset):
    sc = scenes.make_scene(83, 61, 5, 20.0, seed=21)
    st = plane_states(sc, np.random.default_rng(3))
    p = default_params(preset, arith=arith, patchsize=17, depthmax=20.0)
    stereo.set_params(p)
    got = stereo.cost(to_dev(sc.left), to_dev(sc.right), to_dev(st)).cpu().numpy()
    want = oracle.cost_field(p, sc.left, sc.right, st)
    assert_bitexact(got, want, "cost")
    assert (got[0, 0] == 1e5) and (got[0, 1] == 1e5)


def run_both(stereo, oracle, sc, p, normalmap=True):
    stereo.set_params(p)
    dm = torch.empty(0, device="cuda")
    nm = torch.empty(0, device="cuda") if normalmap else None
    tr = {}
    stereo.depthMap(dm, to_dev(sc.left), to_dev(sc.right), p.patchsize, p.depthmax, p.iterations, 4,
                    p.dscale, nm, trace=tr)
    torch.cuda.synchronize()
    want, ex = oracle.depthmap(p, sc.left, sc.right, normalmap=normalmap, trace=True)
    return dm.cpu().numpy(), (nm.cpu().numpy() if normalmap else None), {k: v.cpu().numpy() for k, v in tr.items()}, want, ex


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
def test_depthmap_bitexact(stereo, oracle, mode):
    arith, rng = mode
    sc = scenes.make_scene(96, 64, 4, 16.0, seed=5)
    p = default_params(PRESET_REFERENCE, arith=arith, rng=rng, seed=99, patchsize=7, depthmax=16.0,
                       iterations=3, pd_iterations=20)
    dm, nm, tr, want, ex = run_both(stereo, oracle, sc, p)
    assert_bitexact(tr["winners"], ex["winners"], "winners")
    assert_bitexact(tr["valid"], ex["valid"], "valid")
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")
    assert_bitexact(nm, ex["normalmap"], "normalmap")


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
def test_shared_windows_match_per_pixel_neighbours(oracle, mode):
    """The 8 neighbour candidates evaluated plane by plane over shared
    windows give the same bits as the per-pixel evaluation (memory budget 0),
    and both match the oracle — in FAST and in the reference's EXACT
    arithmetic.  150 pixels wide: the row-pipelined warps and the per-lane
    border warps both run."""
    from cvt_gb300.stereo import PMHuberStereo
    arith, rng = mode
    sc = scenes.make_scene(150, 70, 5, 20.0, seed=12)
    p = default_params(PRESET_BASELINE, arith=arith, rng=rng, patchsize=11, depthmax=20.0, iterations=3,
                       pd_iterations=10)
    outs = []
    for budget in (None, 0):
        st = PMHuberStereo(0)
        if budget is not None:
            st.set_memory_budget(budget)
        outs.append(run_both(st, oracle, sc, p))
    (dm1, nm1, tr1, want, ex), (dm0, nm0, tr0, _, _) = outs
    for k in ("winners", "valid", "states"):
        assert_bitexact(tr1[k], tr0[k], k + " (shared vs per pixel)")
        assert_bitexact(tr1[k], ex[k], k + " (vs oracle)")
    assert_bitexact(dm1, dm0, "dmap")
    assert_bitexact(dm1, want, "dmap vs oracle")


def test_depthmap_theta_ramp(stereo, oracle):
    """7 iterations: the smoothness coupling theta becomes non-zero in the last
    (PMHuberStereo.cpp:264-265)."""
    sc = scenes.make_scene(72, 48, 3, 12.0, seed=8)
    p = default_params(PRESET_REFERENCE, patchsize=5, depthmax=12.0, iterations=7, pd_iterations=12)
    dm, _, tr, want, ex = run_both(stereo, oracle, sc, p, normalmap=False)
    assert_bitexact(tr["winners"], ex["winners"], "winners")
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")


@pytest.mark.parametrize("W,H,P", [(37, 29, 17), (1, 1, 3), (33, 9, 2), (130, 17, 4)])
def test_depthmap_odd_sizes(stereo, oracle, W, H, P):
    sc = scenes.make_scene(W, H, 2, 8.0, seed=W * 100 + H)
    p = default_params(PRESET_BASELINE, patchsize=P, depthmax=8.0, iterations=2, pd_iterations=5)
    dm, nm, tr, want, ex = run_both(stereo, oracle, sc, p)
    assert_bitexact(tr["winners"], ex["winners"], "winners")
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")


@pytest.mark.parametrize("W,H,P", [(2100, 19, 7), (21, 900, 5)], ids=["wide", "tall"])
def test_depthmap_wide_and_tall(stereo, oracle, W, H, P):
    """Strip-shaped pairs: one row of smoother tiles and a single column of
    propagation blocks, with both views' smoothers on their two streams."""
    sc = scenes.make_scene(W, H, 2, 9.0, seed=W + 7 * H)
    p = default_params(PRESET_BASELINE, patchsize=P, depthmax=9.0, iterations=2, pd_iterations=6)
    dm, nm, tr, want, ex = run_both(stereo, oracle, sc, p)
    assert_bitexact(tr["winners"], ex["winners"], "winners")
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")
    assert_bitexact(nm, ex["normalmap"], "normalmap")


def test_pd_tool_time(stereo):
    """cvtpm_tool_pd_time: refused before a depthMap has sized the context,
    a positive time per step afterwards."""
    from cvt_gb300 import _lib
    import ctypes
    from cvt_gb300.stereo import PMHuberStereo
    fresh = PMHuberStereo(0, default_params(PRESET_BASELINE))
    us = ctypes.c_float(0.0)
    assert _lib.lib().cvtpm_tool_pd_time(fresh._h, 8, None, ctypes.byref(us)) != 0
    sc = scenes.make_scene(64, 40, 2, 8.0, seed=5)
    fresh.depthMap(None, to_dev(sc.left), to_dev(sc.right), 5, 8.0, 1, 4)
    assert _lib.lib().cvtpm_tool_pd_time(fresh._h, 7, None, ctypes.byref(us)) != 0      # odd step count
    assert _lib.lib().cvtpm_tool_pd_time(fresh._h, 8, None, ctypes.byref(us)) == 0
    assert us.value > 0.0


def test_pitched_input_and_host_entry(stereo, oracle):
    sc = scenes.make_scene(50, 30, 3, 10.0, seed=4)
    p = default_params(PRESET_BASELINE, patchsize=5, depthmax=10.0, iterations=2, pd_iterations=4)
    stereo.set_params(p)
    wide = torch.zeros((30, 64, 4), device="cuda")
    wide[:, :50] = to_dev(sc.left)
    wide2 = torch.zeros((30, 64, 4), device="cuda")
    wide2[:, :50] = to_dev(sc.right)
    dm = stereo.depthMap(None, wide[:, :50], wide2[:, :50], 5, 10.0, 2, 4)
    want, _ = oracle.depthmap(p, sc.left, sc.right)
    assert_bitexact(dm.cpu().numpy(), want, "dmap pitched")
    host = stereo.depthMapHost(sc.left, sc.right, 5, 10.0, 2, 4)
    assert_bitexact(host, want, "dmap host")


def test_errors(stereo):
    from cvt_gb300.stereo import CVTException
    from cvt_gb300._lib import CvtpmError
    a = torch.zeros((10, 12, 4), device="cuda")
    b = torch.zeros((10, 13, 4), device="cuda")
    with pytest.raises(CVTException):
        stereo.depthMap(None, a, b, 3, 8.0, 1, 4)
    with pytest.raises(CvtpmError):
        stereo.depthMap(None, a, a, 40, 8.0, 1, 4)
    with pytest.raises(CvtpmError):
        stereo.depthMap(None, a, a, 3, -1.0, 1, 4)


@pytest.mark.parametrize("pd_iters", [0, 1, 3, 9])
def test_pd_step_counts(stereo, oracle, pd_iters):
    """PDROF::apply with 0, odd and even step counts (PDROF.h:67-95), through
    the blocked smoother (4 steps per launch) and the one-step path."""
    sc = scenes.make_scene(70, 41, 3, 10.0, seed=30 + pd_iters)
    p = default_params(PRESET_BASELINE, patchsize=4, depthmax=10.0, iterations=2, pd_iterations=pd_iters)
    dm, _, tr, want, ex = run_both(stereo, oracle, sc, p, normalmap=False)
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("iters", [3, 6])
def test_depthmap_inpaint_bitexact(stereo, oracle, mode, iters):
    """PMHuberStereo::depthMapInpaint: odd and even iteration counts (the final
    check reads state buffer 1 either way), theta > 0 from iteration 5."""
    arith, rng = mode
    sc = scenes.make_scene(90, 52, 4, 14.0, seed=31 + iters)
    p = default_params(PRESET_REFERENCE, arith=arith, rng=rng, seed=7, patchsize=7, depthmax=14.0, iterations=iters)
    stereo.set_params(p)
    tr = {}
    dm = stereo.depthMapInpaint(None, to_dev(sc.left), to_dev(sc.right), 7, 14.0, iters, 4, trace=tr)
    torch.cuda.synchronize()
    want, ex = oracle.depthmap_inpaint(p, sc.left, sc.right, trace=True)
    assert_bitexact(tr["winners"].cpu().numpy(), ex["winners"], "winners")
    assert_bitexact(tr["valid"].cpu().numpy(), ex["valid"], "valid")
    assert_bitexact(tr["states"].cpu().numpy(), ex["states"], "states")
    assert_bitexact(dm.cpu().numpy(), want, "dmap")


@pytest.mark.parametrize("mode", [MODES[0], MODES[1]], ids=MODE_IDS[:2])
@pytest.mark.parametrize("W,H", [(96, 64), (75, 41)])
def test_depthmap_redblack_bitexact(stereo, oracle, mode, W, H):
    """The optional red/black schedule (pixels with x+y even first, then odd)
    against the oracle's restatement of it; an odd width puts a different
    number of red and black pixels in each row."""
    from cvt_gb300.params import SCHEDULE_REDBLACK
    arith, rng = mode
    sc = scenes.make_scene(W, H, 4, 16.0, seed=W + H)
    p = default_params(PRESET_REFERENCE, arith=arith, rng=rng, seed=5, patchsize=7, depthmax=16.0, iterations=3,
                       pd_iterations=12, schedule=SCHEDULE_REDBLACK)
    dm, nm, tr, want, ex = run_both(stereo, oracle, sc, p)
    assert_bitexact(tr["winners"], ex["winners"], "winners")
    assert_bitexact(tr["states"], ex["states"], "states")
    assert_bitexact(dm, want, "dmap")
    jac = default_params(PRESET_REFERENCE, arith=arith, rng=rng, seed=5, patchsize=7, depthmax=16.0, iterations=3,
                         pd_iterations=12)
    _, _, trj, _, _ = run_both(stereo, oracle, sc, jac, normalmap=False)
    assert bit_diff(tr["states"], trj["states"]).any()      # a different schedule


def test_depthmap_inpaint_redblack_bitexact(stereo, oracle):
    from cvt_gb300.params import SCHEDULE_REDBLACK
    sc = scenes.make_scene(80, 48, 3, 12.0, seed=77)
    p = default_params(PRESET_BASELINE, patchsize=5, depthmax=12.0, iterations=3, schedule=SCHEDULE_REDBLACK)
    stereo.set_params(p)
    tr = {}
    dm = stereo.depthMapInpaint(None, to_dev(sc.left), to_dev(sc.right), 5, 12.0, 3, 4, trace=tr)
    torch.cuda.synchronize()
    want, ex = oracle.depthmap_inpaint(p, sc.left, sc.right, trace=True)
    assert_bitexact(tr["states"].cpu().numpy(), ex["states"], "states")
    assert_bitexact(dm.cpu().numpy(), want, "dmap")


@pytest.mark.parametrize("mode", [(ARITH_FAST, RNG_PHILOX), (ARITH_EXACT, RNG_MWC64X)], ids=["bench", "reference"])
def test_bench_configuration_band_bitexact(stereo, oracle, mode):
    """The bench's own configuration on a band of its pair: rows 0-47 of the
    1242x375 scene (2 % salt, gain/bias), 35x35 window, dmax 128, LR
    threshold 1 px, 250 PD steps, 2 iterations (theta stays 0; the ramp has
    its own test) — in the bench's arithmetic and in the reference's."""
    arith, rng = mode
    sc = scenes.config_scene(2, pair=0)
    left = np.ascontiguousarray(sc.left[:48])
    right = np.ascontiguousarray(sc.right[:48])
    p = default_params(PRESET_BASELINE, arith=arith, rng=rng, patchsize=17, depthmax=128.0, iterations=2,
                       maxdispdiff=1.0)
    stereo.set_params(p)
    dm = torch.empty(0, device="cuda")
    tr = {}
    stereo.depthMap(dm, to_dev(left), to_dev(right), 17, 128.0, 2, 4, trace=tr)
    torch.cuda.synchronize()
    want, ex = oracle.depthmap(p, left, right, trace=True)
    assert_bitexact(tr["winners"].cpu().numpy(), ex["winners"], "winners")
    assert_bitexact(tr["valid"].cpu().numpy(), ex["valid"], "valid")
    assert_bitexact(tr["states"].cpu().numpy(), ex["states"], "states")
    assert_bitexact(dm.cpu().numpy(), want, "dmap")


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_random_configurations_bitexact(stereo, oracle, seed):
    """Seeded random configurations: sizes 8-89 x 4-59, windows 3x3-35x35,
    dmax, iterations, PD steps, presets, the four arithmetic/RNG modes, both
    schedules, LR thresholds — disparity map, states and winners bit for bit
    against the oracle."""
    from cvt_gb300 import params as P
    rng = np.random.default_rng(seed)
    for case in range(12):
        W, H = int(rng.integers(8, 90)), int(rng.integers(4, 60))
        patch, dmax = int(rng.integers(1, 18)), float(rng.choice([4.0, 9.5, 16.0, 33.0]))
        iters = int(rng.integers(1, 5))
        kw = dict(arith=[P.ARITH_EXACT, P.ARITH_FAST][int(rng.integers(2))],
                  rng=[P.RNG_MWC64X, P.RNG_PHILOX][int(rng.integers(2))], patchsize=patch, depthmax=dmax,
                  iterations=iters, pd_iterations=int(rng.integers(0, 40)), seed=int(rng.integers(1 << 30)))
        if rng.random() < 0.25:
            kw["schedule"] = P.SCHEDULE_REDBLACK
        if rng.random() < 0.3:
            kw["maxdispdiff"] = 1.0
        p = P.default_params([P.PRESET_REFERENCE, P.PRESET_BASELINE][int(rng.integers(2))], **kw)
        sc = scenes.make_scene(W, H, int(rng.integers(1, 5)), dmax, seed=int(rng.integers(1 << 20)))
        dm, _, tr, want, ex = run_both(stereo, oracle, sc, p, normalmap=False)
        what = f"case {case}: {W}x{H} {kw}"
        assert_bitexact(dm, want, "dmap " + what)
        assert_bitexact(tr["states"], ex["states"], "states " + what)
        assert_bitexact(tr["winners"], ex["winners"], "winners " + what)
