"""The comparison baseline (cvt::StereoGCVFilter) on the GPU, bit for bit
against the golden outputs of the reference's own kernels
(tests/golden/make_gcv_golden.py): both views, the fused map, a fractional
step and a descending range, sizes on and off the 16-pixel scan blocks,
each with disparity batches of 1, 3 and the automatic size; and, at the
headline size, the same output for every batch size."""
import os

import numpy as np
import pytest
import torch

from bitcmp import bit_diff
from cvt_gb300 import gcv

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "gcv_reference_golden.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


@pytest.fixture(params=[0, 1, 3])
def batch(request):
    gcv.set_batch(request.param)
    yield request.param
    gcv.set_batch(0)


@pytest.mark.parametrize("name", ["apply_a", "apply_b"])
def test_apply_matches_reference(cuda, G, name, batch):
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    out, d0, d1 = gcv.StereoGCVFilter().apply(torch.from_numpy(G[f"{name}_cam0"]).cuda(),
                                              torch.from_numpy(G[f"{name}_cam1"]).cuda(), dmin, dmax, dt)
    torch.cuda.synchronize()
    assert not bit_diff(d0.cpu().numpy(), G[f"{name}_d0"]).any()
    assert not bit_diff(d1.cpu().numpy(), G[f"{name}_d1"]).any()
    assert np.array_equal(out.cpu().numpy(), G[f"{name}_out"])


@pytest.mark.parametrize("name", ["dm_frac", "dm_desc"])
def test_depthmap_matches_reference(cuda, G, name, batch):
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    d = gcv.StereoGCVFilter().depthmap(torch.from_numpy(G[f"{name}_cam0"]).cuda(),
                                       torch.from_numpy(G[f"{name}_cam1"]).cuda(), dmin, dmax, dt)
    torch.cuda.synchronize()
    assert not bit_diff(d.cpu().numpy(), G[f"{name}_d0"]).any()


def test_batch_size_does_not_change_the_headline_pair(cuda):
    from cvt_gb300 import scenes
    sc = scenes.config_scene(2, pair=0)
    left, right = torch.from_numpy(sc.left).cuda(), torch.from_numpy(sc.right).cuda()
    outs = []
    try:
        for b in (0, 5, 64):
            gcv.set_batch(b)
            assert gcv.plan(1242, 375, 0.0, 128.0, 1.0)["batch"] == (b or 128)
            outs.append([t.cpu().numpy() for t in gcv.StereoGCVFilter().apply(right, left, 0.0, 128.0, 1.0)])
    finally:
        gcv.set_batch(0)
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("W,H,dmin,dmax,dt,batch", [(96, 64, 0.0, 16.0, 1.0, 0), (130, 47, 2.0, 20.0, 0.75, 7),
                                                    (257, 129, 0.0, 32.0, 1.0, 0), (64, 80, 24.0, 3.0, 1.5, 4)])
def test_apply_matches_oracle(cuda, oracle, W, H, dmin, dmax, dt, batch):
    """sizes on and off the 16-pixel blocks, fractional and descending steps,
    several batch sizes, against the oracle's restatement of the reference's
    kernels (pinned on the golden vectors)"""
    from cvt_gb300 import scenes
    sc = scenes.make_scene(W, H, 4, max(abs(dmin), abs(dmax)), seed=300 + W)
    want = oracle.gcv_apply(sc.right, sc.left, dmin, dmax, dt)
    gcv.set_batch(batch)
    try:
        got = gcv.StereoGCVFilter().apply(torch.from_numpy(sc.right).cuda(), torch.from_numpy(sc.left).cuda(),
                                          dmin, dmax, dt)
        torch.cuda.synchronize()
    finally:
        gcv.set_batch(0)
    out, d0, d1 = (t.cpu().numpy() for t in got)
    assert not bit_diff(d0, want[1]).any()
    assert not bit_diff(d1, want[2]).any()
    assert np.array_equal(out, want[0])


def test_scratch_does_not_grow_with_threads(cuda):
    """calls from one host thread after another reuse the library's
    stream-ordered scratch (here about 160 MB a call): device memory after
    four threads equals that after the first"""
    import threading
    from cvt_gb300 import scenes
    sc = scenes.make_scene(300, 200, 3, 64.0, seed=5)
    cam0, cam1 = torch.from_numpy(sc.right).cuda(), torch.from_numpy(sc.left).cuda()
    err, free = [], []

    def work():
        try:
            gcv.StereoGCVFilter().apply(cam0, cam1, 0.0, 64.0, 1.0)
            torch.cuda.synchronize()
        except Exception as e:           # noqa: BLE001 - reported below
            err.append(e)

    for _ in range(4):
        t = threading.Thread(target=work)
        t.start()
        t.join()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert not err, err
    assert abs(free[0] - free[-1]) < 32 << 20, [(f - free[0]) >> 20 for f in free]


def test_trim_returns_the_pool_memory(cuda):
    """after an apply the pool keeps its scratch (about 160 MB here);
    cvtpm_gcv_trim gives it back to the device, and a later apply still
    gives the same bits"""
    from cvt_gb300 import scenes
    sc = scenes.make_scene(300, 200, 3, 64.0, seed=6)
    cam0, cam1 = torch.from_numpy(sc.right).cuda(), torch.from_numpy(sc.left).cuda()
    f = gcv.StereoGCVFilter()
    first = f.apply(cam0, cam1, 0.0, 64.0, 1.0)
    torch.cuda.synchronize()
    held = torch.cuda.mem_get_info()[0]
    gcv.trim(0, 0)
    torch.cuda.synchronize()
    freed = torch.cuda.mem_get_info()[0]
    assert freed - held > 64 << 20, (freed - held) >> 20
    again = f.apply(cam0, cam1, 0.0, 64.0, 1.0)
    torch.cuda.synchronize()
    for a, b in zip(first, again):
        assert torch.equal(a.cpu(), b.cpu())
    with pytest.raises(Exception):
        gcv.trim(-1, 0)
