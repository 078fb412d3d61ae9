"""cvtpm_cost_eval_noalloc: the cost evaluator for callers that may not
allocate device memory.

Some callers cannot call cudaMalloc: a host application that owns every
device allocation through its own pool or budget, or a real-time pipeline
that reserves its memory once at start and treats any later allocation as a
fault.  They can only hand over their own input and output buffers.  This
entry point takes exactly those and keeps its intermediate images in a fixed
device array inside the library.  Its results must be the ones the normal
context-based cvtpm_cost_eval produces, bit for bit (the tolerance every
parity test here uses), on consecutive calls that reuse the shared array.
"""
import ctypes

import numpy as np
import pytest
import torch

from cvt_gb300 import scenes
from cvt_gb300.params import default_params, PRESET_REFERENCE, PRESET_BASELINE

from bitcmp import bit_diff

pytestmark = pytest.mark.gpu

CVTPM_ERR_SIZE = 2


def _plane_states(sc, seed):
    rng = np.random.default_rng(seed)
    H, W = sc.labels.shape
    pf = sc.plane_field().astype(np.float64)
    st = np.zeros((H, W, 4), np.float32)
    st[..., 0] = 1.0 - pf[..., 0] + rng.normal(0, 0.01, (H, W))
    st[..., 1] = -pf[..., 1] + rng.normal(0, 0.01, (H, W))
    st[..., 2] = -pf[..., 2] + rng.normal(0, 1.0, (H, W))
    return st


def _noalloc(p, left, right, states):
    from cvt_gb300 import _lib
    H, W = left.shape[:2]
    out = torch.empty((H, W), dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = _lib.lib().cvtpm_cost_eval_noalloc(ctypes.byref(p), left.data_ptr(), right.data_ptr(), W, H, W * 16,
                                           states.data_ptr(), out.data_ptr(), stream)
    return rc, out


def test_noalloc_matches_cost_eval_on_consecutive_calls(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    ctx = PMHuberStereo(0)
    cases = [
        (default_params(PRESET_REFERENCE, patchsize=17), scenes.make_scene(83, 61, 5, 20.0, seed=41), 1),
        (default_params(PRESET_BASELINE, patchsize=9), scenes.make_scene(97, 45, 4, 16.0, seed=42), 2),
    ]
    for p, sc, seed in cases:                     # two calls in a row on the shared array
        left = torch.from_numpy(sc.left).cuda()
        right = torch.from_numpy(sc.right).cuda()
        states = torch.from_numpy(_plane_states(sc, seed)).cuda()
        ctx.set_params(p)
        want = ctx.cost(left, right, states)
        rc, got = _noalloc(p, left, right, states)
        assert rc == 0
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert not bit_diff(g, w).any()


def test_noalloc_at_its_size_limit_matches_cost_eval(cuda):
    """366 x 366 is the largest square image the 16 MiB array holds (its
    layout ends 124 KB before the array does, where an off-by-one in the
    layout would show); 367 x 367 is refused."""
    from cvt_gb300.stereo import PMHuberStereo
    ctx = PMHuberStereo(0)
    sc = scenes.make_scene(366, 366, 6, 24.0, seed=43)
    for p in (default_params(PRESET_BASELINE, patchsize=17), default_params(PRESET_REFERENCE, patchsize=17)):
        left = torch.from_numpy(sc.left).cuda()
        right = torch.from_numpy(sc.right).cuda()
        states = torch.from_numpy(_plane_states(sc, 5)).cuda()
        ctx.set_params(p)
        want = ctx.cost(left, right, states)
        rc, got = _noalloc(p, left, right, states)
        assert rc == 0
        torch.cuda.synchronize()
        assert not bit_diff(got.cpu().numpy(), want.cpu().numpy()).any()
    big = scenes.make_scene(367, 367, 2, 8.0, seed=44)
    left = torch.from_numpy(big.left).cuda()
    states = torch.zeros((367, 367, 4), dtype=torch.float32, device="cuda")
    rc, _ = _noalloc(default_params(PRESET_BASELINE, patchsize=17), left, left, states)
    assert rc == CVTPM_ERR_SIZE


def test_cost_eval_rejects_misaligned_states(cuda):
    """Both evaluators read the states as float4: a pointer that is not
    16-byte aligned is refused before any launch."""
    from cvt_gb300 import _lib
    from cvt_gb300.stereo import PMHuberStereo
    ctx = PMHuberStereo(0, default_params(PRESET_REFERENCE, patchsize=5))
    img = torch.zeros((8, 16, 4), dtype=torch.float32, device="cuda")
    states = torch.zeros(8 * 16 * 4 + 4, dtype=torch.float32, device="cuda")
    cost = torch.empty((8, 16), dtype=torch.float32, device="cuda")
    rc = _lib.lib().cvtpm_cost_eval(ctx._h, img.data_ptr(), img.data_ptr(), 16, 8, 16 * 16, states.data_ptr() + 4,
                                    1, cost.data_ptr(), None)
    assert rc == 1
    p = default_params(PRESET_REFERENCE, patchsize=5)
    rc = _lib.lib().cvtpm_cost_eval_noalloc(ctypes.byref(p), img.data_ptr(), img.data_ptr(), 16, 8, 16 * 16,
                                           states.data_ptr() + 4, cost.data_ptr(), None)
    assert rc == 1
    torch.cuda.synchronize()


def test_noalloc_rejects_images_beyond_its_limit(cuda):
    p = default_params(PRESET_REFERENCE, patchsize=5)
    small = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    from cvt_gb300 import _lib
    out = torch.empty((8, 8), dtype=torch.float32, device="cuda")
    W, H = 2000, 1000                             # 2 Mpx needs ~250 MB, far over 16 MiB
    rc = _lib.lib().cvtpm_cost_eval_noalloc(ctypes.byref(p), small.data_ptr(), small.data_ptr(), W, H, W * 16,
                                           small.data_ptr(), out.data_ptr(), None)
    assert rc == CVTPM_ERR_SIZE
