"""The comparison baseline (cvt::StereoGCVFilter) on the GPU, bit for bit
against the golden outputs of the reference's own kernels
(tests/golden/make_gcv_golden.py): both views, the fused map, a fractional
step and a descending range, sizes on and off the 16-pixel scan blocks."""
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


@pytest.mark.parametrize("name", ["apply_a", "apply_b"])
def test_apply_matches_reference(cuda, G, name):
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    out, d0, d1 = gcv.StereoGCVFilter().apply(torch.from_numpy(G[f"{name}_cam0"]).cuda(),
                                              torch.from_numpy(G[f"{name}_cam1"]).cuda(), dmin, dmax, dt)
    torch.cuda.synchronize()
    assert not bit_diff(d0.cpu().numpy(), G[f"{name}_d0"]).any()
    assert not bit_diff(d1.cpu().numpy(), G[f"{name}_d1"]).any()
    assert np.array_equal(out.cpu().numpy(), G[f"{name}_out"])


@pytest.mark.parametrize("name", ["dm_frac", "dm_desc"])
def test_depthmap_matches_reference(cuda, G, name):
    dmin, dmax, dt = (float(v) for v in G[f"{name}_args"])
    d = gcv.StereoGCVFilter().depthmap(torch.from_numpy(G[f"{name}_cam0"]).cuda(),
                                       torch.from_numpy(G[f"{name}_cam1"]).cuda(), dmin, dmax, dt)
    torch.cuda.synchronize()
    assert not bit_diff(d.cpu().numpy(), G[f"{name}_d0"]).any()
