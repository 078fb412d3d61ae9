"""libcvtpm.so in the reference configuration (EXACT arithmetic, MWC64X
streams, reference constants) against the golden fixtures produced by the
reference's own code: bit for bit."""
import os

import numpy as np
import pytest
import torch

from cvt_gb300.params import default_params, PRESET_REFERENCE

from bitcmp import bit_diff

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "pm_reference_golden.npz")


def assert_bits(got, want, what):
    got, want = np.ascontiguousarray(got), np.ascontiguousarray(want)
    assert got.shape == want.shape, what
    d = bit_diff(got, want)
    assert not d.any(), f"{what}: {int(d.sum())} of {d.size} values differ"


@pytest.fixture(scope="module")
def setup(cuda):
    from cvt_gb300.stereo import PMHuberStereo
    return PMHuberStereo(0), np.load(GOLDEN)


@pytest.mark.parametrize("P", [17, 6])
def test_cost_field(setup, P):
    st, G = setup
    st.set_params(default_params(PRESET_REFERENCE, patchsize=P))
    c = st.cost(torch.from_numpy(G["k_left"]).cuda(), torch.from_numpy(G["k_right"]).cuda(),
                torch.from_numpy(G["k_states"]).cuda())
    assert_bits(c.cpu().numpy(), G[f"k_cost_p{P}"], "cost")


@pytest.mark.parametrize("name", ["run_a", "run_b", "run_c"])
def test_depthmap_runs(setup, name):
    st, G = setup
    W, H, P, iters, dmax = G[f"{name}_cfg"]
    p = default_params(PRESET_REFERENCE, patchsize=int(P), depthmax=float(dmax), iterations=int(iters))
    st.set_params(p)
    L, R = torch.from_numpy(G[f"{name}_left"]).cuda(), torch.from_numpy(G[f"{name}_right"]).cuda()
    nm = torch.empty(0, device="cuda")
    tr = {}
    dm = st.depthMap(None, L, R, int(P), float(dmax), int(iters), 4, -1.0, nm, trace=tr)
    torch.cuda.synchronize()
    assert_bits(tr["states"].cpu().numpy(), G[f"{name}_states"], "states")
    assert_bits(dm.cpu().numpy(), G[f"{name}_dmap"], "dmap")
    assert_bits(nm.cpu().numpy(), G[f"{name}_normalmap"], "normalmap")


@pytest.mark.parametrize("name", ["inp_a", "inp_b"])
def test_depthmap_inpaint_golden(setup, name):
    st, G = setup
    W, H, P, iters, dmax = G[f"{name}_cfg"]
    p = default_params(PRESET_REFERENCE, patchsize=int(P), depthmax=float(dmax), iterations=int(iters))
    st.set_params(p)
    tr = {}
    dm = st.depthMapInpaint(None, torch.from_numpy(G[f"{name}_left"]).cuda(), torch.from_numpy(G[f"{name}_right"]).cuda(),
                            int(P), float(dmax), int(iters), 4, trace=tr)
    torch.cuda.synchronize()
    assert_bits(tr["states"].cpu().numpy(), G[f"{name}_states"], "states")
    assert_bits(dm.cpu().numpy(), G[f"{name}_dmap"], "dmap")
