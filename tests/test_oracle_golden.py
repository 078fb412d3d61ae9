"""The oracle against golden fixtures produced by the reference's own code
(tests/golden/make_golden.py: cvt/cl/kernel/*.cl and
cvt/vision/PMHuberStereo.cpp run through the OpenCL-C emulation).  Everything
is compared bit for bit."""
import os

import numpy as np
import pytest

from cvt_gb300.params import default_params, PRESET_REFERENCE

from bitcmp import bit_diff

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "pm_reference_golden.npz")


@pytest.fixture(scope="module")
def G():
    return np.load(GOLDEN)


def assert_bits(got, want, what):
    got, want = np.ascontiguousarray(got), np.ascontiguousarray(want)
    assert got.shape == want.shape, what
    d = bit_diff(got, want)
    assert not d.any(), f"{what}: {int(d.sum())} of {d.size} values differ"


def test_gradxy_weight(oracle, G):
    assert_bits(oracle.gradxy(G["k_left"]), G["k_gradxy_left"], "gradxy")
    assert_bits(oracle.edge_weight(G["k_left"]), G["k_weight_left"], "weight")


@pytest.mark.parametrize("P", [17, 6])
def test_cost_field(oracle, G, P):
    p = default_params(PRESET_REFERENCE, patchsize=P)
    assert_bits(oracle.cost_field(p, G["k_left"], G["k_right"], G["k_states"]), G[f"k_cost_p{P}"], "cost")


def test_init_both_views(oracle, G):
    p = default_params(PRESET_REFERENCE, patchsize=17, depthmax=14.0)
    assert_bits(oracle.init(p, G["k_left"], G["k_right"], 1), G["k_init_lr1"], "init left")
    assert_bits(oracle.init(p, G["k_right"], G["k_left"], 0), G["k_init_lr0"], "init right")


@pytest.mark.parametrize("it,lam", [(250, 5.0), (7, 17.5)])
def test_pdrof(oracle, G, it, lam):
    u = oracle.pd_apply(G["k_pd_warm"], G["k_pd_input"], G["k_weight_left"], lam, it)
    assert_bits(u, G[f"k_pd_{it}"], f"PDROF {it}")


@pytest.mark.parametrize("name", ["run_a", "run_b", "run_c"])
def test_depthmap_runs(oracle, G, name):
    W, H, P, iters, dmax = G[f"{name}_cfg"]
    p = default_params(PRESET_REFERENCE, patchsize=int(P), depthmax=float(dmax), iterations=int(iters))
    dmap, ex = oracle.depthmap(p, G[f"{name}_left"], G[f"{name}_right"], normalmap=True, trace=True)
    assert_bits(ex["states"], G[f"{name}_states"], "states")
    assert_bits(dmap, G[f"{name}_dmap"], "dmap")
    assert_bits(ex["normalmap"], G[f"{name}_normalmap"], "normalmap")


@pytest.mark.parametrize("lr", [1, 0])
def test_occmap_normal_depth(oracle, G, lr):
    a, b = (G["k_init_lr1"], G["k_init_lr0"]) if lr else (G["k_init_lr0"], G["k_init_lr1"])
    assert_bits(oracle.occmap(a, b, 0.5, lr), np.ascontiguousarray(G[f"k_occmap_lr{lr}"][..., 0]), "occmap")
    assert_bits(oracle.normal_depth(a, 14.0, lr), G[f"k_normal_depth_lr{lr}"], "normal_depth")


@pytest.mark.parametrize("it,lam", [(100, 5.0), (7, 17.5)])
def test_pdrof_inpaint(oracle, G, it, lam):
    mask = np.ascontiguousarray(G["k_pdi_mask"][..., 0])
    u = oracle.pd_apply_inpaint(G["k_pd_warm"], G["k_pd_input"], G["k_weight_left"], mask, lam, it)
    assert_bits(u, G[f"k_pdi_{it}"], f"PDROFInpaint {it}")


@pytest.mark.parametrize("name", ["inp_a", "inp_b"])
def test_depthmap_inpaint_runs(oracle, G, name):
    W, H, P, iters, dmax = G[f"{name}_cfg"]
    p = default_params(PRESET_REFERENCE, patchsize=int(P), depthmax=float(dmax), iterations=int(iters))
    dmap, ex = oracle.depthmap_inpaint(p, G[f"{name}_left"], G[f"{name}_right"], trace=True)
    assert_bits(ex["states"], G[f"{name}_states"], "states")
    assert_bits(dmap, G[f"{name}_dmap"], "dmap")
