"""The project's elementary functions (cvt_gb300/csrc/pm_math.h) against
float64 references: they replace the reference's native_exp / exp / pow /
acospi (cvt/cl/kernel/pmhstereo.cl:199,462,781), whose accuracy OpenCL leaves
to the implementation."""
import numpy as np


def ulp_err(got, want):
    got = got.astype(np.float64)
    spacing = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    return np.abs(got - want) / spacing


def test_exp_within_2ulp(oracle):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-87, 88, 200000), rng.uniform(-2, 2, 100000),
                        np.array([0.0, -0.0, 1.0, -1.0, 88.0, -87.0])]).astype(np.float32)
    y = np.empty_like(x)
    oracle.lib().orc_exp_array(x, y, x.size)
    want = np.exp(x.astype(np.float64))
    assert ulp_err(y, want).max() <= 2.0
    assert oracle.lib().orc_exp(0.0) == 1.0


def test_exp_edges(oracle):
    f = oracle.lib().orc_exp
    assert f(-200.0) == 0.0
    assert f(-104.0) == 0.0
    assert np.isinf(f(100.0))
    assert np.isnan(f(float("nan")))
    # subnormal results: within 1 subnormal step of the true value
    for v in (-88.0, -95.0, -100.0, -103.0):
        want = np.exp(np.float64(v))
        assert abs(f(v) - want) <= 1.5e-45 + 4e-7 * want


def test_pow_and_acospi(oracle):
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 2, 100000).astype(np.float32)
    y = np.empty_like(x)
    oracle.lib().orc_pow_array(x, np.float32(0.8), y, x.size)
    want = np.power(x.astype(np.float64), 0.8)
    rel = np.abs(y - want) / np.maximum(want, 1e-30)
    assert rel.max() < 2e-6
    assert oracle.lib().orc_pow(0.0, 0.8) == 0.0
    c = rng.uniform(-1, 1, 100000).astype(np.float32)
    a = np.empty_like(c)
    oracle.lib().orc_acospi_array(c, a, c.size)
    want = np.arccos(c.astype(np.float64)) / np.pi
    assert np.abs(a - want).max() < 3e-7
    assert np.isnan(oracle.lib().orc_acospi(1.0000001))


def test_weight_exp(oracle):
    """pm_wexp, the ASW weight's exponential (the reference's native_exp,
    pmhstereo.cl:199): within 2 ulp of exp on its range, a floor of
    e^-87.3 below it (and for NaN), and the same floats as pm_exp wherever
    both round k the same way."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-87.3, 88.7, 300000), rng.uniform(-30, 0, 300000),
                        np.array([0.0, -0.0, -1.0, 1.0, -87.3, 88.7])]).astype(np.float32)
    y = np.empty_like(x)
    oracle.lib().orc_wexp_array(x, y, x.size)
    assert ulp_err(y, np.exp(x.astype(np.float64))).max() <= 2.0
    assert oracle.lib().orc_wexp(0.0) == 1.0
    e = np.empty_like(x)
    oracle.lib().orc_exp_array(x, e, x.size)
    assert (y != e).mean() < 1e-3
    f = oracle.lib().orc_wexp
    floor = f(-87.3)
    assert 1.17e-38 < floor < 1.3e-38
    assert f(-100.0) == floor and f(-1e30) == floor and f(float("nan")) == floor
