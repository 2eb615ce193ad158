"""Variance reduction on the GPU (kx_price with KX_VR_* flags) against the
oracle's restatement of pricer.rs:108-230: in FP64 on the same Philox paths the
prices agree to rounding of the sums; FP32 within the standard error; the
antithetic flag on a Heston model prices the plain paths bit for bit."""
import math

import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

S = kx.S("S")
CONTRACTS = {
    "euro_call": lambda: kx.european_call("S", 100.0, 1.0),
    "up_and_out": lambda: kx.up_and_out_call("S", 100.0, 130.0, 1.0),
    "asian": lambda: kx.scale((kx.average(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "digital": lambda: kx.cash_or_nothing_call("S", 100.0, 10.0, 0.75),
}


@pytest.mark.parametrize("flags", [(True, False), (False, True), (True, True)])
@pytest.mark.parametrize("name", sorted(CONTRACTS))
def test_vr_matches_the_oracle_fp64(orc, name, flags):
    c = CONTRACTS[name]()
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.04, asset="S")
    anti, cv = flags
    for n in (20_001, 1):
        g = c.price(m, n_paths=n, seed=11, steps_per_year=52, antithetic=anti, control_variate=cv, precision="fp64")
        o = orc.price_vr(c.to_json(), m, n_paths=n, seed=11, steps_per_year=52, antithetic=anti, control_variate=cv)
        assert g.n_paths == o.n_paths
        if n == 1 and anti and cv:  # no pair: the Black-Scholes value and a 0 / 0 standard error
            assert g.price == o.price and math.isnan(g.std_error) and math.isnan(o.std_error)
            continue
        assert abs(g.price - o.price) <= 1e-12 * max(1.0, abs(o.price)), (n, g.price, o.price)
        assert abs(g.std_error - o.std_error) <= 1e-9 * max(1.0, o.std_error)


@pytest.mark.parametrize("flags", [(True, False), (False, True), (True, True)])
def test_vr_fp32_within_the_standard_error(orc, flags):
    c = CONTRACTS["up_and_out"]()
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.04, asset="S")
    anti, cv = flags
    g = c.price(m, n_paths=200_000, seed=5, steps_per_year=252, antithetic=anti, control_variate=cv)
    o = orc.price_vr(c.to_json(), m, n_paths=200_000, seed=5, steps_per_year=252, antithetic=anti, control_variate=cv)
    assert abs(g.price - o.price) < 3 * o.std_error + 1e-6


def test_antithetic_cuts_the_error_of_a_call():
    c = CONTRACTS["euro_call"]()
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    plain = c.price(m, n_paths=400_000, seed=1)
    anti = c.price(m, n_paths=400_000, seed=1, antithetic=True)
    cv = c.price(m, n_paths=400_000, seed=1, control_variate=True)
    assert anti.sample_std < 0.75 * plain.sample_std  # VR-1 (tests/j15_variance_reduction.rs)
    assert cv.std_error < 1e-6 * plain.std_error     # the control is the target itself


def test_heston_has_no_antithetic_paths():
    c = CONTRACTS["up_and_out"]()
    h = kx.heston(100.0, 0.04, 1.5, 0.04, 0.4, -0.6, 0.03, asset="S")
    plain = c.price(h, n_paths=50_000, seed=3, steps_per_year=100)
    anti = c.price(h, n_paths=50_000, seed=3, steps_per_year=100, antithetic=True)
    assert (anti.price, anti.std_error, anti.n_paths) == (plain.price, plain.std_error, plain.n_paths)


def test_vr_has_no_per_path_values():
    c = CONTRACTS["euro_call"]()
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    with pytest.raises(kx.KontractError):
        c.price(m, n_paths=100, antithetic=True, per_path=True)
