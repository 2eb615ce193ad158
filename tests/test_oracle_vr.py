"""The oracle's variance reduction against the reference's own checks
(tests/j15_variance_reduction.rs): antithetic pairs cut the sample std of a
European call below 0.75 of the plain estimate (VR-1) and price it within 1 %
of Black-Scholes (VR-2); the at-the-money call as a control prices the same
call within 1 % (VR-4); price_antithetic_with_cv's quirk (the standard error of
the target over sqrt(2 n_half)) and the fallback of other models."""
import math

import kontracts_gb300 as kx


def _call():
    return kx.european_call("S", 100.0, 1.0)


def test_vr1_antithetic_reduces_the_sample_std(orc):
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    base = orc.price(_call().to_json(), m, n_paths=20_000, seed=42, steps_per_year=50)
    anti = orc.price_vr(_call().to_json(), m, n_paths=40_000, seed=42, steps_per_year=50, antithetic=True)
    assert anti.n_paths == 20_000
    assert anti.sample_std < 0.75 * base.sample_std


def test_vr2_antithetic_price_matches_bs(orc):
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    anti = orc.price_vr(_call().to_json(), m, n_paths=100_000, seed=99, steps_per_year=50, antithetic=True)
    bs = orc.bs_call(100.0, 100.0, 1.0, 0.05, 0.2)
    assert abs(anti.price - bs) / bs < 0.01


def test_vr4_control_variate_unbiased(orc):
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    cv = orc.price_vr(_call().to_json(), m, n_paths=100_000, seed=2024, steps_per_year=50, control_variate=True)
    bs = orc.bs_call(100.0, 100.0, 1.0, 0.05, 0.2)
    assert abs(cv.price - bs) / bs < 0.01
    # the control is the target itself: every path's correction cancels its noise
    assert cv.sample_std < 1e-9


def test_antithetic_with_control_variate_formula(orc):
    """price = target pairs - (control pairs - bs); std error = the target
    pairs' sample std / sqrt(2 n_half) (pricer.rs:185-219)."""
    # a European put: its grid [0, 1] is the control call's, so the call priced alone sees the same paths
    put = kx.european_put("S", 95.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    n = 30_001
    both = orc.price_vr(put.to_json(), m, n_paths=n, seed=7, steps_per_year=100, antithetic=True,
                        control_variate=True)
    t = orc.price_vr(put.to_json(), m, n_paths=n, seed=7, steps_per_year=100, antithetic=True)
    c = orc.price_vr(_call().to_json(), m, n_paths=n, seed=7, steps_per_year=100, antithetic=True)
    bs = orc.bs_call(100.0, 100.0, 1.0, 0.05, 0.2)
    assert both.price == t.price - 1.0 * (c.price - bs)
    assert both.sample_std == t.sample_std
    assert both.n_paths == 2 * (n // 2)
    assert both.std_error == t.sample_std / math.sqrt(2 * (n // 2))


def test_other_models_have_no_antithetic_paths(orc):
    """Simulator::simulate_antithetic_paths is None but for GBM: the plain
    paths; the control variate falls back to s0 = 100, sigma = 0.2."""
    h = kx.heston(100.0, 0.04, 1.5, 0.04, 0.4, -0.6, 0.03, asset="S")
    js = _call().to_json()
    plain = orc.price(js, h, n_paths=5_000, seed=3, steps_per_year=52)
    anti = orc.price_vr(js, h, n_paths=5_000, seed=3, steps_per_year=52, antithetic=True)
    assert (anti.price, anti.std_error, anti.n_paths) == (plain.price, plain.std_error, plain.n_paths)
    cv = orc.price_vr(js, h, n_paths=5_000, seed=3, steps_per_year=52, control_variate=True)
    bs = orc.bs_call(100.0, 100.0, 1.0, 0.03, 0.2)
    assert abs(cv.price - bs) < 1e-9  # the control is the same call on the same paths
