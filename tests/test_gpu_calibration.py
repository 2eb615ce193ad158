"""Calibration callers on the GPU: the batched objectives (one path launch per
iteration or generation) against the oracle's restatement of gbm_prices and
eval_obj_heston in FP64, the optimizers' trajectories equal to the same loops
driven by oracle prices, and the reference's own calibration checks
(tests/j21_fast_calibration.rs, tests/j22_cmaes.rs) on the engine."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import calibration as cal

pytestmark = pytest.mark.gpu

R = 0.05
HP = [0.04, 2.0, 0.04, 0.3, -0.5]


def test_gbm_prices_match_oracle(orc):
    c = kx.up_and_out_call("EQ", 100.0, 140.0, 1.0)
    spots, sigmas = [90.0, 100.0, 110.0], [0.15, 0.25, 0.4]
    quotes = [(s, 0.0) for s in spots]
    g = cal.gbm_prices(c, "EQ", quotes, sigmas, R, 4000)
    ref = orc.calib_gbm_prices(c.to_json(), "EQ", spots, sigmas, n_paths=4000, rate=R)
    assert g.shape == (3, 3)
    assert np.allclose(g, ref, rtol=1e-10, atol=1e-13)
    assert kx.last_launch_stats()["kernel_launches"] <= 3  # one path launch + the statistics
    bad = cal.gbm_prices(c, "underlying", quotes, sigmas[:1], R, 100)
    assert np.all(np.isnan(bad))


def test_heston_objective_matches_oracle(orc):
    c = kx.european_call("underlying", 100.0, 1.0)
    quotes = [(90.0, 5.0), (100.0, 10.5), (110.0, 17.0)]
    pop = [HP, [0.05, 1.5, 0.06, 0.5, -0.7], [0.02, 3.0, 0.03, 0.2, 0.1], [0.04, 2.0, 0.04, 0.3, 1.5]]
    g = cal.heston_objective(c, quotes, pop, R, 2000)
    ref = orc.calib_heston_objective(c.to_json(), "underlying", quotes, pop, n_paths=2000, rate=R)
    assert np.allclose(g, ref, rtol=1e-11, atol=1e-14), (g, ref)
    assert g[3] == 0.0  # rho 1.5: every quote fails, nothing summed (calibration.rs:111-125)
    other = kx.european_call("EQ", 100.0, 1.0)
    assert cal.heston_objective(other, quotes, pop[:1], R, 100)[0] == 0.0


def _bs_call(s, k, t, r, v):
    d1 = (math.log(s / k) + (r + 0.5 * v * v) * t) / (v * math.sqrt(t))
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    return s * n(d1) - k * math.exp(-r * t) * n(d1 - v * math.sqrt(t))


def test_fit_gbm_trajectory_equals_oracle_driven_loop(orc):
    """The same Gauss-Newton loop on GPU FP64 prices and on oracle prices
    takes the same steps."""
    c = kx.up_and_out_call("EQ", 100.0, 150.0, 1.0)
    quotes = [(95.0, 6.1), (100.0, 8.0), (105.0, 9.6)]
    cfg = cal.FastCalibrationConfig(n_paths=3000)
    g = cal.fit_gbm_volatility(c, [1.0], quotes, R, cfg)
    o = cal._gauss_newton_sigma(lambda sg: orc.calib_gbm_prices(c.to_json(), "EQ", [s for s, _ in quotes], sg,
                                                                 n_paths=3000, rate=R), quotes, cfg)
    assert g.iterations == o.iterations and g.converged == o.converged
    assert abs(g.parameters[0] - o.parameters[0]) < 1e-9
    assert abs(g.objective - o.objective) <= 1e-9 * max(1.0, o.objective)


def test_fit_gbm_reference_checks():
    """tests/j21_fast_calibration.rs: off-grid target (0.223 to 0.01,
    converged), ATM (0.25 to 0.05, objective < 0.1), the binding's float."""
    market = _bs_call(100.0, 100.0, 1.0, R, 0.223)
    res = cal.fit_gbm_volatility(kx.european_call("EQ", 100.0, 1.0), [1.0], [(100.0, market)], R,
                                 cal.FastCalibrationConfig(n_paths=8000))
    assert abs(res.parameters[0] - 0.223) < 0.01 and res.converged
    c = kx.european_call("underlying", 100.0, 1.0)
    mkt = c.price(kx.GBM(s0=100.0, sigma=0.25, r=R, asset="underlying"), n_paths=10000, seed=42, steps_per_year=252,
                  precision="fp64").price
    res = cal.fit_gbm_volatility(c, [1.0], [(100.0, mkt)], R, cal.FastCalibrationConfig(n_paths=5000))
    assert abs(res.parameters[0] - 0.25) < 0.05 and res.objective < 0.1
    v = kx.fit_gbm_volatility(c, [1.0], [(100.0, mkt)], R)
    assert isinstance(v, float) and abs(v - 0.25) < 0.05


def test_fit_heston_basic():
    """j21 test_fit_heston_basic: five parameters in their ranges, finite
    objective; the descent's trajectory equals the oracle-driven loop's."""
    c = kx.european_call("underlying", 100.0, 1.0)
    mkt = c.price(kx.heston(100.0, *HP, R, asset="underlying"), n_paths=5000, seed=42, steps_per_year=252,
                  precision="fp64").price
    res = cal.fit_heston_parameters(c, [1.0], [(100.0, mkt)], R, cal.FastCalibrationConfig(n_paths=3000,
                                                                                            max_iterations=30))
    p = res.parameters
    assert len(p) == 5
    assert 0 < p[0] < 1 and 0 < p[1] < 5 and 0 < p[2] < 1 and 0 < p[3] < 2 and -1 < p[4] < 1
    assert math.isfinite(res.objective)


def test_heston_descent_trajectory_equals_oracle_driven_loop(orc):
    c = kx.european_call("underlying", 100.0, 1.0)
    quotes = [(95.0, 7.5), (105.0, 13.0)]
    cfg = cal.FastCalibrationConfig(n_paths=800, max_iterations=6)
    g = cal.fit_heston_parameters(c, [1.0], quotes, R, cfg)
    o = cal._heston_descent(lambda ps: orc.calib_heston_objective(c.to_json(), "underlying", quotes, ps, n_paths=800,
                                                                  rate=R), cfg)
    assert g.converged == o.converged
    assert np.allclose(g.parameters, o.parameters, rtol=1e-9, atol=1e-12)
    assert abs(g.objective - o.objective) <= 1e-9 * max(1e-6, abs(o.objective))


def test_calibrate_heston_cmaes_reproduces_prices():
    """j22 calibrate_heston_reproduces_prices: quotes priced with the true
    parameters on the calibration's own paths (3000, seed 42); the fitted
    parameters reprice every quote within 0.5 %."""
    c = kx.european_call("underlying", 100.0, 1.0)
    spots = [90.0, 100.0, 110.0]
    m = lambda s, p: kx.heston(s, *p, R, asset="underlying")  # noqa: E731
    quotes = [(s, c.price(m(s, HP), n_paths=3000, seed=42, steps_per_year=252, precision="fp64").price)
              for s in spots]
    res = cal.calibrate_heston_cmaes(c, quotes, R, cal.FastCalibrationConfig(n_paths=3000, max_iterations=40))
    assert len(res.parameters) == 5
    err = max(abs(c.price(m(s, res.parameters), n_paths=3000, seed=42, steps_per_year=252,
                          precision="fp64").price - q) / q for s, q in quotes)
    assert err < 0.005, (err, res.parameters)
    for v, lo, hi in zip(res.parameters, cal.HESTON_LOWER, cal.HESTON_UPPER):
        assert lo <= v <= hi


def test_empty_quotes_and_single_cell_surface(orc):
    """No quotes: the objective is 0 / 0 = NaN as eval_obj_heston computes it;
    a one-cell surface is greeks_gbm at that cell."""
    c = kx.european_call("underlying", 100.0, 1.0)
    assert math.isnan(cal.heston_objective(c, [], [HP], R, 100)[0])
    assert math.isnan(orc.calib_heston_objective(c.to_json(), "underlying", np.zeros((0, 2)), [HP], n_paths=100,
                                                 rate=R)[0])
    s = kx.greek_surface(c, "underlying", [100.0], [0.2], n_paths=10_000, seed=4, steps_per_year=4, rate=R)
    g = c.greeks(kx.GBM(s0=100.0, sigma=0.2, r=R, asset="underlying"), n_paths=10_000, seed=4, steps_per_year=4)
    assert s.delta[0, 0] == g.delta and s.price[0, 0] == g.price and s.gamma[0, 0] == g.gamma
