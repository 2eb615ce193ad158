"""Calibration callers on the CPU: the optimizers' host logic and the
oracle's restatement of the objectives they call.

- cmaes_minimize on the reference's analytic checks (tests/j22_cmaes.rs:20-123):
  sphere, Rosenbrock, an optimum outside the box, reproducibility.
- The oracle's gbm_prices / eval_obj_heston (calibration.rs:72-126): each
  entry is the oracle's price_gbm, failing quotes give NaN / are skipped.
- fit_gbm_volatility's Gauss-Newton loop on oracle prices against the
  reference's assertions (tests/j21_fast_calibration.rs).
"""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import calibration as cal


def test_cmaes_minimizes_sphere():
    res = cal.cmaes_minimize(lambda x: float(np.sum(np.square(x))), [3.0, 3.0, 3.0],
                             cal.Bounds([-5.0] * 3, [5.0] * 3), cal.CmaesConfig(sigma0=1.0, max_generations=200, seed=7))
    assert math.sqrt(sum(x * x for x in res.best_params)) < 1e-3
    assert res.best_objective < 1e-5


def test_cmaes_minimizes_rosenbrock():
    f = lambda v: (1.0 - v[0]) ** 2 + 100.0 * (v[1] - v[0] * v[0]) ** 2  # noqa: E731
    res = cal.cmaes_minimize(f, [-1.0, -1.0], cal.Bounds([-5.0, -5.0], [5.0, 5.0]),
                             cal.CmaesConfig(population_size=16, sigma0=2.0, max_generations=500, seed=11))
    assert abs(res.best_params[0] - 1.0) < 0.01 and abs(res.best_params[1] - 1.0) < 0.01
    assert res.best_objective < 1e-3


def test_cmaes_respects_bounds():
    f = lambda x: float(np.sum((np.asarray(x) - 10.0) ** 2))  # noqa: E731
    res = cal.cmaes_minimize(f, [0.0, 0.0, 0.0], cal.Bounds([-1.0] * 3, [1.0] * 3),
                             cal.CmaesConfig(sigma0=0.5, max_generations=100, seed=3))
    for p in res.best_params:
        assert -1.0 <= p <= 1.0 and p > 0.9


def test_cmaes_is_reproducible_and_batch_equals_scalar():
    sphere = lambda x: float(np.sum(np.square(x)))  # noqa: E731
    b = cal.Bounds([-5.0] * 4, [5.0] * 4)
    cfg = cal.CmaesConfig(sigma0=1.0, max_generations=50, seed=99)
    r1 = cal.cmaes_minimize(sphere, [2.0, -2.0, 1.0, -1.0], b, cfg)
    r2 = cal.cmaes_minimize(sphere, [2.0, -2.0, 1.0, -1.0], b, cfg)
    r3 = cal.cmaes_minimize(None, [2.0, -2.0, 1.0, -1.0], b, cfg, objective_batch=lambda xs: [sphere(x) for x in xs])
    assert r1.best_params == r2.best_params == r3.best_params
    assert r1.best_objective == r2.best_objective == r3.best_objective


def test_strategy_constants():
    """optimizer.rs:113-170 at n = 5, lambda = 40 (the Heston calibration)."""
    st = cal._Strategy(5, 40)
    assert st.mu == 20 and abs(st.weights.sum() - 1.0) < 1e-15
    assert np.all(np.diff(st.weights) < 0)
    assert 0 < st.c_1 < 1 and 0 <= st.c_mu <= 1 - st.c_1
    assert abs(st.chi_n - math.sqrt(5) * (1 - 1 / 20 + 1 / 525)) < 1e-15


def test_oracle_gbm_prices_are_prices(orc):
    c = kx.european_call("EQ", 100.0, 1.0)
    out = orc.calib_gbm_prices(c.to_json(), "EQ", [90.0, 110.0], [0.2, 0.3], n_paths=4000, rate=0.05)
    for k, sg in enumerate([0.2, 0.3]):
        for i, s in enumerate([90.0, 110.0]):
            r = orc.price(c.to_json(), kx.GBM(s0=s, sigma=sg, r=0.05, asset="EQ"), n_paths=4000, seed=42,
                          steps_per_year=252)
            assert out[k, i] == r.price
    bad = orc.calib_gbm_prices(c.to_json(), "underlying", [100.0], [0.2], n_paths=100, rate=0.05)
    assert math.isnan(bad[0, 0])  # unknown asset: NaN (calibration.rs:86)


def test_oracle_heston_objective_semantics(orc):
    c = kx.european_call("underlying", 100.0, 1.0)
    p = [0.04, 2.0, 0.04, 0.3, -0.5]
    quotes = [(95.0, 9.0), (105.0, 14.0)]
    obj = orc.calib_heston_objective(c.to_json(), "underlying", quotes, [p], n_paths=500, rate=0.05)
    m = lambda s: kx.heston(s, *p, 0.05, asset="underlying")  # noqa: E731
    prices = [orc.price(c.to_json(), m(s), n_paths=500, seed=42, steps_per_year=252).price for s, _ in quotes]
    want = ((prices[0] - 9.0) ** 2 + (prices[1] - 14.0) ** 2) / 2
    assert obj[0] == want
    # the reference simulates "underlying": a contract on another asset prices nothing, objective 0
    other = kx.european_call("EQ", 100.0, 1.0)
    assert orc.calib_heston_objective(other.to_json(), "underlying", quotes, [p], n_paths=100, rate=0.05)[0] == 0.0
    # a parameter vector the model rejects prices nothing either (rho outside [-1, 1])
    assert orc.calib_heston_objective(c.to_json(), "underlying", quotes, [p[:4] + [1.5]], n_paths=100,
                                      rate=0.05)[0] == 0.0


def _bs_call(s, k, t, r, v):
    d1 = (math.log(s / k) + (r + 0.5 * v * v) * t) / (v * math.sqrt(t))
    d2 = d1 - v * math.sqrt(t)
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    return s * n(d1) - k * math.exp(-r * t) * n(d2)


def _oracle_fit(orc, contract, asset, quotes, rate, cfg):
    return cal._gauss_newton_sigma(
        lambda sigmas: orc.calib_gbm_prices(contract.to_json(), asset, [s for s, _ in quotes], sigmas,
                                            n_paths=cfg.n_paths, rate=rate), quotes, cfg)


def test_fit_gbm_off_grid_target(orc):
    """j21 test_fit_gbm_volatility_off_grid_target: sigma 0.223 to 0.01, converged."""
    market = _bs_call(100.0, 100.0, 1.0, 0.05, 0.223)
    c = kx.european_call("EQ", 100.0, 1.0)
    res = _oracle_fit(orc, c, cal.contract_asset(c), [(100.0, market)], 0.05, cal.FastCalibrationConfig(n_paths=8000))
    assert abs(res.parameters[0] - 0.223) < 0.01 and res.converged


def test_fit_gbm_multiple_spots_and_put(orc):
    """j21 test_fit_gbm_volatility_multiple_spots / test_fit_gbm_put."""
    c = kx.european_call("underlying", 100.0, 0.5)
    quotes = [(s, orc.price(c.to_json(), kx.GBM(s0=s, sigma=0.2, r=0.05, asset="underlying"), n_paths=10000,
                            seed=42, steps_per_year=252).price) for s in (90.0, 100.0, 110.0)]
    res = _oracle_fit(orc, c, "underlying", quotes, 0.05, cal.FastCalibrationConfig(n_paths=5000))
    assert abs(res.parameters[0] - 0.2) < 0.05
    put = kx.european_put("underlying", 100.0, 1.0)
    q = [(100.0, orc.price(put.to_json(), kx.GBM(s0=100.0, sigma=0.3, r=0.05, asset="underlying"), n_paths=10000,
                           seed=42, steps_per_year=252).price)]
    res = _oracle_fit(orc, put, "underlying", q, 0.05, cal.FastCalibrationConfig(n_paths=5000))
    assert abs(res.parameters[0] - 0.3) < 0.05 and res.objective < 0.1


def test_config_defaults():
    """j21 test_calibration_config_default."""
    c = cal.FastCalibrationConfig()
    assert c.n_paths == 1000 and c.max_iterations == 50 and c.tol_param > 0 and c.tol_obj > 0


def test_heston_clamp():
    """calibration.rs:128-141."""
    assert cal._clamp_heston([0.0, 0.0, 0.0, 3.0, -2.0]) == [0.001, 0.01, 0.001, 2.0, -0.99]
    assert cal._clamp_heston([0.5, 3.0, 0.2, 0.005, 1.5]) == [0.5, 3.0, 0.2, 0.01, 0.99]
