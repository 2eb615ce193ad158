"""Multilevel Monte Carlo on the CPU: the oracle's restatement of
price_mlmc_detailed (mlmc.rs) against the reference's own checks
(tests/j18_mlmc.rs), and optimal_allocation of the library (host arithmetic)
equal to the oracle's."""
import math

import numpy as np

import kontracts_gb300 as kx

S0, K, T, R, SIGMA = 100.0, 100.0, 1.0, 0.05, 0.2


def _call():
    return kx.european_call("S", K, T)


def _heston():
    return kx.heston(S0, 0.04, 1.5, 0.04, 0.3, -0.7, R, asset="S")


def _bs(s, k, t, r, v):
    d1 = (math.log(s / k) + (r + 0.5 * v * v) * t) / (v * math.sqrt(t))
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    return s * n(d1) - k * math.exp(-r * t) * n(d1 - v * math.sqrt(t))


def test_mlmc_call_matches_black_scholes_gbm(orc):
    """j18 mlmc_call_matches_black_scholes_gbm: within 0.06 and inside the CI."""
    r = orc.price_mlmc(_call().to_json(), kx.GBM(s0=S0, sigma=SIGMA, r=R, asset="S"), n_levels=6, pilot_paths=2000,
                       target_variance=0.02 ** 2, seed=7)
    bs = _bs(S0, K, T, R, SIGMA)
    assert abs(r["price"].price - bs) < 0.06
    assert r["price"].ci95_low <= bs <= r["price"].ci95_high


def test_variance_decomposition_decays_with_level(orc):
    """j18 variance_decomposition_decays_with_level (Heston, Euler)."""
    d = orc.price_mlmc(_call().to_json(), _heston(), n_levels=5, pilot_paths=8000, target_variance=0.05 ** 2,
                       seed=11)
    v = d["level_variances"]
    assert v[1] < 0.5 * v[0] and v[5] < 0.5 * v[1]
    assert np.mean([v[l + 1] / v[l] for l in range(1, 5)]) < 0.95


def test_cost_scales_as_epsilon_minus_two(orc):
    """j18 cost_scales_as_epsilon_minus_two: halving the tolerance costs 2.5x..6x."""
    cost = lambda tol: orc.price_mlmc(_call().to_json(), _heston(), n_levels=5, pilot_paths=1000,  # noqa: E731
                                      target_variance=tol * tol, seed=11)["total_cost"]
    assert 2.5 <= cost(0.04) / cost(0.08) <= 6.0


def test_mlmc_heston_matches_single_level_mc(orc):
    """j18 mlmc_heston_matches_single_level_mc: within 2 % of plain MC
    (400,000 paths, 64 steps a year)."""
    m = orc.price_mlmc(_call().to_json(), _heston(), n_levels=6, pilot_paths=2000, target_variance=0.03 ** 2,
                       seed=11)["price"].price
    std = orc.price(_call().to_json(), _heston(), n_paths=400_000, seed=99, steps_per_year=64).price
    assert abs(m - std) / std < 0.02


def test_level_zero_is_one_step_and_levels_telescope(orc):
    """Level 0 is P_0 on the grid [0, T]; a European payoff under exact GBM
    has fine and coarse terminal values equal up to rounding at every level."""
    m = kx.GBM(s0=S0, sigma=SIGMA, r=R, asset="S")
    y0 = orc.mlmc_level_values(_call().to_json(), m, 0, 5000, seed=3)
    assert abs(y0.mean() - _bs(S0, K, T, R, SIGMA)) < 4 * y0.std() / math.sqrt(5000)
    for level in (1, 3, 5):
        y = orc.mlmc_level_values(_call().to_json(), m, level, 2000, seed=3)
        assert np.max(np.abs(y)) < 1e-9


def test_optimal_allocation(orc):
    """j18 optimal_allocation_proportional_to_sqrt_variance, and the library's
    host arithmetic equal to the oracle's."""
    v = [200.0, 50.0, 12.5, 3.125, 0.781]
    c = [1, 3, 6, 12, 24]
    a = kx.optimal_allocation(v, c, 0.01 ** 2)
    assert a == orc.mlmc_optimal_allocation(v, c, 0.01 ** 2)
    assert all(n >= 1 for n in a)
    for k in range(len(v) - 1):
        want = math.sqrt(v[k] / c[k]) / math.sqrt(v[k + 1] / c[k + 1])
        assert abs(a[k] / a[k + 1] - want) / want < 0.01
    assert kx.optimal_allocation([0.0, 1.0], [1, 3], 0.1) == orc.mlmc_optimal_allocation([0.0, 1.0], [1, 3], 0.1)
    assert kx.optimal_allocation([0.0, 1.0], [1, 3], 0.1)[0] == 1
    assert kx.optimal_allocation([1.0, 1.0], [1, 3], 0.0) == [0, 0]
    assert kx.optimal_allocation([], [], 0.1) == []
