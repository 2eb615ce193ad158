"""Multilevel Monte Carlo on the GPU (kx_price_mlmc): the per-level
statistics of the coupled fine / coarse paths against the oracle's
level_samples in FP64, whole estimates (allocation, level paths, price)
against the oracle's price_mlmc_detailed, and the reference's own checks
(tests/j18_mlmc.rs) on the engine."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

S0, K, T, R = 100.0, 100.0, 1.0, 0.05


def _heston():
    return kx.heston(S0, 0.04, 1.5, 0.04, 0.3, -0.7, R, asset="S")


MODELS = {"gbm": lambda: kx.GBM(s0=S0, sigma=0.2, r=R, asset="S"), "heston": _heston}
CONTRACTS = {
    "call": lambda: kx.european_call("S", K, T),
    "up_and_out": lambda: kx.up_and_out_call("S", K, 125.0, T),
    "asian": lambda: kx.scale((kx.average(kx.S("S")) - K).clip(0.0), kx.one()) @ kx.at(T),
}


@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("name", sorted(CONTRACTS))
def test_level_variance_matches_oracle(orc, model, name):
    """estimate_variance_at_level = the oracle's sample variance of
    P_l - P_(l-1) over the same coupled Philox paths (FP64)."""
    c, m = CONTRACTS[name](), MODELS[model]()
    for level in (0, 1, 4):
        ys = orc.mlmc_level_values(c.to_json(), m, level, 3000, seed=5)
        ref = float(np.var(ys, ddof=1))
        got = kx.estimate_variance_at_level(c, m, level, 3000, seed=5)
        assert abs(got - ref) <= 1e-9 * max(ref, 1e-12), (name, model, level, got, ref)


@pytest.mark.parametrize("model", sorted(MODELS))
def test_price_mlmc_matches_oracle(orc, model):
    c, m = CONTRACTS["up_and_out"](), MODELS[model]()
    g = kx.price_mlmc_detailed(c, m, kx.MlmcConfig(n_levels=5, pilot_paths=2000, target_variance=0.05 ** 2),
                               seed=11)
    o = orc.price_mlmc(c.to_json(), m, n_levels=5, pilot_paths=2000, target_variance=0.05 ** 2, seed=11)
    assert g.level_paths == o["level_paths"] and g.level_costs == o["level_costs"]
    assert g.total_cost == o["total_cost"]
    assert abs(g.price.price - o["price"].price) <= 1e-10 * abs(o["price"].price)
    assert abs(g.price.std_error - o["price"].std_error) <= 1e-8 * o["price"].std_error
    for a, b in zip(g.level_variances, o["level_variances"]):
        assert abs(a - b) <= 1e-8 * max(b, 1e-12)


def test_mlmc_call_matches_black_scholes_gbm():
    """j18 mlmc_call_matches_black_scholes_gbm."""
    r = kx.price_mlmc(CONTRACTS["call"](), MODELS["gbm"](), kx.MlmcConfig(n_levels=6, pilot_paths=2000,
                                                                          target_variance=0.02 ** 2), seed=7)
    d1 = (math.log(S0 / K) + (R + 0.02) * T) / 0.2
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    bs = S0 * n(d1) - K * math.exp(-R * T) * n(d1 - 0.2)
    assert abs(r.price - bs) < 0.06 and r.ci95_low <= bs <= r.ci95_high


def test_heston_variance_decay_and_cost_scaling():
    """j18 variance_decomposition_decays_with_level and
    cost_scales_as_epsilon_minus_two."""
    d = kx.price_mlmc_detailed(CONTRACTS["call"](), _heston(), kx.MlmcConfig(n_levels=5, pilot_paths=8000,
                                                                            target_variance=0.05 ** 2), seed=11)
    v = d.level_variances
    assert v[1] < 0.5 * v[0] and v[5] < 0.5 * v[1]
    assert np.mean([v[l + 1] / v[l] for l in range(1, 5)]) < 0.95
    cost = lambda tol: kx.price_mlmc_detailed(CONTRACTS["call"](), _heston(),  # noqa: E731
                                              kx.MlmcConfig(n_levels=5, pilot_paths=1000, target_variance=tol * tol),
                                              seed=11).total_cost
    assert 2.5 <= cost(0.04) / cost(0.08) <= 6.0


def test_mlmc_heston_matches_single_level_mc():
    """j18 mlmc_heston_matches_single_level_mc (plain MC on the engine)."""
    m = kx.price_mlmc(CONTRACTS["call"](), _heston(), kx.MlmcConfig(n_levels=6, pilot_paths=2000,
                                                                     target_variance=0.03 ** 2), seed=11).price
    std = CONTRACTS["call"]().price(_heston(), n_paths=400_000, seed=99, steps_per_year=64, precision="fp64").price
    assert abs(m - std) / std < 0.02


def test_rejections():
    c = CONTRACTS["call"]()
    with pytest.raises(kx.KontractError) as e:
        kx.price_mlmc(c, MODELS["gbm"](), kx.MlmcConfig(n_levels=21))
    assert e.value.status == "InvalidArgument"
    with pytest.raises(kx.KontractError) as e:
        kx.price_mlmc(c, kx.heston(S0, 0.04, 1.5, 0.04, 0.3, -0.7, R, asset="S", scheme="full_truncation"))
    assert e.value.status == "Unsupported"


def test_no_pilot_allocates_one_path_per_level(orc):
    """pilot_paths = 0: every level's variance is 0, optimal_allocation gives
    one path per level (mlmc.rs:250-252), all on the second seed."""
    c, m = CONTRACTS["call"](), MODELS["gbm"]()
    g = kx.price_mlmc_detailed(c, m, kx.MlmcConfig(n_levels=3, pilot_paths=0, target_variance=1e-4), seed=2)
    o = orc.price_mlmc(c.to_json(), m, n_levels=3, pilot_paths=0, target_variance=1e-4, seed=2)
    assert g.level_paths == o["level_paths"] == [1, 1, 1, 1]
    assert abs(g.price.price - o["price"].price) <= 1e-10 * max(1.0, abs(o["price"].price))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("model", sorted(MODELS))
@pytest.mark.parametrize("name", sorted(CONTRACTS))
def test_lean_level_pairs_equal_general_kernel(monkeypatch, precision, model, name):
    """The paths of a level pair in one k_mlmc_pairs launch (fine and coarse
    paths on the same Philox blocks; contracts on static schedules without
    averages), or on k_lean (the Asian: the running average in registers),
    and on k_paths (KX_PATH_KERNEL=general) are the same arithmetic on the
    same normals: the level variances agree exactly."""
    c, m = CONTRACTS[name](), MODELS[model]()
    got = [kx.estimate_variance_at_level(c, m, level, 20_000, seed=3, precision=precision) for level in (1, 3, 6)]
    assert (kx.last_launch_stats()["path_kernel"] == 6) == (name != "asian")
    monkeypatch.setenv("KX_PATH_KERNEL", "general")
    ref = [kx.estimate_variance_at_level(c, m, level, 20_000, seed=3, precision=precision) for level in (1, 3, 6)]
    assert got == ref, (name, model, precision, got, ref)
