"""Correlated multi-factor GBM on the CPU: the oracle's restatement of
CorrelatedGbmN pricing against the reference's own checks
(tests/j27_basket.rs): the simulated correlation, a 3-asset basket against
Black-Scholes on the basket volatility, a spread against Margrabe, perfect
correlation degenerating to one asset, and the constructor's rejections."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx
from oracle import OracleError

S = kx.S


def _bs(s, k, t, r, v):
    d1 = (math.log(s / k) + (r + 0.5 * v * v) * t) / (v * math.sqrt(t))
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    return s * n(d1) - k * math.exp(-r * t) * n(d1 - v * math.sqrt(t))


def test_correlated_gbm_recovers_rho(orc):
    """j27 test_correlated_gbm_n_recovers_rho: the log-returns' correlation
    within 0.02 of 0.7 (two contracts paying S1(1) and S2(1) on the same paths)."""
    m = kx.CorrelatedGbmN([("S1", 100.0, 0.0, 0.25), ("S2", 100.0, 0.0, 0.20)], [[1.0, 0.7], [0.7, 1.0]])
    _, a = orc.price_multi((kx.scale(S("S1"), kx.one()) @ kx.at(1.0)).to_json(), m, n_paths=100_000,
                           steps_per_year=1, per_path=True)
    _, b = orc.price_multi((kx.scale(S("S2"), kx.one()) @ kx.at(1.0)).to_json(), m, n_paths=100_000,
                           steps_per_year=1, per_path=True)
    rho = np.corrcoef(np.log(a / 100.0), np.log(b / 100.0))[0, 1]
    assert abs(rho - 0.7) < 0.02


def test_basket_three_assets_vs_black_scholes(orc):
    s0, k, t, r, sg, rho = 100.0, 100.0, 1.0, 0.03, 0.2, 0.5
    m = kx.CorrelatedGbmN([(f"S{i}", s0, r, sg) for i in (1, 2, 3)],
                          [[1.0, rho, rho], [rho, 1.0, rho], [rho, rho, 1.0]], rate=r)
    c = kx.scale(((S("S1") + S("S2") + S("S3")) / 3.0 - k).clip(0.0), kx.one()) @ kx.at(t)
    res = orc.price_multi(c.to_json(), m, n_paths=200_000, seed=7, steps_per_year=50)
    ref = _bs(s0, k, t, r, sg * math.sqrt((1 + 2 * rho) / 3))
    assert abs(res.price - ref) / ref < 0.03


def test_spread_option_vs_margrabe(orc):
    s0, t, r, s1, s2, rho = 100.0, 1.0, 0.03, 0.2, 0.2, 0.5
    m = kx.CorrelatedGbmN([("S1", s0, r, s1), ("S2", s0, r, s2)], [[1.0, rho], [rho, 1.0]], rate=r)
    c = kx.scale((S("S1") - S("S2")).clip(0.0), kx.one()) @ kx.at(t)
    res = orc.price_multi(c.to_json(), m, n_paths=300_000, seed=11, steps_per_year=50)
    ref = _bs(s0, s0, t, 0.0, math.sqrt(s1 * s1 + s2 * s2 - 2 * rho * s1 * s2))
    assert abs(res.price - ref) / ref < 0.03


def test_perfect_correlation_degenerates_to_single_asset(orc):
    s0, k, t, r, sg = 100.0, 100.0, 1.0, 0.03, 0.2
    m = kx.CorrelatedGbmN([("S1", s0, r, sg), ("S2", s0, r, sg)], [[1.0, 1.0], [1.0, 1.0]], rate=r)
    c = kx.scale(((S("S1") + S("S2")) / 2.0 - k).clip(0.0), kx.one()) @ kx.at(t)
    res = orc.price_multi(c.to_json(), m, n_paths=100_000, seed=3, steps_per_year=50)
    assert abs(res.price - _bs(s0, k, t, r, sg)) / _bs(s0, k, t, r, sg) < 0.02


def test_constructor_validates_inputs(orc):
    with pytest.raises(kx.KontractError):
        kx.CorrelatedGbmN([("S1", 100.0, 0.03, 0.2), ("S2", 100.0, 0.03, 0.2), ("S3", 100.0, 0.03, 0.2)],
                          [[1.0, 0.5], [0.5, 1.0]])
    one = kx.CorrelatedGbmN([("S1", 100.0, 0.03, 0.2)], [[1.0]])
    c = kx.european_call("S1", 100.0, 1.0)
    with pytest.raises(OracleError) as e:
        orc.price_multi(c.to_json(), one, n_paths=100)
    assert e.value.status == "MalformedContract"
    neg = kx.CorrelatedGbmN([("S1", 100.0, 0.03, 0.2), ("S2", 100.0, 0.03, -0.1)], [[1.0, 0.0], [0.0, 1.0]])
    with pytest.raises(OracleError) as e:
        orc.price_multi(c.to_json(), neg, n_paths=100)
    assert e.value.status == "MalformedContract"
    two = kx.CorrelatedGbmN([("S1", 100.0, 0.03, 0.2), ("S2", 100.0, 0.03, 0.2)], [[1.0, 0.0], [0.0, 1.0]])
    with pytest.raises(OracleError) as e:
        orc.price_multi(kx.european_call("S9", 100.0, 1.0).to_json(), two, n_paths=100)
    assert e.value.status == "UnknownAsset"
