"""Correlated multi-factor GBM on the GPU (kx_price_multi, the M_MULTI path
kernel): per-path values equal to the oracle's restatement in FP64 (baskets,
spreads, a barrier on the second factor, an average of the third), FP32
within the standard error, and the reference's own checks
(tests/j27_basket.rs) on the engine."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

S = kx.S
R = 0.03
M3 = lambda: kx.CorrelatedGbmN([("S1", 100.0, R, 0.2), ("S2", 95.0, R, 0.3), ("S3", 110.0, 0.01, 0.15)],  # noqa: E731
                               [[1.0, 0.5, 0.2], [0.5, 1.0, -0.3], [0.2, -0.3, 1.0]], rate=R)

CONTRACTS = {
    "basket": lambda: kx.scale(((S("S1") + S("S2") + S("S3")) / 3.0 - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "spread": lambda: kx.scale((S("S1") - S("S2")).clip(0.0), kx.one()) @ kx.at(0.75),
    "barrier_on_s2": lambda: kx.until(S("S2") >= 130.0, kx.scale((S("S1") - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)),
    "asian_on_s3": lambda: kx.scale((kx.average(S("S3")) - S("S1")).clip(0.0), kx.one()) @ kx.at(1.0),
    "worst_of": lambda: kx.scale(S("S1").min(S("S2")).min(S("S3")), kx.one()) @ kx.at(1.0),
}


@pytest.mark.parametrize("name", sorted(CONTRACTS))
def test_fp64_paths_equal_oracle(orc, name):
    c, m = CONTRACTS[name](), M3()
    r, pp = c.price(m, n_paths=4000, seed=5, steps_per_year=52, precision="fp64", per_path=True)
    o, op = orc.price_multi(c.to_json(), m, n_paths=4000, seed=5, steps_per_year=52, per_path=True)
    assert np.allclose(np.asarray(pp), op, rtol=1e-11, atol=1e-11), name
    assert abs(r.price - o.price) <= 1e-11 * max(1.0, abs(o.price))
    assert kx.last_launch_stats()["kernel_launches"] >= 1


@pytest.mark.parametrize("name", sorted(CONTRACTS))
def test_fp32_within_standard_error(orc, name):
    c, m = CONTRACTS[name](), M3()
    r = c.price(m, n_paths=200_000, seed=9, steps_per_year=52)
    o = orc.price_multi(c.to_json(), m, n_paths=200_000, seed=9, steps_per_year=52)
    assert abs(r.price - o.price) <= 0.05 * o.std_error + 1e-6 * abs(o.price), name


def _bs(s, k, t, r, v):
    d1 = (math.log(s / k) + (r + 0.5 * v * v) * t) / (v * math.sqrt(t))
    n = lambda x: 0.5 * (1 + math.erf(x / math.sqrt(2)))  # noqa: E731
    return s * n(d1) - k * math.exp(-r * t) * n(d1 - v * math.sqrt(t))


def test_reference_basket_spread_and_degenerate_checks():
    """tests/j27_basket.rs: basket vs BS(sigma_basket) < 3 %, spread vs
    Margrabe < 3 %, perfect correlation vs one asset < 2 %."""
    rho = 0.5
    m = kx.CorrelatedGbmN([(f"S{i}", 100.0, R, 0.2) for i in (1, 2, 3)],
                          [[1.0, rho, rho], [rho, 1.0, rho], [rho, rho, 1.0]], rate=R)
    b = CONTRACTS["basket"]().price(m, n_paths=200_000, seed=7, steps_per_year=50, precision="fp64").price
    ref = _bs(100.0, 100.0, 1.0, R, 0.2 * math.sqrt((1 + 2 * rho) / 3))
    assert abs(b - ref) / ref < 0.03
    m2 = kx.CorrelatedGbmN([("S1", 100.0, R, 0.2), ("S2", 100.0, R, 0.2)], [[1.0, rho], [rho, 1.0]], rate=R)
    sp = (kx.scale((S("S1") - S("S2")).clip(0.0), kx.one()) @ kx.at(1.0)).price(m2, n_paths=300_000, seed=11,
                                                                                steps_per_year=50).price
    ref = _bs(100.0, 100.0, 1.0, 0.0, math.sqrt(0.08 - 2 * rho * 0.04))
    assert abs(sp - ref) / ref < 0.03
    m1 = kx.CorrelatedGbmN([("S1", 100.0, R, 0.2), ("S2", 100.0, R, 0.2)], [[1.0, 1.0], [1.0, 1.0]], rate=R)
    d = (kx.scale(((S("S1") + S("S2")) / 2.0 - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)).price(
        m1, n_paths=100_000, seed=3, steps_per_year=50).price
    assert abs(d - _bs(100.0, 100.0, 1.0, R, 0.2)) / _bs(100.0, 100.0, 1.0, R, 0.2) < 0.02


def test_rejections():
    c = kx.european_call("S9", 100.0, 1.0)
    with pytest.raises(kx.KontractError) as e:
        c.price(M3(), n_paths=100)
    assert e.value.status == "UnknownAsset"
    with pytest.raises(kx.KontractError) as e:
        kx.european_call("S1", 100.0, 1.0).price(kx.CorrelatedGbmN([("S1", 100.0, R, 0.2)], [[1.0]]), n_paths=100)
    assert e.value.status == "MalformedContract"


def test_seven_factors_equal_oracle_and_eight_rejected(orc):
    """The largest factor count (KX_MAX_ASSETS = 7) in FP64 against the oracle;
    an eighth factor is refused on the host."""
    fac = [(f"A{i}", 90.0 + 3 * i, 0.02, 0.1 + 0.03 * i) for i in range(7)]
    corr = [[1.0 if i == j else 0.3 - 0.02 * abs(i - j) for j in range(7)] for i in range(7)]
    m = kx.CorrelatedGbmN(fac, corr, rate=R)
    tot = S("A0")
    for i in range(1, 7):
        tot = tot + S(f"A{i}")
    c = kx.until(S("A6") >= 150.0, kx.scale((tot / 7.0 - 100.0).clip(0.0), kx.one()) @ kx.at(1.0))
    r, pp = c.price(m, n_paths=3000, seed=21, steps_per_year=24, precision="fp64", per_path=True)
    o, op = orc.price_multi(c.to_json(), m, n_paths=3000, seed=21, steps_per_year=24, per_path=True)
    assert np.allclose(np.asarray(pp), op, rtol=1e-11, atol=1e-11)
    with pytest.raises(ValueError):
        kx.CorrelatedGbmN(fac + [("A7", 100.0, 0.0, 0.2)], [[1.0] * 8] * 8)
