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


# ---------------------------------------------------------------------------
# k_multi_lean: contracts whose price conditions and amounts are affine in the
# factor spots, on a static schedule of time events (path_kernel 5); the
# others (an average, a min of two spots) stay on the general kernel (1).
# ---------------------------------------------------------------------------
def _basket3():
    return (S("S1") + S("S2") + S("S3")) / 3.0


LEAN = {
    "basket_knock_out": lambda: kx.until(_basket3() >= 125.0,
                                         kx.scale((_basket3() - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)),
    "spread_down_and_out": lambda: kx.until(S("S2") - S("S1") <= -30.0,
                                            kx.scale((S("S1") - S("S2")).clip(0.0), kx.one()) @ kx.at(0.75)),
    "bermudan_strip": lambda: (kx.scale((_basket3() - 100.0).clip(0.0), kx.one()) @ kx.at(0.5))
    + (kx.scale((_basket3() - 105.0).clip(0.0), kx.one()) @ kx.at(1.0)),
    "short_basket_put": lambda: -(kx.scale((100.0 - _basket3()).clip(0.0), kx.one()) @ kx.at(1.0)),
    "digital_double_knock_out": lambda: kx.until(_basket3() >= 125.0,
                                                 kx.until(S("S1") <= 80.0, kx.one() @ kx.at(1.0))),
    "capped_basket": lambda: kx.scale(_basket3().min(110.0), kx.one()) @ kx.at(1.0),
    "forward_on_difference": lambda: kx.scale(2.0 * S("S1") - S("S3"), kx.one()) @ kx.at(1.0),
    "knock_in_window": lambda: kx.until(S("S3") <= 90.0, kx.scale((S("S2") - 95.0).clip(0.0), kx.one()) @ kx.at(1.0))
    @ kx.at(0.25),
}


@pytest.mark.parametrize("name", sorted(LEAN))
def test_affine_kernel_fp64_paths_equal_oracle(orc, name):
    c, m = LEAN[name](), M3()
    r, pp = c.price(m, n_paths=4000, seed=5, steps_per_year=52, precision="fp64", per_path=True)
    assert kx.last_launch_stats()["path_kernel"] == 5, name
    o, op = orc.price_multi(c.to_json(), m, n_paths=4000, seed=5, steps_per_year=52, per_path=True)
    assert np.allclose(np.asarray(pp), op, rtol=1e-11, atol=1e-11), name
    assert abs(r.price - o.price) <= 1e-11 * max(1.0, abs(o.price))


@pytest.mark.parametrize("name", ["asian_on_s3", "worst_of"])
def test_non_affine_contracts_stay_on_the_general_kernel(name):
    CONTRACTS[name]().price(M3(), n_paths=1000, seed=5, steps_per_year=52)
    assert kx.last_launch_stats()["path_kernel"] == 1


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(LEAN))
def test_affine_kernel_equals_general_kernel(monkeypatch, name, precision):
    """The same paths through the general kernel (KX_PATH_KERNEL=general): FP64
    to 1e-12; FP32 to the rounding of the affine forms, which add their terms
    in another order than the interpreter (a few FP32 ulps of the spot level,
    1e-6 of max(|pv|, 100))."""
    c, m = LEAN[name](), M3()
    kw = dict(n_paths=50_000, seed=13, steps_per_year=252, precision=precision, per_path=True)
    r, pp = c.price(m, **kw)
    assert kx.last_launch_stats()["path_kernel"] == 5
    monkeypatch.setenv("KX_PATH_KERNEL", "general")
    g, gp = c.price(m, **kw)
    assert kx.last_launch_stats()["path_kernel"] == 1
    pp, gp = np.asarray(pp), np.asarray(gp)
    if precision == "fp64":
        assert np.allclose(pp, gp, rtol=1e-12, atol=1e-12), name
    else:
        d = np.abs(pp - gp)
        assert np.all(d <= 1e-6 * np.maximum(np.abs(gp), 100.0)), (name, float(d.max()))
    assert abs(r.price - g.price) <= 1e-3 * r.std_error + 1e-12


def _scaled(m, f):
    return kx.CorrelatedGbmN([(n, s0 * f, mu, sg) for n, s0, mu, sg in m.factors], m.corr, rate=m.rate)


def test_affine_kernel_fp32_per_path_at_benchmark_shape(orc):
    """The 5-factor knock-out basket of the benchmark (252 steps a year) in
    FP32 against the FP64 oracle, path by path: forward error 1e-5, or the
    oracle's value for every spot scaled by 1 +- 1e-5 (the factor log-spots
    do not depend on s0, so the whole path scales). The backward form serves
    the paths whose basket ends near the strike: the FP32 basket carries the
    rounding of five spots and of the Cholesky mix (measured: 1.9 % of
    paths)."""
    from parity import REL, fp32_check
    n_f = 5
    m = kx.CorrelatedGbmN([(f"S{i}", 100.0, 0.03, 0.15 + 0.05 * i) for i in range(n_f)],
                          [[1.0 if i == j else 0.4 for j in range(n_f)] for i in range(n_f)], rate=0.03)
    basket = (S("S0") + S("S1") + S("S2") + S("S3") + S("S4")) / 5.0
    c = kx.until(basket >= 130.0, kx.scale((basket - 100.0).clip(0.0), kx.one()) @ kx.at(1.0))
    n, kw = 20_000, dict(seed=42, steps_per_year=252)
    r, pp = c.price(m, n_paths=n, precision="fp32", per_path=True, **kw)
    assert kx.last_launch_stats()["path_kernel"] == 5
    _, ref = orc.price_multi(c.to_json(), m, n_paths=n, per_path=True, **kw)
    _, dn = orc.price_multi(c.to_json(), _scaled(m, 1.0 - REL), n_paths=n, per_path=True, **kw)
    _, up = orc.price_multi(c.to_json(), _scaled(m, 1.0 + REL), n_paths=n, per_path=True, **kw)
    ok, fwd = fp32_check(pp, ref, dn, up)
    assert ok.all(), (int((~ok).sum()), np.flatnonzero(~ok)[:5])
    assert fwd.mean() > 0.95, float(fwd.mean())
