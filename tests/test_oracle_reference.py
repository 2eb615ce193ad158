"""The oracle pinned against the reference's own tests (CPU only).

The reference publishes no per-path golden vectors; its tests pin exact
sigma = 0 prices, closed forms (Black-Scholes, Reiner-Rubinstein + BGK, CRR),
compiler plans and statistical tolerances. Each test below restates one of
them (file:line in the docstring) against the oracle. The reference draws
ChaCha8 normals (unpinned third-party crates), the oracle Philox ones, so the
stochastic assertions use the same tolerances on a different stream.
"""
import json
import math
import os

import numpy as np
import pytest

import kontracts_gb300 as kx

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def gbm(s0=100.0, sigma=0.2, r=0.05, asset="AAPL", q=0.0):
    return kx.GBM(s0=s0, sigma=sigma, r=r, q=q, asset=asset)


# ---- exact cases -----------------------------------------------------------
@pytest.mark.parametrize("case", GOLD["sigma_zero"], ids=lambda c: c["ref"])
def test_sigma_zero_exact(orc, case):
    """tests/pricer.rs:58-106 (sigma = 0, Gbm(AAPL, 100, 0.05, 0), n=16, spy=4)."""
    m = gbm(sigma=0.0, r=0.05)
    r = orc.price(case["json"], m, n_paths=16, seed=1, steps_per_year=4, rate=case["rate"])
    assert abs(r.price - case["price"]) <= case["tol"]


@pytest.mark.parametrize("case", GOLD["barrier_exact"], ids=lambda c: c["ref"])
def test_barrier_exact(orc, case):
    """tests/barriers.rs:104-153."""
    m = kx.GBM(s0=case["s0"], sigma=case["sigma"], r=case["mu"], asset="AAPL")
    r = orc.price(case["json"], m, n_paths=case["n_paths"], seed=case["seed"], steps_per_year=case["spy"],
                  rate=case["rate"])
    assert abs(r.price - case["price"]) <= case["tol"]


@pytest.mark.parametrize("case", GOLD["on_path"], ids=lambda c: c["ref"])
def test_observables_on_hand_built_paths(orc, case):
    """tests/j26_temporal_obs.rs:23-71: averages and running extrema on fixed paths."""
    v = orc.value_on_path(case["json"], case["times"], case["values"], "S", 0.0)
    assert abs(v - case["value"]) <= case["tol"]


def test_or_is_unsupported(orc):
    """tests/pricer.rs:132-140."""
    with pytest.raises(ValueError) as e:
        orc.price('{"Or":[{"One":"USD"},{"One":"USD"}]}', gbm(sigma=0.0), n_paths=16, seed=1, steps_per_year=4)
    assert e.value.status == "Unsupported"


# ---- compiler --------------------------------------------------------------
@pytest.mark.parametrize("case", GOLD["plans"], ids=lambda c: c["ref"])
def test_plans(orc, case):
    """tests/compiler.rs:19-122."""
    p = orc.plan(case["json"])
    assert p["assets"] == case["assets"]
    assert p["fixed_dates"] == case["fixed_dates"]
    assert p["horizon"] == case["horizon"]
    assert p["needs_fine_grid"] == case["needs_fine_grid"]
    for spy, g in case.get("grids", {}).items():
        assert orc.time_grid(case["json"], int(spy)) == g
    for spy, n in case.get("grid_len", {}).items():
        g = orc.time_grid(case["json"], int(spy))
        assert len(g) == n and g[0] == 0.0 and g[-1] == 1.0
    for spy, t in case.get("grid_contains", {}).items():
        assert any(abs(x - t) < 1e-12 for x in orc.time_grid(case["json"], int(spy)))


def test_negative_date_is_malformed(orc):
    for case in GOLD["malformed"]:
        with pytest.raises(ValueError) as e:
            orc.plan(case["json"])
        assert e.value.status == case["status"]


def test_garbage_json_rejected(orc):
    """tests/ast.rs:98-102."""
    for case in GOLD["garbage"]:
        with pytest.raises(ValueError) as e:
            orc.parse(case["json"])
        assert e.value.status == "Serde"


@pytest.mark.parametrize("js", GOLD["roundtrip"])
def test_roundtrip_contracts_parse(orc, js):
    """tests/ast.rs:77-97: the ten contracts parse from their serde form."""
    orc.parse(js)


# ---- diagnostics (tests/diagnostics.rs) -------------------------------------
CALL = GOLD["roundtrip"][8].replace("150.0", "100.0")


def test_deterministic_payoff_has_zero_error(orc):
    """tests/diagnostics.rs:14-31."""
    r = orc.price('{"When":[{"At":1.0},{"One":"USD"}]}', gbm(sigma=0.0), n_paths=1000, seed=1, steps_per_year=1)
    assert r.sample_std < 1e-12 and r.std_error < 1e-12
    assert abs(r.ci95_low - r.price) < 1e-12 and abs(r.ci95_high - r.price) < 1e-12
    assert r.n_paths == 1000


def test_ci_width_and_bracketing(orc):
    """tests/diagnostics.rs:33-50."""
    r = orc.price(CALL, gbm(), n_paths=100_000, seed=7, steps_per_year=1)
    assert r.std_error > 0 and r.ci95_low < r.price < r.ci95_high
    assert abs((r.ci95_high - r.ci95_low) - 2 * GOLD["z95"]["value"] * r.std_error) < 1e-9


def test_bs_value_inside_interval(orc):
    """tests/diagnostics.rs:52-71 (BS 10.450583572185565, 500k paths): asserted
    as |price - BS| < 3 SE on the oracle's Philox stream."""
    r = orc.price(CALL, gbm(), n_paths=500_000, seed=2024, steps_per_year=1)
    bs = GOLD["bs_call_atm"]["value"]
    assert abs(r.price - bs) < 3 * r.std_error
    assert abs(orc.bs_call(100, 100, 1, 0.05, 0.2) - bs) < 1e-5  # A&S cdf (~1e-7) vs exact


def test_paths_for_tolerance(orc):
    """tests/diagnostics.rs:73-105."""
    r = orc.price(CALL, gbm(), n_paths=50_000, seed=11, steps_per_year=1)
    a, b = r.paths_for_tolerance(0.10), r.paths_for_tolerance(0.05)
    assert b > a and abs(b / a - 4.0) < 0.05
    z = orc.price('"Zero"', gbm(sigma=0.0, r=0.0), n_paths=100, seed=1, steps_per_year=1)
    assert z.paths_for_tolerance(0.01) == 0


# ---- pricer vs closed forms ---------------------------------------------------
def test_european_call_vs_bs(orc):
    """tests/pricer.rs:108-130 (400k paths, rel < 1%)."""
    r = orc.price(CALL, gbm(), n_paths=400_000, seed=2024, steps_per_year=1)
    bs = orc.bs_call(100, 100, 1, 0.05, 0.2)
    assert abs(r.price - bs) / bs < 0.01


def test_down_and_out_vs_reiner_rubinstein_bgk(orc):
    """tests/barriers.rs:55-84 (H=90, 250 steps, 300k paths, BGK shift, rel < 2%)."""
    ko = '{"Until":[{"Le":[{"Spot":"AAPL"},{"Const":90.0}]},%s]}' % CALL
    r = orc.price(ko, gbm(), n_paths=300_000, seed=2024, steps_per_year=250)
    dt = 1.0 / 250
    an = orc.down_and_out_call(100, 100, 90 * math.exp(-0.5826 * 0.2 * math.sqrt(dt)), 0.05, 0.2, 1.0)
    assert abs(r.price - an) / an < 0.02


def test_unreachable_barrier_is_vanilla(orc):
    """tests/barriers.rs:86-102."""
    ko = '{"Until":[{"Le":[{"Spot":"AAPL"},{"Const":1.0}]},%s]}' % CALL
    r = orc.price(ko, gbm(), n_paths=200_000, seed=7, steps_per_year=50)
    bs = orc.bs_call(100, 100, 1, 0.05, 0.2)
    assert abs(r.price - bs) / bs < 0.01


def test_knock_out_below_vanilla(orc):
    """tests/barriers.rs:155-176."""
    ko = '{"Until":[{"Le":[{"Spot":"AAPL"},{"Const":95.0}]},%s]}' % CALL
    r = orc.price(ko, gbm(), n_paths=100_000, seed=3, steps_per_year=100)
    assert 0 < r.price < orc.bs_call(100, 100, 1, 0.05, 0.2)


def test_up_and_out_vs_closed_form(orc):
    """Up-and-out call (the C2 contract shape) vs the Reiner-Rubinstein formula
    with the upward BGK shift; the reference only has inequality tests for it
    (tests/products_validation.rs:119-131), this pins the oracle's barrier
    semantics to a published formula."""
    uo = kx.up_and_out_call("AAPL", 100.0, 130.0, 1.0).to_json()
    spy = 252
    r = orc.price(uo, gbm(), n_paths=400_000, seed=99, steps_per_year=spy)
    an = orc.up_and_out_call(100, 100, 130 * math.exp(0.5826 * 0.2 * math.sqrt(1.0 / spy)), 0.05, 0.2, 1.0)
    assert abs(r.price - an) < max(4 * r.std_error, 0.01 * an), (r.price, an, r.std_error)
    van = orc.price(CALL, gbm(), n_paths=100_000, seed=1, steps_per_year=spy)
    assert r.price < van.price


# ---- greeks (tests/greeks.rs) --------------------------------------------------
@pytest.fixture(scope="module")
def call_greeks(orc):
    return orc.greeks(CALL, gbm(), n_paths=500_000, seed=2024, steps_per_year=1)


def test_greeks_vs_bs(orc, call_greeks):
    """tests/greeks.rs:65-122: delta < 1%, vega < 2%, rho < 2%."""
    bs = orc.bs_call_greeks(100, 100, 1, 0.05, 0.2)
    g = call_greeks
    assert abs(g["delta"] - bs["delta"]) / bs["delta"] < 0.01
    assert abs(g["vega"] - bs["vega"]) / bs["vega"] < 0.02
    assert abs(g["rho"] - bs["rho"]) / bs["rho"] < 0.02
    assert 0 < g["delta"] < 1 and g["gamma"] > 0 and g["vega"] > 0


def test_gamma_vs_bs(orc):
    """tests/greeks.rs:124-148: gamma with a 1.0 spot bump, < 5%."""
    g = orc.greeks(CALL, gbm(), n_paths=500_000, seed=2024, steps_per_year=1, bumps=(1.0, 1e-2, 1e-4))
    bs = orc.bs_call_greeks(100, 100, 1, 0.05, 0.2)
    assert abs(g["gamma"] - bs["gamma"]) / bs["gamma"] < 0.05


# ---- simulator (tests/simulator.rs) ----------------------------------------------
def test_simulator_moments_and_reproducibility(orc):
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="AAPL")
    a = orc.simulate(m, [0.0, 0.5, 1.0], 1000, 7)
    assert np.all(a[:, 0] == 100.0)  # tests/simulator.rs:29-36
    st = orc.simulate(m, [0.0, 1.0], 200_000, 42)[:, 1]
    theo = 100 * math.exp(0.05)
    var = 100 ** 2 * math.exp(0.1) * (math.exp(0.04) - 1)
    assert abs(st.mean() - theo) < 3 * math.sqrt(var / len(st))  # :38-56
    lg = np.log(orc.simulate(m, [0.0, 1.0], 200_000, 123)[:, 1] / 100)
    assert abs(lg.mean() - (0.05 - 0.02)) < 3 * math.sqrt(0.04 / len(lg))  # :58-82
    assert abs(lg.var(ddof=1) - 0.04) / 0.04 < 0.02
    x = orc.simulate(m, [0.0, 1.0], 1000, 2024)
    assert np.array_equal(x, orc.simulate(m, [0.0, 1.0], 1000, 2024))  # :84-89
    assert not np.array_equal(x, orc.simulate(m, [0.0, 1.0], 1000, 2025))  # :91-96


def test_invalid_grids_rejected(orc):
    """tests/simulator.rs:115-129."""
    m = gbm()
    for g in ([], [0.0, 1.0, 0.5]):
        with pytest.raises(ValueError) as e:
            orc.simulate(m, g, 10, 1)
        assert e.value.status == "InconsistentPath"


# ---- batch (tests/portfolio.rs) ---------------------------------------------------
def test_batch_matches_individual_and_is_monotone(orc):
    calls = [kx.european_call("AAPL", float(k), 1.0).to_json() for k in range(80, 121)]
    m = gbm()
    batch = orc.price_batch(calls, m, n_paths=50_000, seed=2024, steps_per_year=1)
    for js, b in zip(calls[::8], batch[::8]):
        assert abs(orc.price(js, m, n_paths=50_000, seed=2024, steps_per_year=1).price - b.price) < 1e-12
    assert all(a.price >= b.price - 1e-9 for a, b in zip(batch, batch[1:]))
    assert orc.price_batch([], m) == []


# ---- Heston (tests/j12_heston_dupire.rs) -------------------------------------------
def test_heston_sigma_v_zero_is_bs(orc):
    """:73-101 (sigma_v = 0, 300k paths, spy 50, rel < 1%)."""
    h = kx.heston(100.0, 0.04, 1.0, 0.04, 0.0, 0.0, 0.05, asset="AAPL")
    r = orc.price(CALL, h, n_paths=300_000, seed=42, steps_per_year=50)
    bs = orc.bs_call(100, 100, 1, 0.05, 0.2)
    assert abs(r.price - bs) / bs < 0.01


def test_heston_high_kappa_is_near_bs(orc):
    """:103-128 (kappa 100, sigma_v 0.01, rel < 1.5%)."""
    h = kx.heston(100.0, 0.04, 100.0, 0.04, 0.01, 0.0, 0.05, asset="AAPL")
    r = orc.price(CALL, h, n_paths=300_000, seed=42, steps_per_year=50)
    bs = orc.bs_call(100, 100, 1, 0.05, 0.2)
    assert abs(r.price - bs) / bs < 0.015


def test_heston_rho_moves_otm_call(orc):
    """:163-220 (K=115, kappa 0.5, sigma_v 0.8, 100 steps, 200k paths)."""
    grid = [i / 100 for i in range(101)]
    otm = kx.european_call("X", 115.0, 1.0).to_json()
    pos = orc.price_on_grid(otm, kx.heston(100, 0.04, 0.5, 0.04, 0.8, 0.8, 0.05, asset="X"), grid, 200_000, 42)
    neg = orc.price_on_grid(otm, kx.heston(100, 0.04, 0.5, 0.04, 0.8, -0.8, 0.05, asset="X"), grid, 200_000, 42)
    assert pos.price - neg.price > 0.05


def test_heston_validation(orc):
    """simulator.rs:556-580."""
    with pytest.raises(ValueError) as e:
        orc.price(CALL, kx.heston(100, 0.04, 1, 0.04, 0.3, 1.5, 0.05, asset="AAPL"), n_paths=10)
    assert e.value.status == "MalformedContract"


# ---- LSM (tests/j17_lsm.rs) ----------------------------------------------------------
def _put(k): return kx.scale((kx.const_(k) - kx.S("AAPL")).clip(0.0), kx.one()).to_json()
def _callp(k): return kx.scale((kx.S("AAPL") - kx.const_(k)).clip(0.0), kx.one()).to_json()
def _dates(t, n): return [t * i / n for i in range(1, n + 1)]


def test_lsm_call_equals_european(orc):
    """:109-131 (20 dates, 60k paths, seed 7, rel < 2%)."""
    r = orc.price_american(_callp(95.0), gbm(), _dates(1.0, 20), n_paths=60_000, seed=7, n_basis=3)
    bs = orc.bs_call(100, 95, 1, 0.05, 0.2)
    assert abs(r.price - bs) / bs < 0.02


def test_lsm_put_exceeds_european(orc):
    """:133-155."""
    m = gbm(r=0.06, sigma=0.25)
    r = orc.price_american(_put(110.0), m, _dates(1.0, 20), n_paths=60_000, seed=7, n_basis=3)
    assert r.price - orc.bs_put(100, 110, 1, 0.06, 0.25) > 0.05


def test_lsm_vs_crr(orc):
    """:157-209 (50 dates, CRR 500 steps, rel < 1%)."""
    c = orc.price_american(_callp(100.0), gbm(), _dates(1.0, 50), n_paths=60_000, seed=7, n_basis=3)
    crr_c = orc.crr_american(100, 100, 1, 0.05, 0.2, 500, True)
    assert abs(c.price - crr_c) / crr_c < 0.01
    m = gbm(r=0.06, sigma=0.25)
    p = orc.price_american(_put(100.0), m, _dates(1.0, 50), n_paths=60_000, seed=7, n_basis=3)
    crr_p = orc.crr_american(100, 100, 1, 0.06, 0.25, 500, False)
    assert abs(p.price - crr_p) / crr_p < 0.01
    assert p.price >= 0.0


def test_lsm_basis_sensitivity(orc):
    """:211-231."""
    m = gbm(r=0.05, sigma=0.3)
    p2 = orc.price_american(_put(105.0), m, _dates(1.0, 40), n_paths=60_000, seed=7, n_basis=2).price
    p3 = orc.price_american(_put(105.0), m, _dates(1.0, 40), n_paths=60_000, seed=7, n_basis=3).price
    crr = orc.crr_american(100, 105, 1, 0.05, 0.3, 500, False)
    assert abs(p2 - p3) / p3 < 0.02 and abs(p3 - crr) / crr < 0.02


def test_lsm_validation(orc):
    """lsm.rs:87-105."""
    for dates, nb in (([], 3), ([0.5, 0.5], 3), ([0.0, 1.0], 3), ([1.0], 1)):
        with pytest.raises(ValueError) as e:
            orc.price_american(_put(100.0), gbm(), dates, n_paths=10, n_basis=nb)
        assert e.value.status == "MalformedContract"


# ---- temporal observables (tests/j26_temporal_obs.rs) ----------------------------
def test_asian_below_and_lookback_above_vanilla(orc):
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    asian = (kx.scale((kx.average(kx.S("S")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)).to_json()
    van = (kx.scale((kx.S("S") - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)).to_json()
    a = orc.price(asian, m, n_paths=100_000, seed=42, steps_per_year=252).price
    v = orc.price(van, m, n_paths=100_000, seed=42, steps_per_year=252).price
    assert 0 < a < v
    lb = (kx.scale((kx.running_max(kx.S("S")) - 90.0).clip(0.0), kx.one()) @ kx.at(1.0)).to_json()
    v90 = (kx.scale((kx.S("S") - 90.0).clip(0.0), kx.one()) @ kx.at(1.0)).to_json()
    assert orc.price(lb, m, n_paths=100_000, seed=43, steps_per_year=252).price > \
        orc.price(v90, m, n_paths=100_000, seed=43, steps_per_year=252).price


# ---- properties (tests/properties.rs) ------------------------------------------------
@pytest.mark.parametrize("s_lo,bump,vol", [(20.0, 5.0, 0.05), (80.0, 1.0, 0.4), (110.0, 30.0, 0.8)])
def test_call_monotone_in_spot_and_strike(orc, s_lo, bump, vol):
    lo = orc.price(CALL, kx.GBM(s_lo, vol, 0.03, asset="AAPL"), n_paths=4000, seed=7, steps_per_year=1).price
    hi = orc.price(CALL, kx.GBM(s_lo + bump, vol, 0.03, asset="AAPL"), n_paths=4000, seed=7, steps_per_year=1).price
    assert hi >= lo - 1e-9 and lo >= -1e-9
    k_lo = kx.european_call("AAPL", s_lo, 1.0).to_json()
    k_hi = kx.european_call("AAPL", s_lo + bump, 1.0).to_json()
    m = kx.GBM(100.0, vol, 0.03, asset="AAPL")
    assert orc.price(k_hi, m, n_paths=4000, seed=9, steps_per_year=1).price <= \
        orc.price(k_lo, m, n_paths=4000, seed=9, steps_per_year=1).price + 1e-9


# ---- Philox stream -------------------------------------------------------------------
def test_philox_normals_are_standard(orc):
    z = np.concatenate([orc.normals(42, p, 64) for p in range(3000)])
    assert abs(z.mean()) < 4 / math.sqrt(len(z))
    assert abs(z.var() - 1) < 0.02
    assert not np.array_equal(orc.normals(42, 0, 8), orc.normals(43, 0, 8))


def test_heston_closed_form_limits_and_monte_carlo(orc):
    """The Heston Fourier price (oracle extra, not in the reference): as
    sigma_v -> 0 it tends to Black-Scholes at sigma = sqrt(theta) = sqrt(v0),
    linearly in rho * sigma_v; a fine-grid full-truncation Monte Carlo of the
    oracle agrees within 3 standard errors."""
    bs = orc.bs_call(100.0, 100.0, 1.0, 0.05, 0.2)
    d1 = orc.heston_call(100.0, 100.0, 1.0, 0.05, 0.04, 2.0, 0.04, 0.01, -0.5) - bs
    d2 = orc.heston_call(100.0, 100.0, 1.0, 0.05, 0.04, 2.0, 0.04, 0.001, -0.5) - bs
    assert abs(d1) < 0.01 and abs(d2) < 0.001 and abs(d1 / d2 - 10.0) < 1.0
    import kontracts_gb300 as kx
    m = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="X", scheme="full_truncation")
    r = orc.price(kx.european_call("X", 100.0, 1.0).to_json(), m, n_paths=100_000, seed=5, steps_per_year=400)
    cf = orc.heston_call(100.0, 100.0, 1.0, 0.05, 0.04, 2.0, 0.04, 0.3, -0.5)
    assert abs(r.price - cf) < 3 * r.std_error + 0.01, (r.price, r.std_error, cf)


def test_lsm_laguerre_basis_vs_crr(orc):
    """The weighted-Laguerre basis (an extra mode beside the reference's
    monomials) prices the American put within 1% of the CRR tree, like the
    monomial basis does (j17_lsm.rs:157-209 tolerance)."""
    m = gbm(r=0.06, sigma=0.25)
    for nb in (3, 4):
        p = orc.price_american(_put(100.0), m, _dates(1.0, 50), n_paths=60_000, seed=7, n_basis=nb, basis="laguerre")
        crr = orc.crr_american(100, 100, 1, 0.06, 0.25, 500, False)
        assert abs(p.price - crr) / crr < 0.01, (nb, p.price, crr)
