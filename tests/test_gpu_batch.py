"""GPU batch pricing: price_batch_gbm semantics (one shared simulation of the
merged grid, tests/portfolio.rs) and the uneven persistent portfolio launch
(the 256-contract book of tests/golden/portfolio_256.json)."""
import json
import os

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

BOOK = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "portfolio_256.json")))


def test_batch_matches_individual_same_grid():
    """tests/portfolio.rs:26-40: same maturity, so the merged grid is each
    contract's own grid and batch == individual to 1e-12."""
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="AAPL")
    calls = [kx.european_call("AAPL", float(k), 1.0) for k in range(80, 121, 4)]
    batch = kx.price_batch(calls, m, n_paths=50_000, seed=2024, steps_per_year=1, precision="fp64")
    for c, b in zip(calls, batch):
        single = c.price(m, n_paths=50_000, seed=2024, steps_per_year=1, precision="fp64")
        assert abs(single.price - b.price) < 1e-12
    assert all(a.price >= b.price - 1e-9 for a, b in zip(batch, batch[1:]))
    assert kx.price_batch([], m) == []


def test_batch_mixed_book_matches_oracle(orc):
    """Static flows (calls/puts at several dates) share one simulation; a
    barrier contract goes through the path kernel on the same grid."""
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X")
    book = [kx.european_call("X", 95.0, 0.5), kx.european_put("X", 105.0, 1.0), kx.european_call("X", 110.0, 2.0),
            kx.up_and_out_call("X", 100.0, 140.0, 1.5), kx.straddle("X", 100.0, 1.0),
            kx.zero_coupon_bond("USD", 2.0) + kx.give(kx.european_call("X", 120.0, 1.0))]
    res = kx.price_batch(book, m, n_paths=20_000, seed=77, steps_per_year=52, precision="fp64")
    ref = orc.price_batch([c.to_json() for c in book], m, n_paths=20_000, seed=77, steps_per_year=52)
    for r, q in zip(res, ref):
        assert abs(r.price - q.price) <= 1e-11 * max(1.0, abs(q.price)), (r.price, q.price)
        assert abs(r.std_error - q.std_error) <= 1e-9 * max(1.0, q.std_error)


def test_heston_batch_shared_simulation_matches_oracle(orc):
    """The Heston book shape (strikes x maturities on one simulation)."""
    h = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="X")
    book = [kx.european_call("X", k, t) for t in (0.5, 1.0, 2.0) for k in (90.0, 100.0, 115.0)]
    res = kx.price_batch(book, h, n_paths=10_000, seed=42, steps_per_year=52, precision="fp64")
    ref = orc.price_batch([c.to_json() for c in book], h, n_paths=10_000, seed=42, steps_per_year=52)
    for r, q in zip(res, ref):
        assert abs(r.price - q.price) <= 1e-9 * max(1.0, q.price), (r.price, q.price)
    r32 = kx.price_batch(book, h, n_paths=200_000, seed=42, steps_per_year=52)
    q32 = orc.price_batch([c.to_json() for c in book], h, n_paths=200_000, seed=42, steps_per_year=52)
    for r, q in zip(r32, q32):
        assert abs(r.price - q.price) < 3 * q.std_error + 1e-6


def _book(step=16, scale=0.05, prec="fp64"):
    sub = BOOK["contracts"][::step]
    cs = [kx.Contract.from_json(c["json"]) for c in sub]
    ms = [kx.GBM(s0=c["s0"], sigma=c["sigma"], r=c["r"], asset="S") for c in sub]
    ns = [max(1000, int(c["n_paths"] * scale)) for c in sub]
    seeds = [c["seed"] for c in sub]
    return sub, cs, ms, ns, seeds


def test_portfolio_equals_individual_prices():
    sub, cs, ms, ns, seeds = _book()
    res = kx.price_portfolio(cs, ms, ns, seeds, steps_per_year=252, precision="fp64")
    for c, m, n, s, r in zip(cs, ms, ns, seeds, res):
        single = c.price(m, n_paths=n, seed=s, steps_per_year=252, precision="fp64")
        assert single.price == r.price and single.std_error == r.std_error  # same paths, same reduction


def test_portfolio_matches_oracle(orc):
    sub, cs, ms, ns, seeds = _book(step=32, scale=0.02)
    res = kx.price_portfolio(cs, ms, ns, seeds, steps_per_year=252, precision="fp64")
    for c, m, n, s, r in zip(cs, ms, ns, seeds, res):
        q = orc.price(c.to_json(), m, n_paths=n, seed=s, steps_per_year=252)
        assert abs(r.price - q.price) <= 1e-12 * max(1.0, abs(q.price))


def test_portfolio_sensitivities_equal_individual_adjoints():
    sub, cs, ms, ns, seeds = _book(step=24, scale=0.02)
    res, sens = kx.price_portfolio(cs, ms, ns, seeds, steps_per_year=252, precision="fp64", greeks=True)
    for c, m, n, s, r, g in zip(cs, ms, ns, seeds, res, sens):
        a = c.adjoint(m, n_paths=n, seed=s, steps_per_year=252, precision="fp64")
        assert abs(g.d_s0 - a.d_s0) <= 1e-12 * max(1.0, abs(a.d_s0))
        assert abs(g.d_sigma - a.d_sigma) <= 1e-12 * max(1.0, abs(a.d_sigma))
        p = c.price(m, n_paths=n, seed=s, steps_per_year=252, precision="fp64")
        assert abs(r.price - p.price) <= 1e-10 * max(1.0, abs(p.price))  # hard-barrier price


def test_heston_book_matches_fourier_price(orc):
    """The Heston book shape (strikes x maturities on one simulation, full
    truncation, FP32 paths): every price within 3 standard errors plus the
    Euler bias allowance (0.03 at 252 steps a year) of the Fourier price."""
    h = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="X", scheme="full_truncation")
    ks, ts = (80.0, 95.0, 100.0, 110.0, 120.0), (0.5, 1.0, 2.0)
    book = [kx.european_call("X", k, t) for t in ts for k in ks]
    res = kx.price_batch(book, h, n_paths=1_000_000, seed=42, steps_per_year=252)
    for (t, k), r in zip([(t, k) for t in ts for k in ks], res):
        cf = orc.heston_call(100.0, k, t, 0.05, 0.04, 2.0, 0.04, 0.3, -0.5)
        assert abs(r.price - cf) < 3 * r.std_error + 0.03, (k, t, r.price, r.std_error, cf)
