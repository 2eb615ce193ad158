"""GPU Longstaff-Schwartz against the oracle's restatement of lsm.rs.

On shared FP64 normals the engine must reproduce the oracle path by path
(1e-12) except where an exercise decision flips because payoff and fitted
continuation value agree to within 1e-9 (the Gram sums are added in a
different order; the oracle reports each path's margin); on Philox normals and in FP32 the price must sit within 3 combined
standard errors, and the American put must match the CRR tree (the
reference's own check, tests/j17_lsm.rs:40-72)."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu


def put(k, asset="X"):
    return kx.scale((kx.const_(k) - kx.S(asset)).clip(0.0), kx.one())


def dates(t, n):
    return [t * i / n for i in range(1, n + 1)]


@pytest.mark.parametrize("n_basis", [2, 3, 4])
def test_lsm_shared_draws_fp64_per_path(orc, n_basis):
    rng = np.random.default_rng(n_basis)
    n, nd = 4000, 25
    z = rng.standard_normal((n, nd))
    kx.set_shared_draws(z)
    orc.set_shared_draws(z)
    m = kx.GBM(s0=40.0, sigma=0.2, r=0.06, asset="X")
    c = put(40.0)
    ds = dates(1.0, nd)
    res, pv = c.price_american(m, ds, n_paths=n, seed=0, n_basis=n_basis, precision="fp64", shared_draws=True,
                               per_path=True)
    ref, rpv, _, margin = orc.price_american_detail(c.to_json(), m, ds, n_paths=n, seed=0, n_basis=n_basis,
                                                    shared=True)
    diff = np.abs(pv - rpv)
    bad = diff > 1e-12 * np.maximum(np.abs(rpv), 1.0)
    # a path may differ only through a decision within 1e-9 of the exercise boundary
    assert np.all(margin[bad] < 1e-9), float(margin[bad].max())
    assert abs(res.price - ref.price) <= float(diff.sum()) / n + 1e-12 * abs(ref.price)
    assert res.n_paths == n


def test_lsm_philox_fp64_and_fp32_match_oracle(orc):
    m = kx.GBM(s0=36.0, sigma=0.2, r=0.06, asset="X")
    c = put(40.0)
    ds = dates(1.0, 50)
    ref = orc.price_american(c.to_json(), m, ds, n_paths=50_000, seed=9, n_basis=4)
    r64 = c.price_american(m, ds, n_paths=50_000, seed=9, n_basis=4, precision="fp64")
    assert abs(r64.price - ref.price) < 1e-6 * ref.price
    r32 = c.price_american(m, ds, n_paths=50_000, seed=9, n_basis=4, precision="fp32")
    assert abs(r32.price - ref.price) < 3 * ref.std_error


@pytest.mark.parametrize("s0,sigma,t", [(36.0, 0.2, 1.0), (40.0, 0.4, 2.0), (44.0, 0.2, 2.0)])
def test_american_put_vs_crr(orc, s0, sigma, t):
    """Longstaff-Schwartz (2001) table cases, 50 exercise dates a year, 1M paths."""
    m = kx.GBM(s0=s0, sigma=sigma, r=0.06, asset="X")
    res = put(40.0).price_american(m, dates(t, int(50 * t)), n_paths=1_000_000, seed=42, n_basis=4)
    crr = orc.crr_american(s0, 40.0, t, 0.06, sigma, 1000, False)
    # LSM with a finite basis is biased low by a few cents at 50 dates a year
    assert abs(res.price - crr) < 0.01 * crr + 4 * res.std_error, (res.price, crr)
    assert res.price > orc.bs_put(s0, 40.0, t, 0.06, sigma)


def test_lsm_validation_and_unsupported_payoffs():
    m = kx.GBM(s0=40.0, sigma=0.2, r=0.06, asset="X")
    for ds, nb in (([], 3), ([0.5, 0.5], 3), ([0.0, 1.0], 3), ([1.0], 1)):
        with pytest.raises(kx.KontractError) as e:
            put(40.0).price_american(m, ds, n_paths=100, n_basis=nb)
        assert e.value.status == "MalformedContract"
    with pytest.raises(kx.KontractError) as e:
        (put(40.0) @ kx.at(1.0)).price_american(m, [0.5, 1.0], n_paths=100)
    assert e.value.status == "Unsupported"


def test_lsm_heston_matches_oracle(orc):
    h = kx.heston(40.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.06, asset="X")
    ds = dates(1.0, 12)
    ref = orc.price_american(put(40.0).to_json(), h, ds, n_paths=30_000, seed=5, n_basis=3)
    res = put(40.0).price_american(h, ds, n_paths=30_000, seed=5, n_basis=3, precision="fp64")
    assert abs(res.price - ref.price) < 1e-6 * ref.price


@pytest.mark.parametrize("n_basis", [3, 4])
def test_lsm_laguerre_shared_draws_fp64_matches_oracle(orc, n_basis):
    """Weighted-Laguerre basis on shared FP64 normals: the device and the
    oracle compute the same regression (up to the order of the Gram sums and
    the last bit of exp), so every path's value agrees to 1e-9 relative except
    a decision within 1e-9 of the exercise boundary."""
    rng = np.random.default_rng(10 + n_basis)
    n, nd = 4000, 25
    z = rng.standard_normal((n, nd))
    kx.set_shared_draws(z)
    orc.set_shared_draws(z)
    m = kx.GBM(s0=40.0, sigma=0.2, r=0.06, asset="X")
    c = put(40.0)
    ds = dates(1.0, nd)
    res, pv = c.price_american(m, ds, n_paths=n, seed=0, n_basis=n_basis, precision="fp64", shared_draws=True,
                               basis="laguerre", per_path=True)
    ref, rpv, _, margin = orc.price_american_detail(c.to_json(), m, ds, n_paths=n, seed=0, n_basis=n_basis,
                                                    shared=True, basis="laguerre")
    diff = np.abs(pv - rpv)
    bad = diff > 1e-9 * np.maximum(np.abs(rpv), 1.0)
    assert np.all(margin[bad] < 1e-9), float(margin[bad].max())
    assert abs(res.price - ref.price) <= float(diff.sum()) / n + 1e-9 * abs(ref.price)


@pytest.mark.parametrize("s0,sigma,t", [(36.0, 0.2, 1.0), (44.0, 0.4, 2.0)])
def test_american_put_laguerre_vs_crr(orc, s0, sigma, t):
    """The LSM benchmark shape with the weighted-Laguerre basis: 4 functions,
    50 dates a year, 1M paths stored in FP32."""
    m = kx.GBM(s0=s0, sigma=sigma, r=0.06, asset="X")
    res = put(40.0).price_american(m, dates(t, int(50 * t)), n_paths=1_000_000, seed=42, n_basis=4,
                                   basis="laguerre")
    crr = orc.crr_american(s0, 40.0, t, 0.06, sigma, 1000, False)
    assert abs(res.price - crr) < 0.01 * crr + 4 * res.std_error, (res.price, crr)


@pytest.mark.parametrize("precision,basis", [("fp32", "monomial"), ("fp32", "laguerre"), ("fp64", "laguerre")])
def test_lsm_batch_equals_single_calls(precision, basis):
    """One batched call over cases with different date counts, paths, seeds and
    models returns each case's single-call result bit for bit."""
    h = kx.heston(spot=100.0, v0=0.04, kappa=1.5, theta=0.04, sigma_v=0.3, rho=-0.6, r=0.03, asset="X")
    cases = [
        (put(40.0), kx.GBM(s0=36.0, sigma=0.2, r=0.06, asset="X"), dates(1.0, 50), 65_536, 1),
        (put(40.0), kx.GBM(s0=44.0, sigma=0.4, r=0.06, asset="X"), dates(2.0, 100), 40_000, 2),
        (put(100.0), h, dates(0.5, 12), 30_001, 3),
        (put(40.0), kx.GBM(s0=40.0, sigma=0.3, r=0.06, asset="X"), dates(1.0, 1), 17, 4),
    ]
    got = kx.price_american_batch(cases, n_basis=3, precision=precision, basis=basis)
    for (c, m, ds, n, seed), g in zip(cases, got):
        one = c.price_american(m, ds, n_paths=n, seed=seed, n_basis=3, precision=precision, basis=basis)
        assert (g.price, g.std_error, g.n_paths) == (one.price, one.std_error, one.n_paths)


def test_lsm_batch_rejects_a_bad_case():
    m = kx.GBM(s0=36.0, sigma=0.2, r=0.06, asset="X")
    c = put(40.0)
    with pytest.raises(kx.KontractError):
        kx.price_american_batch([(c, m, dates(1.0, 4), 100, 1)], n_basis=1)
    with pytest.raises(kx.KontractError):
        kx.price_american_batch([(c, m, dates(1.0, 4), 100, 1)] * 1025)
    assert kx.price_american_batch([]) == []


def test_lsm_wait_that_runs_out_is_a_device_timeout_and_the_next_call_is_exact(monkeypatch):
    """Failure detection without a fault: every wait of the cooperative
    backward launch (a tile block for its case's previous regression, a
    coordinator for a case's tiles) gives up after a bounded number of polls
    and sets an error word that the others see. With the limit forced to zero
    polls (KX_LSM_SPIN_LIMIT) the first wait that finds its flag unset gives
    up, the launch ends, the call fails with KX_DEVICE_TIMEOUT, and the
    context stays usable: the next call returns the exact price."""
    m = kx.GBM(s0=36.0, sigma=0.2, r=0.06, asset="X")
    ds = dates(1.0, 50)
    good = put(40.0).price_american(m, ds, n_paths=200_000, seed=3, n_basis=4)
    monkeypatch.setenv("KX_LSM_SPIN_LIMIT", "0")
    for prec in ("fp32", "fp64"):
        with pytest.raises(kx.KontractError) as e:
            put(40.0).price_american(m, ds, n_paths=200_000, seed=3, n_basis=4, precision=prec)
        assert e.value.status == "DeviceTimeout"
    monkeypatch.delenv("KX_LSM_SPIN_LIMIT")
    again = put(40.0).price_american(m, ds, n_paths=200_000, seed=3, n_basis=4)
    assert (again.price, again.std_error) == (good.price, good.std_error)
