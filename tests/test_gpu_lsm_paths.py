"""Longstaff-Schwartz path by path at the benchmark shape: American puts on
GBM, s0 36 and 44, K 40, 50 exercise dates a year (50 and 100 dates), the
reference's monomial basis with n_basis = 4, on shared draws (the same
normals in the engine and in the oracle's restatement of lsm.rs:80-229).

Each path's realised value (the payoff at its exercise date, discounted to
t = 0, lsm.rs:226) is compared, and through it the exercise decision. FP64
values agree to 1e-12 (relative to max(|pv|, 1)) wherever the two take the
same decisions. A decision can differ only where the exercise value and the
fitted continuation are nearly equal: the Gram sums are added in another
order (tiles of paths on the device, one serial loop in the reference),
which moves the fitted continuation by about 1e-9, so a handful of paths
whose margin (the oracle's |exercise - continuation|, smallest over the
path's decisions) is that small decide the other way. Each such path's
realised value then differs by O(1), which moves the regressions of the
earlier dates by O(1 / n); with 1,000,000 paths that flips further paths
whose margin is below about 1e-3 (25 ppm of the strike), a few hundred in
measured runs. The test bounds that cascade; below it, with 200,000 paths,
only first-order flips (margin < 1e-6) remain.

FP32 (paths stored and regressed in FP32, sums and solve in float-float)
rounds the continuation at about 1e-5 of its value, so decisions within
that margin flip and cascade further; FP32 LSM is checked at the price
level against the FP64 oracle on the same draws, and its flipped decisions
are counted."""
import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

K = 40.0
CASES = [(36.0, 0.2, 1.0), (44.0, 0.4, 2.0)]


def _put():
    return kx.scale((kx.const_(K) - kx.S("X")).clip(0.0), kx.one())


def _run(orc, s0, sigma, t, n, precision, seed):
    nd = int(50 * t)
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, nd))
    if precision == "fp32":
        z = z.astype(np.float32)
    kx.set_shared_draws(z)
    orc.set_shared_draws(z.astype(np.float64))
    del z
    m = kx.GBM(s0=s0, sigma=sigma, r=0.06, asset="X")
    ds = [t * i / nd for i in range(1, nd + 1)]
    c = _put()
    res, pv = c.price_american(m, ds, n_paths=n, seed=0, n_basis=4, precision=precision, shared_draws=True,
                               per_path=True)
    ref, rpv, ex, margin = orc.price_american_detail(c.to_json(), m, ds, n_paths=n, seed=0, n_basis=4, shared=True)
    return res, np.asarray(pv), ref, rpv, ex, margin


@pytest.mark.parametrize("s0,sigma,t", CASES)
def test_lsm_fp64_per_path_at_benchmark_shape(orc, s0, sigma, t):
    n = 1_000_000
    res, pv, ref, rpv, _, margin = _run(orc, s0, sigma, t, n, "fp64", seed=int(s0 * 100 + t))
    diff = np.abs(pv - rpv)
    bad = diff > 1e-12 * np.maximum(np.abs(rpv), 1.0)
    # every differing path is a decision within 1e-3 of indifference, and they are few
    assert np.all(margin[bad] < 1e-3), (int(bad.sum()), float(margin[bad].max()))
    assert bad.sum() <= n // 1000, int(bad.sum())
    # the price is the mean of those values: it differs by no more than they do
    assert abs(res.price - float(np.mean(pv))) <= 1e-12 * ref.price
    assert abs(res.price - ref.price) <= float(diff.sum()) / n + 1e-12 * ref.price, (res.price, ref.price)


@pytest.mark.parametrize("s0,sigma,t", CASES)
def test_lsm_fp64_per_path_first_order_flips_only(orc, s0, sigma, t):
    n = 200_000
    res, pv, ref, rpv, _, margin = _run(orc, s0, sigma, t, n, "fp64", seed=5)
    diff = np.abs(pv - rpv)
    bad = diff > 1e-12 * np.maximum(np.abs(rpv), 1.0)
    assert bad.sum() <= 5 and np.all(margin[bad] < 1e-6), (int(bad.sum()), margin[bad])
    assert abs(res.price - ref.price) <= float(diff.sum()) / n + 1e-12 * ref.price


@pytest.mark.parametrize("s0,sigma,t", CASES)
def test_lsm_fp32_at_benchmark_shape(orc, s0, sigma, t):
    """FP32 paths against the FP64 oracle on the same 1,000,000 paths: the
    price moves by a small fraction of a standard error; the paths whose value
    differs by more than FP32 rounding (1e-5 relative plus 2^-20 of the spot)
    are a small share, and nearly all of them are decisions within 0.05 of
    indifference (the few beyond are the cascade of earlier flips into the
    regressions of earlier dates, as in FP64 but from a larger first step)."""
    n = 1_000_000
    res, pv, ref, rpv, ex, margin = _run(orc, s0, sigma, t, n, "fp32", seed=int(s0 * 100 + t))
    nd = int(50 * t)
    disc = np.exp(-0.06 * t * np.arange(1, nd + 1) / nd)
    d_ex = np.where(ex >= 0, disc[np.maximum(ex, 0)], 0.0)
    s_ex = np.where(ex >= 0, K - rpv / np.where(ex >= 0, d_ex, 1.0), 0.0)
    tol = 1e-5 * np.abs(rpv) + 2.0 ** -20 * s_ex * d_ex + 1e-9
    flip = np.abs(pv - rpv) > tol
    assert flip.mean() <= 0.05, float(flip.mean())
    assert np.quantile(margin[flip], 0.99) < 5e-2, np.quantile(margin[flip], [0.5, 0.99, 1.0])
    assert abs(res.price - ref.price) <= 0.25 * ref.std_error, (res.price, ref.price, ref.std_error)
