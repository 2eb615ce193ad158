"""Longstaff-Schwartz path by path at the benchmark shape: American puts on
GBM, 1,000,000 paths, 50 exercise dates a year (50 and 100 dates), the
reference's monomial basis with n_basis = 4, on shared draws (the same
normals in the engine and in the oracle's restatement of lsm.rs:80-229).

Each path's realised value (the payoff at its exercise date, discounted to
t = 0, lsm.rs:226) is compared, and through it the exercise decision. A
decision can differ only where the exercise value and the fitted
continuation agree to within the difference of the two fits: the Gram sums
are added in another order (tiles of paths on the device, one serial loop in
the reference), which moves the fitted continuation by a few ulps of its
value. The oracle reports each path's decision margin (the smallest
|exercise - continuation| over its regression decisions); a path may differ
only if its margin is below that bound, stated per precision below."""
import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

N_PATHS = 1_000_000
K = 40.0
# FP64: values within 1e-12 relative; a decision may flip only on paths whose
# margin is below 1e-9 (about 1e-11 of the strike's order of magnitude times
# the fits' conditioning). FP32 (paths stored and regressed in FP32, the
# regression sums and solve in float-float): values within 1e-5 relative
# plus the FP32 spot's rounding (2^-20 of S: payoff K - S moves by that
# much when S does), flips only where the margin is below 1e-4 (a few FP32
# ulps of the continuation, which is evaluated in FP32 on x = S / s0).
TOL = {"fp64": (1e-12, 0.0, 1e-9), "fp32": (1e-5, 2.0 ** -20, 1e-4)}


def _put():
    return kx.scale((kx.const_(K) - kx.S("X")).clip(0.0), kx.one())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("s0,sigma,t", [(36.0, 0.2, 1.0), (44.0, 0.4, 2.0)])
def test_lsm_per_path_matches_oracle_at_benchmark_shape(orc, precision, s0, sigma, t):
    nd = int(50 * t)
    rng = np.random.default_rng(int(s0 * 100 + sigma * 10 + t))
    z = rng.standard_normal((N_PATHS, nd))
    if precision == "fp32":
        z = z.astype(np.float32)
    kx.set_shared_draws(z)
    orc.set_shared_draws(z.astype(np.float64))
    del z
    m = kx.GBM(s0=s0, sigma=sigma, r=0.06, asset="X")
    ds = [t * i / nd for i in range(1, nd + 1)]
    c = _put()
    res, pv = c.price_american(m, ds, n_paths=N_PATHS, seed=0, n_basis=4, precision=precision, shared_draws=True,
                               per_path=True)
    ref, rpv, ex, margin = orc.price_american_detail(c.to_json(), m, ds, n_paths=N_PATHS, seed=0, n_basis=4,
                                                     shared=True)
    rel, spot_ulp, flip_margin = TOL[precision]
    # the spot at each path's exercise date (the oracle's), for the FP32 rounding term
    disc = np.exp(-0.06 * np.asarray(ds))
    s_ex = np.where(ex >= 0, K - rpv / np.where(ex >= 0, disc[np.maximum(ex, 0)], 1.0), 0.0)
    tol = rel * np.abs(rpv) + spot_ulp * np.abs(s_ex) * np.where(ex >= 0, disc[np.maximum(ex, 0)], 0.0) + 1e-300
    diff = np.abs(pv - rpv)
    bad = diff > tol
    n_bad = int(bad.sum())
    # every differing path is a decision within the stated margin of the boundary
    assert np.all(margin[bad] < flip_margin), (n_bad, float(margin[bad].max()))
    assert n_bad <= N_PATHS // 1000, n_bad
    # the exercise decisions: the engine's value is the payoff at the oracle's date on every other path
    agree = ~bad
    assert agree.sum() >= N_PATHS - N_PATHS // 1000
    # the price is the mean of those values, so it differs from the oracle's by
    # no more than the per-path differences do (no allowance beyond them)
    assert abs(res.price - float(np.mean(pv))) <= 1e-12 * ref.price
    assert abs(res.price - ref.price) <= float(diff.sum()) / N_PATHS + 1e-12 * ref.price, (res.price, ref.price)
