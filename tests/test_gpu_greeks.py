"""GPU Greeks: bump-and-reprice (greeks.rs semantics) and the pathwise adjoint.

The adjoint differentiates the barrier-smoothed payoff; it is checked against
CRN central differences of that same smoothed payoff (bump kernel with the
same width) to 1e-4 relative in FP64, against Black-Scholes on a European
call (3 standard errors), and for Heston against CRN differences of the
pricing kernel (1e-4 relative, both variance schemes)."""
import math

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu


def test_bump_greeks_vs_black_scholes(orc):
    """tests/greeks.rs:65-122 on the engine: delta < 1%, vega < 2%, rho < 2%."""
    c = kx.european_call("AAPL", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="AAPL")
    g = c.greeks(m, n_paths=500_000, seed=2024, steps_per_year=1)
    bs = orc.bs_call_greeks(100, 100, 1, 0.05, 0.2)
    assert abs(g.delta - bs["delta"]) / bs["delta"] < 0.01
    assert abs(g.vega - bs["vega"]) / bs["vega"] < 0.02
    assert abs(g.rho - bs["rho"]) / bs["rho"] < 0.02
    assert g.gamma > 0


@pytest.mark.parametrize("barrier,k", [(200.0, 100.0), (150.0, 100.0)])
def test_adjoint_matches_crn_differences_of_smoothed_payoff(barrier, k):
    uo = kx.up_and_out_call("X", k, barrier, 1.0)
    s0, sig, r = (180.0 if barrier == 200.0 else 120.0), 0.25, 0.05
    m = kx.GBM(s0=s0, sigma=sig, r=r, asset="X")
    w = 0.5 * sig * math.sqrt(1 / 365)
    n = 100_000
    adj = uo.adjoint(m, n_paths=n, seed=9, steps_per_year=365, smoothing_width=w, precision="fp64")
    h = 1e-5
    b = uo.greeks(m, n_paths=n, seed=9, steps_per_year=365, bumps=(h, h, h), relative=True, smooth_width=w,
                  precision="fp64")
    assert abs(adj.price - b.price) <= 1e-10 * abs(b.price)
    for a_, b_ in ((adj.d_s0, b.delta), (adj.d_sigma, b.vega), (adj.d_r, b.rho)):
        assert abs(a_ - b_) <= 1e-4 * max(abs(b_), 1e-3), (a_, b_)
    assert abs(adj.smoothing_width - w) < 1e-15


def test_adjoint_european_call_vs_black_scholes(orc):
    c = kx.european_call("X", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="X")
    a = c.adjoint(m, n_paths=1_000_000, seed=5, steps_per_year=1)
    bs = orc.bs_call_greeks(100, 100, 1, 0.05, 0.2)
    assert abs(a.d_s0 - bs["delta"]) < 3 * a.se_s0 + 1e-3
    assert abs(a.d_sigma - bs["vega"]) < 3 * a.se_sigma + 0.05
    assert abs(a.d_r - bs["rho"]) < 3 * a.se_r + 0.05
    p = c.price(m, n_paths=1_000_000, seed=5, steps_per_year=1)
    assert abs(a.price - p.price) < 1e-6 * p.price  # same paths (FP32)


def test_adjoint_asian_and_lookback_vs_crn():
    m = kx.GBM(s0=100.0, sigma=0.3, r=0.03, asset="X")
    for c in (kx.scale((kx.average(kx.S("X")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
              kx.scale((kx.running_max(kx.S("X")) - 95.0).clip(0.0), kx.one()) @ kx.at(1.0)):
        a = c.adjoint(m, n_paths=50_000, seed=3, steps_per_year=52, precision="fp64")
        b = c.greeks(m, n_paths=50_000, seed=3, steps_per_year=52, bumps=(1e-6, 1e-6, 1e-6), relative=True,
                     precision="fp64")
        for a_, b_ in ((a.d_s0, b.delta), (a.d_sigma, b.vega), (a.d_r, b.rho)):
            assert abs(a_ - b_) <= 2e-4 * max(abs(b_), 1e-2), (c, a_, b_)


HP = dict(s0=100.0, v0=0.04, kappa=2.0, theta=0.04, sigma_v=0.3, rho=-0.5, r=0.05)


def _heston(**kw):
    p = dict(HP, **kw)
    return kx.heston(p["s0"], p["v0"], p["kappa"], p["theta"], p["sigma_v"], p["rho"], p["r"], asset="X")


def _heston_s(scheme, **kw):
    p = dict(HP, **kw)
    return kx.heston(p["s0"], p["v0"], p["kappa"], p["theta"], p["sigma_v"], p["rho"], p["r"], asset="X",
                     scheme=scheme)


@pytest.mark.parametrize("scheme", ["reference", "full_truncation"])
def test_heston_adjoint_vs_crn_differences(scheme):
    """All seven Heston sensitivities against CRN central differences of the
    same FP64 paths, within 1e-4 relative. The parameters satisfy Feller's
    condition (2 kappa theta = 0.16 > sigma_v^2 = 0.09) and the bumps are
    1e-7 of each parameter: the payoff kink max(S - K, 0) and the variance
    floor max(v, 0) are then straddled by a negligible share of paths, and
    the differences' rounding (about 1e-16 / 1e-7 of the price) stays far
    below the tolerance. Measured: every relative difference below 1e-6."""
    c = kx.european_call("X", 100.0, 1.0)
    n, spy = 40_000, 100
    a = c.adjoint(_heston_s(scheme), n_paths=n, seed=11, steps_per_year=spy, precision="fp64")
    base = c.price(_heston_s(scheme), n_paths=n, seed=11, steps_per_year=spy, precision="fp64")
    assert abs(a.price - base.price) < 1e-10 * base.price
    for name, field in (("s0", "d_s0"), ("v0", "d_v0"), ("kappa", "d_kappa"), ("theta", "d_theta"),
                        ("sigma_v", "d_sigma_v"), ("rho", "d_rho"), ("r", "d_r")):
        h = 1e-7 * max(abs(HP[name]), 1e-2)
        up = c.price(_heston_s(scheme, **{name: HP[name] + h}), n_paths=n, seed=11, steps_per_year=spy,
                     precision="fp64").price
        dn = c.price(_heston_s(scheme, **{name: HP[name] - h}), n_paths=n, seed=11, steps_per_year=spy,
                     precision="fp64").price
        fd = (up - dn) / (2 * h)
        got = getattr(a, field)
        assert abs(got - fd) <= 1e-4 * abs(fd), (name, got, fd)


def test_autograd_function_heston():
    """heston_price as a torch.autograd.Function: the forward value is the
    adjoint's price, backward returns the incoming gradient times the seven
    pathwise sensitivities (s0, v0, kappa, theta, sigma_v, rho, r)."""
    torch = pytest.importorskip("torch")
    from kontracts_gb300.autograd import heston_price
    c = kx.european_call("X", 100.0, 1.0)
    vals = [HP[k] for k in ("s0", "v0", "kappa", "theta", "sigma_v", "rho", "r")]
    p = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    price = heston_price(c, p, asset="X", n_paths=100_000, seed=4, steps_per_year=252, checkpoint_every=16)
    (3.0 * price).backward()
    a = c.adjoint(_heston(), n_paths=100_000, seed=4, steps_per_year=252, checkpoint_every=16)
    assert price.item() == a.price
    want = 3.0 * np.array([a.d_s0, a.d_v0, a.d_kappa, a.d_theta, a.d_sigma_v, a.d_rho, a.d_r])
    assert np.array_equal(p.grad.numpy(), want)
    # the gradient is the sensitivity of the price: a step along it raises the price
    step = 1e-4 * torch.tensor(want / np.abs(want).max())
    q = (p.detach() + step).requires_grad_(False)
    higher = heston_price(c, q, asset="X", n_paths=100_000, seed=4, steps_per_year=252, checkpoint_every=16)
    assert higher.item() > price.item()


def test_autograd_function_gbm():
    torch = pytest.importorskip("torch")
    from kontracts_gb300.autograd import gbm_price
    c = kx.european_call("X", 100.0, 1.0)
    p = torch.tensor([100.0, 0.2, 0.05], dtype=torch.float64, requires_grad=True)
    price = gbm_price(c, p, asset="X", n_paths=200_000, seed=1, steps_per_year=1)
    (2.0 * price).backward()
    a = c.adjoint(kx.GBM(100.0, 0.2, 0.05, asset="X"), n_paths=200_000, seed=1, steps_per_year=1)
    assert abs(price.item() - a.price) < 1e-12
    assert np.allclose(p.grad.numpy(), 2.0 * np.array([a.d_s0, a.d_sigma, a.d_r]))


def test_adjoint_rejects_unsupported_contracts():
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="X")
    bad = kx.when(kx.S("X") >= 110.0, kx.one() @ kx.at(1.0))  # price-dependent when
    with pytest.raises(kx.KontractError) as e:
        bad.adjoint(m, n_paths=1000)
    assert e.value.status == "Unsupported"


def test_portfolio_adjoint_every_greek_within_1e4_of_crn_bump():
    """The 256-contract book fixture (European, up-and-out and arithmetic-Asian
    calls), 20,000 paths per contract, FP64: each contract's pathwise delta
    and vega from the one portfolio adjoint launch against CRN central
    differences of the same smoothed payoff (bump kernel, the width the
    adjoint reports, bumps of 1e-6 relative). The largest relative difference
    over all 512 Greeks must stay below 1e-4."""
    import json
    import os
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "portfolio_256.json")))["contracts"]
    cs = [kx.Contract.from_json(f["json"]) for f in fx]
    ms = [kx.GBM(s0=f["s0"], sigma=f["sigma"], r=f["r"], asset="S") for f in fx]
    n = 20_000
    seeds = [int(f["seed"]) for f in fx]
    _, sens = kx.price_portfolio(cs, ms, [n] * len(cs), seeds, steps_per_year=252, precision="fp64", greeks=True)
    worst = 0.0
    for c, m, sd, a in zip(cs, ms, seeds, sens):
        b = c.greeks(m, n_paths=n, seed=sd, steps_per_year=252, bumps=(1e-6, 1e-6, 1e-6), relative=True,
                     smooth_width=a.smoothing_width, precision="fp64")
        for got, fd in ((a.d_s0, b.delta), (a.d_sigma, b.vega)):
            worst = max(worst, abs(got - fd) / max(abs(fd), 1e-8))
    assert worst <= 1e-4, worst


SMOOTH_CASES = [
    ("up_and_out", lambda: kx.up_and_out_call("X", 100.0, 200.0, 1.0), lambda: kx.GBM(180.0, 0.25, 0.05, asset="X")),
    ("down_and_out", lambda: kx.down_and_out_call("X", 100.0, 90.0, 1.0), lambda: kx.GBM(100.0, 0.3, 0.02, asset="X")),
    ("double_barrier", lambda: kx.until(kx.S("X") >= 130.0, kx.until(kx.S("X") <= 80.0, kx.european_call("X", 100.0, 1.0))),
     lambda: kx.GBM(100.0, 0.2, 0.03, asset="X")),
    ("late_barrier", lambda: kx.when(kx.at(0.25), kx.until(kx.S("X") >= 125.0, kx.european_put("X", 100.0, 1.0))),
     lambda: kx.GBM(100.0, 0.25, 0.01, asset="X")),
]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name,mk_c,mk_m", SMOOTH_CASES, ids=[c[0] for c in SMOOTH_CASES])
def test_smoothed_bump_on_lean_kernel_equals_general_kernel(monkeypatch, prec, name, mk_c, mk_m):
    """The bump of the smoothed payoff runs its seven reprices as plain jobs
    of the lean kernel's static family, the barriers weighed in registers
    (path_kernel 3); every estimator must equal, bit for bit, the general
    kernel's (KX_PATH_KERNEL=general: the survival weights of on_event)."""
    import math
    c, m = mk_c(), mk_m()
    kw = dict(n_paths=50_000, seed=3, steps_per_year=252, bumps=(1e-3, 1e-3, 1e-3), relative=True,
              smooth_width=0.5 * m.sigma * math.sqrt(1 / 252), precision=prec)
    lean = c.greeks(m, **kw)
    assert kx.last_launch_stats()["path_kernel"] == 3
    monkeypatch.setenv("KX_PATH_KERNEL", "general")
    gen = c.greeks(m, **kw)
    assert kx.last_launch_stats()["path_kernel"] == 1
    for f in ("price", "delta", "gamma", "vega", "rho", "price_se", "delta_se", "gamma_se", "vega_se", "rho_se"):
        assert getattr(lean, f) == getattr(gen, f), (f, getattr(lean, f), getattr(gen, f))


ACC_CASES = {
    "asian": lambda: kx.scale((kx.average(kx.S("X")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "lookback_max": lambda: kx.scale((kx.running_max(kx.S("X")) - 95.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "lookback_min_put": lambda: kx.scale((105.0 - kx.running_min(kx.S("X"))).clip(0.0), kx.one()) @ kx.at(1.0),
    "asian_up_and_out": lambda: kx.until(kx.S("X") >= 140.0,
                                         kx.scale((kx.average(kx.S("X")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)),
    "window_and_strip": lambda: (kx.scale((kx.average_over(kx.S("X"), 0.25, 0.75) - 100.0).clip(0.0), kx.one())
                                 @ kx.at(0.75))
    + (kx.scale((kx.running_max(kx.S("X")) - 110.0).clip(0.0), kx.one()) @ kx.at(1.0)),
}


ACC_CASES.update({
    "european": lambda: kx.european_call("X", 100.0, 1.0),
    "up_and_out": lambda: kx.up_and_out_call("X", 100.0, 140.0, 1.0),
    "double_barrier_put": lambda: kx.until(kx.S("X") >= 130.0,
                                           kx.until(kx.S("X") <= 80.0, kx.european_put("X", 100.0, 1.0))),
})


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", sorted(ACC_CASES))
def test_gbm_adjoint_kernels_equal_generic_kernel(monkeypatch, prec, name):
    """The GBM reverse-sweep kernels (the register-resident barrier kernel and
    the kernel that keeps accumulators in registers and its records in shared
    memory, tuned over checkpoint interval and register budget) perform the
    generic kernel's operations in the same order, so every output equals the
    generic kernel's (KX_ADJOINT_KERNEL=general) bit for bit, for each of
    them. (The forward-mode kernel the tuner may also keep is checked against
    the generic kernel to rounding below.)"""
    c, m = ACC_CASES[name](), kx.GBM(s0=100.0, sigma=0.3, r=0.03, asset="X")
    kw = dict(n_paths=20_000, seed=9, steps_per_year=252, precision=prec)
    outs = []
    for q in range(10):  # every candidate (KX_ADJOINT_CANDIDATE is taken modulo their number)
        monkeypatch.setenv("KX_ADJOINT_CANDIDATE", str(q))
        outs.append(c.adjoint(m, **kw))
    monkeypatch.delenv("KX_ADJOINT_CANDIDATE")
    monkeypatch.setenv("KX_ADJOINT_KERNEL", "general")
    g = c.adjoint(m, **kw)
    for q, a in enumerate(outs):
        for f in ("price", "d_s0", "d_sigma", "d_r", "se_s0", "se_sigma", "se_r"):
            assert getattr(a, f) == getattr(g, f), (name, q, f, getattr(a, f), getattr(g, f))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 2e-4)])
@pytest.mark.parametrize("name", sorted(ACC_CASES))
def test_gbm_tangent_kernel_equals_the_reverse_sweep(monkeypatch, prec, tol, name):
    """The forward-mode GBM kernel (KX_ADJOINT_KERNEL=tangent: one pass
    carrying dy/dsigma, dy/dr, the barriers' d log w and the accumulators'
    derivatives) computes the same pathwise derivative as the reverse sweep:
    the price bit for bit (the same primal operations), the sensitivities and
    their standard errors to rounding (1e-9 relative in FP64; FP32: 2e-4 and a
    fiftieth of a standard error)."""
    c, m = ACC_CASES[name](), kx.GBM(s0=100.0, sigma=0.3, r=0.03, asset="X")
    kw = dict(n_paths=20_000, seed=9, steps_per_year=252, precision=prec)
    monkeypatch.setenv("KX_ADJOINT_KERNEL", "general")
    g = c.adjoint(m, **kw)
    monkeypatch.setenv("KX_ADJOINT_KERNEL", "tangent")
    t = c.adjoint(m, **kw)
    assert (t.price, t.price_se) == (g.price, g.price_se)
    for f in ("d_s0", "d_sigma", "d_r"):
        a, b = getattr(t, f), getattr(g, f)
        se = getattr(g, "se" + f[1:])
        assert abs(a - b) <= tol * max(abs(b), 1.0) + (0.02 * se if prec == "fp32" else 0.0), (name, f, a, b)
        assert abs(getattr(t, "se" + f[1:]) - se) <= 10 * tol * max(se, 1e-6), (name, f)
