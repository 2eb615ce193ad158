"""kx_price_batch_sens: a book of Europeans on one shared simulation with
every contract's pathwise sensitivities from one forward (tangent) pass. The
derivatives are those of the checkpointed reverse sweep (kx_greeks_adjoint)
on the same paths, term for term; each contract's values in a book are its
values alone (the merged grid's points are the contract's own); the Heston
ones match CRN central differences of the shared-simulation prices
(price_batch_gbm, pricer.rs:250-294; greeks.rs:60-98 bumps); other contracts
are refused."""
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

HP = dict(s0=100.0, v0=0.04, kappa=2.0, theta=0.04, sigma_v=0.3, rho=-0.5, r=0.05)
FIELDS_HESTON = ("d_s0", "d_r", "d_v0", "d_kappa", "d_theta", "d_sigma_v", "d_rho")
FIELDS_GBM = ("d_s0", "d_r", "d_sigma")


def _heston(scheme="full_truncation", **kw):
    p = dict(HP, **kw)
    return kx.heston(p["s0"], p["v0"], p["kappa"], p["theta"], p["sigma_v"], p["rho"], p["r"], asset="X",
                     scheme=scheme)


def _book():
    S = kx.S("X")
    return [kx.european_call("X", 95.0, 0.5), kx.european_put("X", 105.0, 1.0), kx.european_call("X", 110.0, 2.0),
            kx.scale((S - 100.0).clip(0.0), kx.one()) @ kx.at(1.0), kx.scale(kx.const_(3.0), kx.one()) @ kx.at(2.0),
            kx.european_put("X", 90.0, 0.5), kx.one() @ kx.at(2.0)]


# FP32: the two kernels round the FP32 paths differently, so a path within
# rounding of a strike can fall on either side (each such path moves d_s0 by
# about S / n): FP32 noise of the paths, not of the derivative.
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-3)])
@pytest.mark.parametrize("model", ["gbm", "heston_ft", "heston_ref"])
def test_equals_the_adjoint_on_the_same_paths(model, prec, tol):
    m = {"gbm": kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X"), "heston_ft": _heston("full_truncation"),
         "heston_ref": _heston("reference")}[model]
    fields = FIELDS_GBM if model == "gbm" else FIELDS_HESTON
    for c in (kx.european_call("X", 100.0, 1.0), kx.european_put("X", 95.0, 0.5)):
        res, sens = kx.price_batch([c], m, n_paths=30_000, seed=7, steps_per_year=52, precision=prec, greeks=True)
        a = c.adjoint(m, n_paths=30_000, seed=7, steps_per_year=52, precision=prec)
        plain = kx.price_batch([c], m, n_paths=30_000, seed=7, steps_per_year=52, precision=prec)[0]
        assert res[0].price == plain.price and sens[0].price == plain.price
        assert abs(sens[0].price - a.price) <= 1e-12 * abs(a.price) + (tol if prec == "fp32" else 0.0)
        for f in fields:
            got, ref = getattr(sens[0], f), getattr(a, f)
            se = getattr(a, "se" + f[1:])
            assert abs(got - ref) <= tol * max(abs(ref), 1.0) + (0.5 * se if prec == "fp32" else 0.0), (f, got, ref)


def test_book_contracts_have_their_solo_values():
    """Heston books run on the fine grid, whose points are every contract's
    own: each contract's values in the book are its values alone. (A GBM book
    of Europeans runs on the merged dates only, pricer.rs:260-279, so its
    contracts see other paths than alone: checked by CRN differences below.)"""
    m = _heston()
    fields = ("price", "price_se") + FIELDS_HESTON
    book = _book()
    res, sens = kx.price_batch(book, m, n_paths=20_000, seed=5, steps_per_year=252, precision="fp64", greeks=True)
    for c, s in zip(book, sens):
        _, solo = kx.price_batch([c], m, n_paths=20_000, seed=5, steps_per_year=252, precision="fp64", greeks=True)
        for f in fields:
            a, b = getattr(s, f), getattr(solo[0], f)
            assert abs(a - b) <= 1e-12 * max(abs(b), 1.0), (f, a, b)
    for i in (4, 6):  # constant amounts (a scaled constant, a bare one()): only the discount moves them
        assert sens[i].d_s0 == 0.0 and sens[i].d_v0 == 0.0 and sens[i].d_sigma == 0.0
        assert abs(sens[i].d_r - (-2.0 * sens[i].price)) <= 1e-12 * sens[i].price
    assert abs(sens[4].price - 3.0 * sens[6].price) <= 1e-12 * sens[4].price


def test_gbm_book_matches_crn_differences():
    """d/ds0, d/dsigma, d/dr of every contract of a GBM book against CRN
    central differences of the shared-simulation prices (bumps of 1e-7 of
    each parameter, FP64), within 1e-4 relative."""
    book = _book()
    base = dict(s0=100.0, sigma=0.25, r=0.03)
    gbm = lambda **kw: kx.GBM(asset="X", **dict(base, **kw))
    _, sens = kx.price_batch(book, gbm(), n_paths=40_000, seed=11, steps_per_year=52, precision="fp64", greeks=True)
    for name, field in (("s0", "d_s0"), ("sigma", "d_sigma"), ("r", "d_r")):
        h = 1e-7 * base[name]
        up = kx.price_batch(book, gbm(**{name: base[name] + h}), n_paths=40_000, seed=11, steps_per_year=52,
                            precision="fp64")
        dn = kx.price_batch(book, gbm(**{name: base[name] - h}), n_paths=40_000, seed=11, steps_per_year=52,
                            precision="fp64")
        for i, s in enumerate(sens):
            fd = (up[i].price - dn[i].price) / (2 * h)
            got = getattr(s, field)
            assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-3 * abs(s.price) + 1e-9), (i, name, got, fd)


@pytest.mark.parametrize("scheme", ["reference", "full_truncation"])
def test_heston_book_matches_crn_differences(scheme):
    """Every sensitivity of every contract against CRN central differences of
    the shared-simulation prices, bumps of 1e-7 of each parameter, within 1e-4
    relative (the parameters satisfy Feller's condition, as in the adjoint's
    own test)."""
    book = _book()
    n, spy = 40_000, 100
    _, sens = kx.price_batch(book, _heston(scheme), n_paths=n, seed=11, steps_per_year=spy, precision="fp64",
                             greeks=True)
    for name, field in (("s0", "d_s0"), ("v0", "d_v0"), ("kappa", "d_kappa"), ("theta", "d_theta"),
                        ("sigma_v", "d_sigma_v"), ("rho", "d_rho"), ("r", "d_r")):
        h = 1e-7 * max(abs(HP[name]), 1e-2)
        up = kx.price_batch(book, _heston(scheme, **{name: HP[name] + h}), n_paths=n, seed=11, steps_per_year=spy,
                            precision="fp64")
        dn = kx.price_batch(book, _heston(scheme, **{name: HP[name] - h}), n_paths=n, seed=11, steps_per_year=spy,
                            precision="fp64")
        for i, s in enumerate(sens):
            fd = (up[i].price - dn[i].price) / (2 * h)
            got = getattr(s, field)
            assert abs(got - fd) <= 1e-4 * max(abs(fd), 1e-3 * abs(s.price) + 1e-9), (i, name, got, fd)


def test_path_dependent_contracts_are_refused():
    c = kx.up_and_out_call("X", 100.0, 130.0, 1.0)
    with pytest.raises(kx.KontractError) as e:
        kx.price_batch([kx.european_call("X", 100.0, 1.0), c], _heston(), n_paths=1000, seed=1, greeks=True)
    assert e.value.status == "Unsupported"


def test_autograd_book_prices():
    """heston_book_price as a torch.autograd.Function: the forward values are
    the shared-simulation prices, backward contracts the incoming gradient
    with every contract's seven sensitivities."""
    torch = pytest.importorskip("torch")
    import numpy as np
    from kontracts_gb300.autograd import heston_book_price
    book = _book()
    vals = [HP[k] for k in ("s0", "v0", "kappa", "theta", "sigma_v", "rho", "r")]
    p = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    prices = heston_book_price(book, p, asset="X", n_paths=20_000, seed=5, steps_per_year=252, precision="fp64",
                               scheme="full_truncation")
    w = torch.arange(1, len(book) + 1, dtype=torch.float64)
    (w * prices).sum().backward()
    res, sens = kx.price_batch(book, _heston(), n_paths=20_000, seed=5, steps_per_year=252, precision="fp64",
                               greeks=True)
    assert prices.tolist() == [r.price for r in res]
    fields = ("d_s0", "d_v0", "d_kappa", "d_theta", "d_sigma_v", "d_rho", "d_r")
    want = sum((i + 1) * np.array([getattr(s, f) for f in fields]) for i, s in enumerate(sens))
    assert np.allclose(p.grad.numpy(), want, rtol=1e-12, atol=1e-12)
