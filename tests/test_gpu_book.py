"""Books: the pricing step of a portfolio captured once in a CUDA graph and
replayed. Every contract's price must equal Contract.price's exactly (same
paths, same kernels, same chunked reduction), replay after replay, with and
without launch tuning, and after new model parameters are set."""
import json
import os

import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

S = kx.S("S")
BOOK = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "portfolio_256.json")))


def _mixed():
    cs = [kx.european_call("S", 100.0, 1.0), kx.up_and_out_call("S", 100.0, 130.0, 1.0),
          kx.scale((kx.average(S) - 100.0).clip(0.0), kx.one()) @ kx.at(0.75),
          kx.until(S <= 80.0, kx.european_put("S", 105.0, 0.5)),
          kx.anytime(S >= 120.0, kx.european_call("S", 100.0, 1.5)),
          kx.scale((kx.running_max(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)]
    ms = [kx.GBM(s0=100.0, sigma=0.15 + 0.05 * i, r=0.03, asset="S") for i in range(len(cs))]
    ns = [20_000, 50_000, 30_000, 7_000, 64_000, 10_000]
    seeds = [11, 12, 13, 14, 15, 16]
    return cs, ms, ns, seeds


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("tune", [False, True])
def test_book_equals_individual_prices(prec, tune):
    cs, ms, ns, seeds = _mixed()
    book = kx.Book(cs, ms, ns, seeds, steps_per_year=252, precision=prec, tune=tune)
    info = book.info()
    # static, static with an accumulator (the Asian and the lookback), lean (knock-in)
    assert info["n_contracts"] == len(cs) and info["n_groups"] == 3
    for rep in range(2):
        res = book.price()
        for c, m, n, s, r in zip(cs, ms, ns, seeds, res):
            single = c.price(m, n_paths=n, seed=s, steps_per_year=252, precision=prec)
            assert r.price == single.price and r.std_error == single.std_error, (rep, r.price, single.price)
            assert r.n_paths == n
    book.close()


def test_book_heston_and_gbm_groups():
    h = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="S")
    g = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    cs = [kx.european_call("S", 100.0, 1.0), kx.up_and_out_call("S", 100.0, 140.0, 1.0),
          kx.european_put("S", 95.0, 0.5)]
    ms = [h, h, g]
    book = kx.Book(cs, ms, [30_000, 20_000, 10_000], [1, 2, 3], steps_per_year=252)
    res = book.price()
    for c, m, n, s, r in zip(cs, ms, [30_000, 20_000, 10_000], [1, 2, 3], res):
        assert r.price == c.price(m, n_paths=n, seed=s, steps_per_year=252).price


def test_book_set_models_prices_the_new_market():
    cs, ms, ns, seeds = _mixed()
    book = kx.Book(cs, ms, ns, seeds, steps_per_year=252)
    base = book.price()
    ms2 = [kx.GBM(s0=101.0, sigma=m.sigma * 1.1, r=0.03, asset="S") for m in ms]
    book.set_models(ms2)
    res = book.price()
    for c, m, n, s, r, b in zip(cs, ms2, ns, seeds, res, base):
        assert r.price == c.price(m, n_paths=n, seed=s, steps_per_year=252).price
    assert any(r.price != b.price for r, b in zip(res, base))
    book.set_models(ms)  # and back: the same paths again
    assert [r.price for r in book.price()] == [r.price for r in base]


def test_book_of_the_256_contract_fixture():
    sub = BOOK["contracts"]
    cs = [kx.Contract.from_json(c["json"]) for c in sub]
    ms = [kx.GBM(s0=c["s0"], sigma=c["sigma"], r=c["r"], asset="S") for c in sub]
    ns = [max(1000, c["n_paths"] // 64) for c in sub]
    seeds = [c["seed"] for c in sub]
    book = kx.Book(cs, ms, ns, seeds, steps_per_year=252)
    res = book.price()
    for i in range(0, len(cs), 37):
        assert res[i].price == cs[i].price(ms[i], n_paths=ns[i], seed=seeds[i], steps_per_year=252).price


def test_book_rejects_shared_draws_and_empty_books():
    import ctypes as C
    from kontracts_gb300 import _abi
    c = kx.european_call("S", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    h = c._handle()
    hs = (C.c_void_p * 1)(h.h.value)
    ms = (_abi.KxModel * 1)(m._c())
    cfg = (_abi.KxMcConfig * 1)(kx._cfg(1000, 1, 52, 0.05, "fp32", True))
    out = C.c_void_p()
    assert kx._lib().kx_book_create(1, hs, ms, cfg, 0, C.byref(out)) == _abi.KX_UNSUPPORTED
    assert not out.value
    assert kx._lib().kx_book_create(0, hs, ms, cfg, 0, C.byref(out)) == _abi.KX_INVALID_ARGUMENT
