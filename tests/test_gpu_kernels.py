"""The path kernels value every path identically: k_lean on compiled static
schedules (the default where a contract has one), k_lean with its general
event handler (KX_PATH_KERNEL=lean) and k_paths (KX_PATH_KERNEL=general), in
both precisions and both models, bit for bit."""
import os

import numpy as np
import pytest

import kontracts_gb300 as kx

pytestmark = pytest.mark.gpu

S = kx.S("X")

LEAN = {
    "euro_call": lambda: kx.european_call("X", 100.0, 1.0),
    "up_and_out": lambda: kx.up_and_out_call("X", 100.0, 130.0, 1.0),
    "up_and_out_strict": lambda: kx.until(S > 130.0, kx.european_call("X", 100.0, 1.0)),
    "down_and_out_put": lambda: kx.until(S < 80.0, kx.european_put("X", 100.0, 1.0)),
    "double_barrier": lambda: kx.until(S >= 125.0, kx.until(S <= 85.0, kx.european_call("X", 100.0, 1.0))),
    "knock_in": lambda: kx.anytime(S >= 120.0, kx.european_call("X", 100.0, 1.0)),
    "first_touch_pays": lambda: kx.one() @ (S <= 90.0),
    "digital": lambda: kx.cash_or_nothing_call("X", 100.0, 10.0, 1.0),
    "nested_when": lambda: kx.when(kx.at(0.5), kx.until(S <= 95.0, kx.scale(S, kx.one()) @ kx.at(1.0))),
    "bermudan_strip": lambda: kx.european_call("X", 100.0, 0.3) + kx.european_call("X", 105.0, 0.61)
    + kx.give(kx.european_put("X", 95.0, 0.9)),
    "knock_at_zero": lambda: kx.until(S <= 200.0, kx.european_call("X", 100.0, 1.0)),
    "late_barrier": lambda: kx.when(kx.at(0.4), kx.until(S >= 115.0, kx.european_call("X", 100.0, 1.0))),
}


def _run(c, model, prec, kernel, n=4000, spy=52):
    old = os.environ.get("KX_PATH_KERNEL")
    if kernel == "auto":
        os.environ.pop("KX_PATH_KERNEL", None)
    else:
        os.environ["KX_PATH_KERNEL"] = kernel
    try:
        return c.price(model, n_paths=n, seed=19, steps_per_year=spy, precision=prec, per_path=True)
    finally:
        if old is None:
            os.environ.pop("KX_PATH_KERNEL", None)
        else:
            os.environ["KX_PATH_KERNEL"] = old


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", sorted(LEAN))
def test_lean_equals_general_gbm(name, prec):
    c = LEAN[name]()
    m = kx.GBM(s0=100.0, sigma=0.3, r=0.04, asset="X")
    r1, p1 = _run(c, m, prec, "general")
    r2, p2 = _run(c, m, prec, "lean")
    r3, p3 = _run(c, m, prec, "auto")
    assert np.array_equal(np.asarray(p1), np.asarray(p2)), name
    assert np.array_equal(np.asarray(p1), np.asarray(p3)), name
    assert r1.price == r2.price == r3.price and r1.std_error == r2.std_error == r3.std_error


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", ["up_and_out", "double_barrier", "knock_in", "bermudan_strip"])
def test_lean_equals_general_heston(name, prec):
    c = LEAN[name]()
    m = kx.heston(100.0, 0.04, 1.5, 0.04, 0.5, -0.7, 0.03, asset="X")
    _, p1 = _run(c, m, prec, "general", n=2000, spy=100)
    _, p2 = _run(c, m, prec, "lean", n=2000, spy=100)
    _, p3 = _run(c, m, prec, "auto", n=2000, spy=100)
    assert np.array_equal(np.asarray(p1), np.asarray(p2)), name
    assert np.array_equal(np.asarray(p1), np.asarray(p3)), name


def test_lean_daily_grid_long_paths():
    """The benchmark's shape (daily grid, barrier far from spot) at a size
    where lanes hold paths of very different lengths."""
    c = kx.up_and_out_call("X", 100.0, 200.0, 1.0)
    m = kx.GBM(s0=180.0, sigma=0.25, r=0.05, asset="X")
    _, p1 = _run(c, m, "fp32", "general", n=100_000, spy=365)
    _, p2 = _run(c, m, "fp32", "lean", n=100_000, spy=365)
    _, p3 = _run(c, m, "fp32", "auto", n=100_000, spy=365)
    assert np.array_equal(np.asarray(p1), np.asarray(p2))
    assert np.array_equal(np.asarray(p1), np.asarray(p3))


AVERAGES = {
    "asian": lambda: kx.scale((kx.average(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "asian_window": lambda: kx.scale((kx.average_over(S, 0.25, 0.75) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "asian_put_early": lambda: kx.scale((100.0 - kx.average(S)).clip(0.0), kx.one()) @ kx.at(0.6),
    "knock_out_asian": lambda: kx.until(S >= 135.0, kx.scale((kx.average(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)),
    "asian_plus_call": lambda: kx.scale((kx.average(S) - 95.0).clip(0.0), kx.one()) @ kx.at(1.0)
    + kx.european_call("X", 110.0, 0.5),
    "lookback_call": lambda: kx.scale((kx.running_max(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
    "lookback_put": lambda: kx.scale((105.0 - kx.running_min(S)).clip(0.0), kx.one()) @ kx.at(0.8),
    "knock_out_lookback": lambda: kx.until(S <= 70.0, kx.scale((kx.running_max(S) - 100.0).clip(0.0), kx.one())
                                           @ kx.at(1.0)),
}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", sorted(AVERAGES))
def test_lean_average_equals_general(name, prec):
    """An average, running max or running min of the spot on a static
    schedule: k_lean keeps the accumulator in registers (an average's sum
    compensated in FP32, as k_paths sums it) and values every path as
    k_paths does, bit for bit, in both models."""
    c = AVERAGES[name]()
    for m, n, spy in ((kx.GBM(s0=100.0, sigma=0.3, r=0.04, asset="X"), 4000, 52),
                      (kx.heston(100.0, 0.04, 1.5, 0.04, 0.5, -0.7, 0.03, asset="X"), 2000, 100)):
        r1, p1 = _run(c, m, prec, "general", n=n, spy=spy)
        r3, p3 = _run(c, m, prec, "auto", n=n, spy=spy)
        assert kx.last_launch_stats()["path_kernel"] == 4, name
        assert np.array_equal(np.asarray(p1), np.asarray(p3)), name
        assert r1.price == r3.price and r1.std_error == r3.std_error


def test_lean_average_daily_grid():
    """An Asian call on a daily grid at a size where lanes hold paths of very
    different ages (the book's Asian shape)."""
    c = AVERAGES["asian"]()
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X")
    _, p1 = _run(c, m, "fp32", "general", n=100_000, spy=252)
    _, p3 = _run(c, m, "fp32", "auto", n=100_000, spy=252)
    assert np.array_equal(np.asarray(p1), np.asarray(p3))


@pytest.mark.parametrize("name,kernel", [("up_and_out", 3), ("double_barrier", 3), ("bermudan_strip", 3),
                                         ("nested_when", 3), ("late_barrier", 3), ("digital", 2),
                                         ("knock_in", 2), ("first_touch_pays", 2)])
def test_kernel_family_selection(name, kernel):
    """Static schedules serve contracts whose whens read only the time;
    price-triggered whens (knock-in, first touch) keep the general handler."""
    m = kx.GBM(s0=100.0, sigma=0.3, r=0.04, asset="X")
    _run(LEAN[name](), m, "fp32", "auto", n=1000)
    assert kx.last_launch_stats()["path_kernel"] == kernel


def test_calibration_loops_are_positive_and_ordered():
    """kx_measure_peak: the pipe microbenchmarks and the bare GBM and Heston
    step loops return positive rates; a Heston step (two normals, a square
    root) is slower than a GBM step."""
    import ctypes as C
    from kontracts_gb300 import _abi
    lib = _abi.load()
    got = {}
    for what in range(5):
        v = C.c_double()
        assert lib.kx_measure_peak(what, C.byref(v)) == 0
        got[what] = v.value
        assert v.value > 1e9
    assert got[4] < got[3]
