"""The statistics of one chunk of per-path values as the device reduction
computes them (kx_chunk_moments, the host mirror of chunk_moments_exact: the
same bits for finite values), against the exact mean and sum of squared
deviations in rational arithmetic. The summary statistics follow
pricer.rs:303-328 (mean, then the squared deviations from it)."""
import ctypes as C
import math
from fractions import Fraction

import numpy as np
import pytest

from kontracts_gb300 import _abi

CHUNK = 16384


@pytest.fixture(scope="module")
def lib():
    return _abi.load()


def _moments(lib, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    pa = a.ctypes.data_as(C.POINTER(C.c_double))
    pb = None
    if b is not None:
        b = np.ascontiguousarray(b, dtype=np.float64)
        pb = b.ctypes.data_as(C.POINTER(C.c_double))
    out = _abi.KxChunkStats()
    assert lib.kx_chunk_moments(pa, pb, len(a), C.byref(out)) == 0
    return out.n, out.mean, out.m2


def _exact(vals):
    fr = [Fraction(float(x)) for x in vals]
    mean = sum(fr) / len(fr)
    return mean, sum((x - mean) ** 2 for x in fr)


def _unit(vals):
    """The fixed-point unit: 2^-2 of the last mantissa bit of the largest exponent."""
    e = max(max((int(np.frexp(np.float64(x))[1]) for x in vals if x != 0.0), default=-1074), -1021)
    return 2.0 ** (e - 53 - 2)


def _check(vals, mean, m2):
    em, e2 = _exact(vals)
    n = len(vals)
    u = _unit(vals)
    # mean: one or two roundings, plus at most one unit of truncation of small values
    tol_m = 3 * 2.0 ** -52 * abs(float(em)) + u + 1e-320
    assert abs(Fraction(mean) - em) <= Fraction(tol_m), (mean, float(em))
    # M2: two roundings, plus the truncation term 2 sqrt(n M2) u + n u^2
    tol_2 = 4 * 2.0 ** -52 * float(e2) + 2 * math.sqrt(n * float(e2)) * u + n * u * u + 1e-320
    assert abs(Fraction(m2) - e2) <= Fraction(tol_2), (m2, float(e2))


CASES = {
    "prices": lambda r: np.maximum(r.normal(15.0, 20.0, CHUNK), 0.0),
    "mixed_signs": lambda r: r.normal(0.0, 3.0, CHUNK),
    "lognormal": lambda r: r.lognormal(0.0, 2.0, CHUNK),
    "near_constant": lambda r: 100.0 + r.normal(0.0, 1e-9, CHUNK),
    "wide_range": lambda r: r.normal(0.0, 1.0, 4096) * 10.0 ** r.uniform(-30, 30, 4096),
    "tiny": lambda r: r.normal(0.0, 1e-300, 2048),
    "subnormal": lambda r: r.integers(-1000, 1000, 512).astype(np.float64) * 5e-324,
    "huge": lambda r: r.normal(1e150, 1e149, 1024),
    "sparse_digital": lambda r: np.where(r.random(CHUNK) < 0.01, 95.12294245007140, 0.0),
    "ragged_7": lambda r: r.normal(5.0, 1.0, 7),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_chunk_moments_are_exact_to_rounding(lib, name):
    vals = CASES[name](np.random.default_rng(7))
    n, mean, m2 = _moments(lib, vals)
    assert n == len(vals)
    _check(vals, mean, m2)


def test_constant_chunk_has_zero_spread(lib):
    for x in (0.0, 1.0, -3.25, 1e-310, 6.02e23):
        n, mean, m2 = _moments(lib, np.full(1000, x))
        assert (mean, m2) == (x, 0.0)


def test_single_value_and_empty_chunk(lib):
    assert _moments(lib, np.array([42.5])) == (1.0, 42.5, 0.0)
    out = _abi.KxChunkStats()
    assert lib.kx_chunk_moments(None, None, 0, C.byref(out)) == 0
    assert (out.n, out.mean, out.m2) == (0.0, 0.0, 0.0)


def test_difference_mode_takes_the_fp64_differences(lib):
    """values - subtrahend: each difference rounded to FP64 (the per-path
    multilevel difference P_fine - P_coarse the oracle forms), then the exact
    statistics of those differences."""
    r = np.random.default_rng(3)
    fine = r.normal(10.0, 4.0, CHUNK)
    coarse = fine + r.normal(0.0, 0.05, CHUNK)
    n, mean, m2 = _moments(lib, fine, coarse)
    assert (n, mean, m2) == _moments(lib, fine - coarse)
    _check(fine - coarse, mean, m2)


def test_result_does_not_depend_on_value_order(lib):
    """Integer sums: any order, the same bits (the device's blocks sum in any order)."""
    r = np.random.default_rng(11)
    vals = r.lognormal(1.0, 1.5, CHUNK) * np.where(r.random(CHUNK) < 0.3, -1.0, 1.0)
    first = vals[0]
    rest = vals[1:].copy()
    r.shuffle(rest)
    a = _moments(lib, vals)
    b = _moments(lib, np.concatenate([[first], rest]))
    assert a == b


def test_non_finite_values_give_ieee_results(lib):
    vals = np.array([1.0, 2.0, np.nan, 4.0])
    _, mean, m2 = _moments(lib, vals)
    assert math.isnan(mean) and math.isnan(m2)
    _, mean, m2 = _moments(lib, np.array([1.0, np.inf, 3.0]))
    assert mean == math.inf and math.isnan(m2)


def test_chunk_larger_than_the_chunk_size_is_rejected(lib):
    vals = np.zeros(CHUNK + 1)
    out = _abi.KxChunkStats()
    rc = lib.kx_chunk_moments(vals.ctypes.data_as(C.POINTER(C.c_double)), None, CHUNK + 1, C.byref(out))
    assert rc == _abi.KX_INVALID_ARGUMENT


def test_agrees_with_two_pass_fp64_on_prices(lib):
    vals = np.maximum(np.random.default_rng(5).normal(15.0, 20.0, CHUNK), 0.0)
    _, mean, m2 = _moments(lib, vals)
    m = vals.mean()
    assert abs(mean - m) <= 1e-14 * abs(m)
    assert abs(m2 - ((vals - m) ** 2).sum()) <= 1e-13 * m2


def test_merge_of_equal_infinite_means_stays_infinite(lib):
    """Chunks whose means are both +inf merge to +inf (the reference's one-pass
    mean of infinite values), with a NaN spread; equal finite means merge as
    the Chan update with d = 0."""
    from kontracts_gb300 import sharded
    r = sharded.merge([(16384.0, math.inf, math.nan), (16384.0, math.inf, math.nan)])
    assert r.price == math.inf and math.isnan(r.std_error)
    a = sharded.merge([(4.0, 2.5, 1.0), (4.0, 2.5, 3.0)])
    assert a.price == 2.5 and a.std_error == math.sqrt(4.0 / 7.0) / math.sqrt(8.0)
