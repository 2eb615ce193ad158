"""Chunk statistics of non-finite per-path values: a chunk holding a NaN or an
infinity takes the FP64 passes (block 0 of the chunk's cluster) and gives the
IEEE result, as the reference's summarize does on such values
(pricer.rs:303-328: plain f64 sums); prices, two-point and three-point Greek
estimators (the three reduction kernels) alike, and the next call of the
process is unaffected."""
import math

import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import sharded

pytestmark = pytest.mark.gpu

CH = sharded.CHUNK


def _model():
    return kx.GBM(s0=100.0, sigma=0.3, r=0.03, asset="X")


def test_nan_paths_give_a_nan_price_and_greeks():
    S = kx.S("X")
    itm = (S - 100.0).clip(0.0)
    c = kx.scale(itm / itm, kx.one()) @ kx.at(1.0)  # 1 in the money, 0/0 out of it
    r = c.price(_model(), n_paths=3 * CH + 5, seed=3, steps_per_year=12, precision="fp64")
    assert math.isnan(r.price) and math.isnan(r.std_error)
    g = c.greeks(_model(), n_paths=3 * CH + 5, seed=3, steps_per_year=12, precision="fp64")
    assert all(math.isnan(getattr(g, k)) for k in ("price", "delta", "gamma", "vega", "rho"))


def test_infinite_paths_give_an_infinite_price():
    S = kx.S("X")
    c = kx.scale(kx.const_(1.0) / (S - S), kx.one()) @ kx.at(1.0)  # 1 / 0 on every path
    r = c.price(_model(), n_paths=2 * CH, seed=3, steps_per_year=12, precision="fp32")
    assert r.price == math.inf and math.isnan(r.std_error)


def test_finite_price_after_non_finite_chunks_is_unchanged():
    c = kx.up_and_out_call("X", 100.0, 130.0, 1.0)
    before = c.price(_model(), n_paths=2 * CH + 9, seed=8, steps_per_year=52, precision="fp64")
    S = kx.S("X")
    itm = (S - 100.0).clip(0.0)
    nan_price = (kx.scale(itm / itm, kx.one()) @ kx.at(1.0)).price(_model(), n_paths=CH, seed=1, steps_per_year=12)
    assert math.isnan(nan_price.price)
    after = c.price(_model(), n_paths=2 * CH + 9, seed=8, steps_per_year=52, precision="fp64")
    assert (after.price, after.std_error) == (before.price, before.std_error)
