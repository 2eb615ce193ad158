"""Path ranges on the GPU: the chunk statistics of consecutive chunk-aligned
ranges of one stream, merged in path order, are kx_price's result for the
whole range, bit for bit (the ranks of a sharded price each compute one
range)."""
import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import _abi, sharded

pytestmark = pytest.mark.gpu

C = sharded.CHUNK


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", ["up_and_out", "asian", "knock_in"])
def test_ranges_merge_to_the_whole_price(name, prec):
    S = kx.S("X")
    c = {"up_and_out": kx.up_and_out_call("X", 100.0, 130.0, 1.0),
         "asian": kx.scale((kx.average(S) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
         "knock_in": kx.anytime(S >= 120.0, kx.european_call("X", 100.0, 1.0))}[name]
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X")
    n = 5 * C + 123
    full = c.price(m, n_paths=n, seed=5, steps_per_year=252, precision=prec)
    parts = []
    for first, count in (sharded.shard_range(n, 3, r) for r in range(3)):
        parts += sharded.price_chunks(c, m, first, count, seed=5, steps_per_year=252, precision=prec)
    r = sharded.merge(parts)
    assert r.price == full.price and r.std_error == full.std_error and r.n_paths == n


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", ["up_and_out", "short_put_spread"])
def test_device_chunk_statistics_equal_the_host_mirror(name, prec):
    """The device's exact integer chunk sums and the host's give the same bits
    on the same per-path values (a ragged last chunk included)."""
    S = kx.S("X")
    c = {"up_and_out": kx.up_and_out_call("X", 100.0, 130.0, 1.0),
         "short_put_spread": kx.scale((90.0 - S).clip(0.0) - (110.0 - S).clip(0.0), kx.one()) @ kx.at(1.0)}[name]
    m = kx.GBM(s0=100.0, sigma=0.3, r=0.03, asset="X")
    n = 3 * C + 777
    _, pv = c.price(m, n_paths=n, seed=9, steps_per_year=252, precision=prec, per_path=True)
    dev = sharded.price_chunks(c, m, 0, n, seed=9, steps_per_year=252, precision=prec)
    host = [sharded.chunk_moments(pv[q:q + C]) for q in range(0, n, C)]
    assert dev == host


def test_ranges_must_start_on_a_chunk():
    c = kx.european_call("X", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X")
    with pytest.raises(kx.KontractError) as e:
        sharded.price_chunks(c, m, 100, 1000)
    assert e.value.status == "InvalidArgument"


def test_american_case_shards_equal_the_batch():
    """Each rank's share of a batch of American options priced in its own
    batched call gives the same results as the whole batch in one call (the
    cases are independent problems)."""
    put = kx.scale((kx.const_(40.0) - kx.S("X")).clip(0.0), kx.one())
    cases = [(put, kx.GBM(s0=s0, sigma=0.25, r=0.06, asset="X"), [i / 20 for i in range(1, 21)], 40_000, 3)
             for s0 in (34.0, 38.0, 42.0, 46.0, 50.0)]
    whole = kx.price_american_batch(cases, n_basis=3, basis="laguerre")
    for world in (2, 3):
        got = [None] * len(cases)
        for rank in range(world):
            mine = sharded.case_shard(len(cases), world, rank)
            for i, r in zip(mine, kx.price_american_batch([cases[i] for i in mine], n_basis=3, basis="laguerre")):
                got[i] = r
        assert [(r.price, r.std_error) for r in got] == [(r.price, r.std_error) for r in whole]


def test_surface_row_shards_equal_the_whole_surface():
    """Each rank's spot rows of a Greek surface, computed in its own
    kx_greek_surface call, are the whole surface's rows bit for bit (every
    cell reprices on the same seed whichever rows share its launch)."""
    c = kx.up_and_out_call("X", 100.0, 130.0, 1.0)
    spots, vols = [85.0, 95.0, 105.0, 115.0, 125.0], [0.15, 0.3]
    kw = dict(n_paths=20_000, seed=6, steps_per_year=52, rate=0.04)
    whole = kx.greek_surface(c, "X", spots, vols, **kw)
    for world in (2, 3):
        for rank in range(world):
            mine = sharded.case_shard(len(spots), world, rank)
            part = kx.greek_surface(c, "X", [spots[i] for i in mine], vols, **kw)
            for q, i in enumerate(mine):
                for f in kx.GreekSurface.QUANTITIES:
                    assert (getattr(part, f)[q] == getattr(whole, f)[i]).all(), (world, rank, f)
