"""Sharding one price over ranks: the chunk-aligned ranges, and the gather in
rank order + merge over a 2-rank gloo group on the CPU (the GPU call
replaced by synthetic chunk statistics), which must give every rank the
single-process merge of all chunks."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from kontracts_gb300 import sharded


def test_shard_ranges_cover_the_paths_in_whole_chunks():
    C = sharded.CHUNK
    for n in (0, 1, C - 1, C, C + 1, 5 * C + 123, 64 * C):
        for w in (1, 2, 3, 8):
            got = [sharded.shard_range(n, w, r) for r in range(w)]
            pos = 0
            for first, count in got:
                assert first == pos and count >= 0
                assert first % C == 0 or count == 0
                pos += count
            assert pos == n
    with pytest.raises(ValueError):
        sharded.shard_range(10, 2, 2)


def _chunks(first, count):
    """Synthetic per-chunk statistics of the paths [first, first + count):
    a function of the global chunk index only, like the GPU's."""
    C = sharded.CHUNK
    out = []
    for b in range(first, first + count, C):
        rng = np.random.default_rng(b // C)
        n = min(C, first + count - b)
        out.append((float(n), float(rng.normal(10.0, 1.0)), float(rng.uniform(1e3, 1e5))))
    return out


def _worker(rank, world, port, n_paths, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r = sharded.price_sharded(None, None, n_paths, chunk_fn=_chunks)
        q.put((rank, r.price, r.std_error, r.n_paths))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("n_paths", [5 * sharded.CHUNK + 123, sharded.CHUNK // 2])
def test_gloo_two_ranks_give_the_single_process_price(n_paths):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_paths, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = sharded.merge(_chunks(0, n_paths))
    for _, price, se, n in res:
        assert price == ref.price and se == ref.std_error and n == n_paths


def _fake_batch(cases):
    """Stand-in for the GPU batch: a function of each case alone."""
    return [(float(c[0]) * 1.5, float(c[0]) * 0.01, int(c[0]) + 7) for c in cases]


def _american_worker(rank, world, port, n_cases, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cases = [(i,) for i in range(n_cases)]
        q.put((rank, sharded.price_american_sharded(cases, batch_fn=_fake_batch)))
    finally:
        dist.destroy_process_group()


def test_case_shards_cover_every_case_once():
    for n in (0, 1, 5, 12):
        for w in (1, 2, 3, 8):
            got = sorted(i for r in range(w) for i in sharded.case_shard(n, w, r))
            assert got == list(range(n))


@pytest.mark.parametrize("n_cases", [12, 1])
def test_gloo_two_ranks_price_every_american_case(n_cases):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_american_worker, args=(r, 2, port, n_cases, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = _fake_batch([(i,) for i in range(n_cases)])
    for _, got in res:
        assert got == want


def _fake_surface(spots, vols):
    """A deterministic stand-in for one GPU's surface of the given spot rows."""
    import kontracts_gb300 as kx

    class _G:
        def __init__(self, s, v):
            for k, f in enumerate(kx.GreekSurface.QUANTITIES):
                setattr(self, f, s * 1000.0 + v * 10.0 + k)
    return kx.GreekSurface(spots, vols, [_G(s, v) for s in spots for v in vols])


def _surface_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spots, vols = [80.0, 90.0, 100.0, 110.0, 120.0], [0.1, 0.2, 0.3]
        s = sharded.greek_surface_sharded(None, "S", spots, vols, surface_fn=lambda sub: _fake_surface(sub, vols))
        f = sharded.population_sharded(lambda pts: [sum(x * x for x in p) for p in pts])
        pop = [[float(i), 1.0, -float(i)] for i in range(7)]
        q.put((rank, {k: getattr(s, k).tolist() for k in ("price", "delta", "rho_se")}, f(pop)))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_shard_surface_rows_and_populations():
    """Surface rows and calibration candidates split over two gloo ranks: every
    rank assembles the whole surface and every objective, equal to one process."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_surface_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    vols = [0.1, 0.2, 0.3]
    want = _fake_surface([80.0, 90.0, 100.0, 110.0, 120.0], vols)
    pop = [[float(i), 1.0, -float(i)] for i in range(7)]
    for _, surf, objs in res:
        for k in ("price", "delta", "rho_se"):
            assert surf[k] == getattr(want, k).tolist()
        assert objs == [sum(x * x for x in p) for p in pop]
