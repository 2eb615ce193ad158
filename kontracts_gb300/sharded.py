"""Work sharded over ranks (one GPU per rank, torch.distributed).

Paths are independent and the Philox counter of a path is its index, so a
price shards without any exchange on the data path: rank r of w prices a
contiguous, chunk-aligned range of the paths of one stream (the same paths a
single GPU would simulate for that range) and keeps its statistics per chunk
of KX_STATS_CHUNK paths. The only collective is the gather of those chunk
statistics (three doubles per 16,384 paths); every rank merges them in path
order, so every rank returns exactly the price one GPU gives for all paths.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

from . import _abi

CHUNK = _abi.KX_STATS_CHUNK


def shard_range(n_paths: int, world: int, rank: int) -> tuple[int, int]:
    """(first_path, count) of rank `rank`: whole chunks, the first ranks take
    one chunk more when the chunks do not divide evenly."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    n_chunks = (n_paths + CHUNK - 1) // CHUNK
    base, extra = divmod(n_chunks, world)
    c0 = rank * base + min(rank, extra)
    c1 = c0 + base + (1 if rank < extra else 0)
    first = min(c0 * CHUNK, n_paths)
    return first, min(c1 * CHUNK, n_paths) - first


def price_chunks(contract, model, first_path: int, n_paths: int, seed: int = 42, steps_per_year: int = 50,
                 precision: str = "fp32") -> list[tuple[float, float, float]]:
    """Chunk statistics (n, mean, M2) of paths first_path .. first_path + n_paths - 1."""
    from . import _cfg, _check, _lib, _lock
    cm = model._c()
    cfg = _cfg(n_paths, seed, steps_per_year, model.rate, precision, False)
    cap = max(1, (n_paths + CHUNK - 1) // CHUNK)
    out = (_abi.KxChunkStats * cap)()
    n_out = C.c_size_t()
    with _lock:
        _check(_lib().kx_price_chunks(contract._handle().h, C.byref(cm), C.byref(cfg), int(first_path), out, cap,
                                      C.byref(n_out)))
    return [(out[q].n, out[q].mean, out[q].m2) for q in range(n_out.value)]


def chunk_moments(values, subtrahend=None) -> tuple[float, float, float]:
    """(n, mean, M2) of one chunk of at most CHUNK values (values[i], or
    values[i] - subtrahend[i]) on the host, bit for bit as the device's chunk
    reduction computes them for finite values."""
    import numpy as np
    from . import _check, _lib
    a = np.ascontiguousarray(values, dtype=np.float64)
    pb = None
    if subtrahend is not None:
        b = np.ascontiguousarray(subtrahend, dtype=np.float64)
        if b.shape != a.shape:
            raise ValueError("values and subtrahend differ in length")
        pb = b.ctypes.data_as(C.POINTER(C.c_double))
    out = _abi.KxChunkStats()
    _check(_lib().kx_chunk_moments(a.ctypes.data_as(C.POINTER(C.c_double)), pb, len(a), C.byref(out)))
    return (out.n, out.mean, out.m2)


def merge(chunks: Sequence[tuple[float, float, float]]):
    """The price of chunk statistics merged in the given order (the library's
    own merge, so the result equals kx_price's bit for bit)."""
    from . import PriceResult, _check, _lib
    arr = (_abi.KxChunkStats * max(1, len(chunks)))(*[_abi.KxChunkStats(*c) for c in chunks])
    out = _abi.KxPriceResult()
    _check(_lib().kx_merge_chunks(arr, len(chunks), C.byref(out)))
    return PriceResult(out)


def price_sharded(contract, model, n_paths: int, seed: int = 42, steps_per_year: int = 50, precision: str = "fp32",
                  group=None, chunk_fn: Callable[[int, int], list] | None = None):
    """Price over the ranks of `group` (the default process group). Every rank
    returns the same PriceResult, equal to one GPU's. chunk_fn(first, count)
    replaces the GPU call (it returns that range's chunk statistics)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    first, count = shard_range(n_paths, world, rank)
    if chunk_fn is not None:
        mine = chunk_fn(first, count)
    elif count:
        mine = price_chunks(contract, model, first, count, seed, steps_per_year, precision)
    else:
        mine = []
    gathered: list = [None] * world
    dist.all_gather_object(gathered, mine, group=group)
    return merge([c for part in gathered for c in part])


def case_shard(n_cases: int, world: int, rank: int) -> list[int]:
    """The cases of rank `rank`: i = rank, rank + world, ... (every case on
    exactly one rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    return list(range(rank, n_cases, world))


def price_american_sharded(cases: Sequence[tuple], n_basis: int = 3, *, precision: str = "fp32",
                           basis: str = "monomial", group=None, batch_fn: Callable | None = None):
    """Independent American options (the cases of price_american_batch)
    sharded over the ranks of `group`: rank r prices cases r, r + w, ... in
    one batched call on its GPU; the only collective is the gather of the
    results. Every rank returns all results in case order, each equal to the
    single-GPU result of its case. batch_fn(cases) replaces the GPU call (it
    returns one (price, std_error, n_paths) per case)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = case_shard(len(cases), world, rank)
    if batch_fn is not None:
        got = batch_fn([cases[i] for i in mine])
    elif mine:
        from . import price_american_batch
        got = [(r.price, r.std_error, r.n_paths)
               for r in price_american_batch([cases[i] for i in mine], n_basis, precision=precision, basis=basis)]
    else:
        got = []
    gathered: list = [None] * world
    dist.all_gather_object(gathered, list(zip(mine, got)), group=group)
    out: list = [None] * len(cases)
    for part in gathered:
        for i, res in part:
            out[i] = res
    return out


def greek_surface_sharded(contract, asset: str, spots: Sequence[float], vols: Sequence[float], *, group=None,
                          surface_fn: Callable | None = None, **kw):
    """greek_surface (surface.rs:104-137) sharded over the ranks of `group`:
    rank r computes the rows of spots r, r + w, ... (all vols) in one
    kx_greek_surface call on its GPU, all on the same seed as the
    single-GPU surface; the only collective is the gather of the rows. Every
    rank returns the whole GreekSurface, cell for cell the single-GPU one.
    surface_fn(spots_subset) -> GreekSurface replaces the GPU call."""
    import torch.distributed as dist
    from . import GreekSurface, KontractError, greek_surface
    if not spots or not vols:
        raise KontractError(_abi.KX_INCONSISTENT_PATH, "empty surface grid")  # surface.rs:113-117
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = case_shard(len(spots), world, rank)
    rows = []
    if mine:
        sub = [spots[i] for i in mine]
        s = surface_fn(sub) if surface_fn is not None else greek_surface(contract, asset, sub, vols, **kw)
        for q, i in enumerate(mine):
            rows.append((i, {f: [float(x) for x in getattr(s, f)[q]] for f in GreekSurface.QUANTITIES}))
    gathered: list = [None] * world
    dist.all_gather_object(gathered, rows, group=group)
    by_row = {i: r for part in gathered for i, r in part}

    class _Cell:
        pass
    cells = []
    for i in range(len(spots)):
        for j in range(len(vols)):
            c = _Cell()
            for f in GreekSurface.QUANTITIES:
                setattr(c, f, by_row[i][f][j])
            cells.append(c)
    return GreekSurface(spots, vols, cells)


def population_sharded(objective_batch: Callable, *, group=None) -> Callable:
    """A batched calibration objective (for instance a CMA-ES generation, as
    kontracts_gb300.calibration.heston_objective evaluates one) sharded over
    the ranks of `group`: every rank calls the returned function with the
    same population, evaluates candidates r, r + w, ... on its GPU and
    all-gathers the objectives, so every rank's optimizer sees the same
    values and takes the same steps."""
    import torch.distributed as dist

    def sharded(points):
        world = dist.get_world_size(group)
        rank = dist.get_rank(group)
        mine = case_shard(len(points), world, rank)
        vals = list(objective_batch([points[i] for i in mine])) if mine else []
        gathered: list = [None] * world
        dist.all_gather_object(gathered, [(i, float(v)) for i, v in zip(mine, vals)], group=group)
        out = [0.0] * len(points)
        for part in gathered:
            for i, v in part:
                out[i] = v
        return out

    return sharded
