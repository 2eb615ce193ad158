"""Multilevel Monte Carlo (src/mlmc.rs) on the GPU: the telescoping estimator
E[P_L] = E[P_0] + sum_l E[P_l - P_(l-1)] over uniform grids of 2^l steps,
with the reference's pilot phase, optimal allocation and extra phase.

Each phase is two path launches (every level's fine paths, then every
level's coarse paths, whose steps add the normals of two fine steps of the
same Philox stream) and one statistics launch of the per-path differences.
FP64 paths by default (the reference's precision)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

from . import _abi, _cfg, _check, _lib, _lock, Contract, PriceResult


@dataclass
class MlmcConfig:
    """mlmc.rs:50-72 (defaults :63-72)."""
    n_levels: int = 6
    pilot_paths: int = 2_000
    target_variance: float = 1e-4
    cost_per_step: int = 1


@dataclass
class MlmcResult:
    """mlmc.rs:75-96: the estimate and, per level 0..L, the mean and variance
    of P_l - P_(l-1), the cost of one path (steps) and the number of paths."""
    price: PriceResult
    level_means: list
    level_variances: list
    level_costs: list
    level_paths: list
    total_cost: int


def _model_rate(model, rate):
    return float(model.rate if rate is None else rate)


def price_mlmc_detailed(contract: Contract, model, mlmc: MlmcConfig | None = None, *, seed: int = 42,
                        rate: float | None = None, precision: str = "fp64") -> MlmcResult:
    """price_mlmc_detailed (mlmc.rs:107-215) for a GBM or Heston model
    (reference Heston scheme); `seed` and `rate` are McConfig's (the rate
    defaults to the model's)."""
    mlmc = mlmc or MlmcConfig()
    mc = _abi.KxMlmcCfg(n_levels=int(mlmc.n_levels), cost_per_step=int(mlmc.cost_per_step),
                        pilot_paths=int(mlmc.pilot_paths), target_variance=float(mlmc.target_variance))
    cfg = _cfg(0, seed, 0, _model_rate(model, rate), precision, False)
    cm = model._c()
    out = _abi.KxMlmcResult()
    with _lock:
        _check(_lib().kx_price_mlmc(contract._handle().h, C.byref(cm), C.byref(cfg), C.byref(mc), C.byref(out)))
    n = out.n_levels + 1
    return MlmcResult(price=PriceResult(out.price), level_means=list(out.level_means[:n]),
                      level_variances=list(out.level_variances[:n]), level_costs=list(out.level_costs[:n]),
                      level_paths=list(out.level_paths[:n]), total_cost=int(out.total_cost))


def price_mlmc(contract: Contract, model, mlmc: MlmcConfig | None = None, **kw) -> PriceResult:
    """price_mlmc (mlmc.rs:99-106)."""
    return price_mlmc_detailed(contract, model, mlmc, **kw).price


def estimate_variance_at_level(contract: Contract, model, level: int, n_pilot: int, *, seed: int = 42,
                               rate: float | None = None, precision: str = "fp64") -> float:
    """estimate_variance_at_level (mlmc.rs:218-229)."""
    cfg = _cfg(0, seed, 0, _model_rate(model, rate), precision, False)
    cm = model._c()
    v = C.c_double()
    with _lock:
        _check(_lib().kx_mlmc_level_variance(contract._handle().h, C.byref(cm), C.byref(cfg), int(level),
                                             int(n_pilot), C.byref(v)))
    return v.value


def optimal_allocation(variances: Sequence[float], costs: Sequence[int], target_var: float) -> list:
    """optimal_allocation (mlmc.rs:231-258)."""
    n = min(len(variances), len(costs))
    va = (C.c_double * max(1, n))(*[float(v) for v in variances[:n]])
    ca = (C.c_uint64 * max(1, n))(*[int(c) for c in costs[:n]])
    out = (C.c_uint64 * max(1, n))()
    _check(_lib().kx_mlmc_optimal_allocation(va, ca, n, float(target_var), out))
    return [int(x) for x in out[:n]]


__all__ = ["MlmcConfig", "MlmcResult", "price_mlmc", "price_mlmc_detailed", "estimate_variance_at_level",
           "optimal_allocation"]
