"""THE ORACLE (test infrastructure only): ctypes wrapper of oracle/libkx_oracle.so,
the CPU restatement of the reference pricer (see kx_oracle.cpp).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this package; the engine (kontracts_gb300/) never does.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libkx_oracle.so")


def _load_abi():
    """The ctypes mirror of the C structures (kontracts_gb300/_abi.py). When the
    engine package is already imported (the tests), its module is shared, so
    that its model objects pass straight through; otherwise that one file is
    loaded on its own, without the engine package or its library, so that a
    CPU-only run of the oracle loads no engine code."""
    mod = sys.modules.get("kontracts_gb300._abi")
    if mod is not None:
        return mod
    path = os.path.join(os.path.dirname(HERE), "kontracts_gb300", "_abi.py")
    spec = importlib.util.spec_from_file_location("_kx_oracle_abi", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_abi = _load_abi()


def _as_struct(obj, cls):
    """obj as an instance of cls: a structure of the same layout from another
    copy of the mirror module is copied field by field."""
    if isinstance(obj, cls):
        return obj
    out = cls()
    for f, _ in cls._fields_:
        setattr(out, f, getattr(obj, f))
    return out


class OracleError(ValueError):
    def __init__(self, code: int, msg: str):
        self.code = code
        self.status = _abi.STATUS_NAMES.get(code, str(code))
        super().__init__(f"{self.status}: {msg}")


class Result:
    def __init__(self, r: _abi.KxPriceResult):
        self.price, self.sample_std, self.std_error = r.price, r.sample_std, r.std_error
        self.ci95_low, self.ci95_high, self.n_paths = r.ci95_low, r.ci95_high, int(r.n_paths)

    def paths_for_tolerance(self, tol: float) -> int:
        import math
        if tol <= 0.0 or self.sample_std == 0.0:
            return 0
        return int(math.ceil((1.959963984540054 * self.sample_std / tol) ** 2))


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _model_c(model) -> _abi.KxModel:
    return _as_struct(model._c() if hasattr(model, "_c") else model, _abi.KxModel)


def _rate(model, rate):
    if rate is not None:
        return float(rate)
    return float(getattr(model, "rate", 0.0))


class Oracle:
    def __init__(self, threads: int = 0):
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        self.L = L
        D, P = C.c_double, C.POINTER
        L.ko_last_error.restype = C.c_char_p
        L.ko_set_threads.argtypes = [C.c_int]
        L.ko_max_threads.restype = C.c_int
        L.ko_set_shared_draws.argtypes = [P(D), C.c_uint64, C.c_uint64]
        L.ko_parse.argtypes = [C.c_char_p]
        L.ko_plan.argtypes = [C.c_char_p, P(_abi.KxPlanInfo), P(D), C.c_size_t, C.c_char_p, C.c_size_t]
        L.ko_time_grid.argtypes = [C.c_char_p, C.c_uint32, C.c_int, P(D), C.c_size_t, P(C.c_size_t)]
        L.ko_simulate.argtypes = [P(_abi.KxModel), P(D), C.c_size_t, C.c_uint64, P(_abi.KxMcConfig), P(D)]
        L.ko_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_size_t, P(D)]
        L.ko_price.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(_abi.KxPriceResult), P(D)]
        L.ko_price_vr.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), C.c_int, P(_abi.KxPriceResult)]
        L.ko_price_on_grid.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(D), C.c_size_t,
                                       P(_abi.KxPriceResult)]
        L.ko_price_batch.argtypes = [C.c_size_t, P(C.c_char_p), P(_abi.KxModel), P(_abi.KxMcConfig),
                                     P(_abi.KxPriceResult)]
        L.ko_greeks.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(_abi.KxBumps),
                                P(_abi.KxGreeks)]
        L.ko_greek_surface.argtypes = [C.c_char_p, C.c_char_p, P(D), C.c_size_t, P(D), C.c_size_t,
                                       P(_abi.KxMcConfig), P(_abi.KxBumps), P(_abi.KxGreeks)]
        L.ko_calib_gbm_prices.argtypes = [C.c_char_p, C.c_char_p, P(D), C.c_size_t, P(D), C.c_size_t,
                                          P(_abi.KxMcConfig), P(D)]
        L.ko_calib_heston_objective.argtypes = [C.c_char_p, C.c_char_p, P(D), C.c_size_t, P(D), C.c_size_t,
                                                P(_abi.KxMcConfig), P(D)]
        L.ko_mlmc_level_values.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), C.c_uint32, C.c_uint64,
                                           P(D)]
        L.ko_mlmc_optimal_allocation.argtypes = [P(D), P(C.c_uint64), C.c_size_t, C.c_double, P(C.c_uint64)]
        L.ko_price_mlmc.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(_abi.KxMlmcCfg),
                                    P(_abi.KxMlmcResult)]
        L.ko_price_multi.argtypes = [C.c_char_p, P(_abi.KxMultiGbm), P(_abi.KxMcConfig), P(_abi.KxPriceResult), P(D)]
        L.ko_price_american.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(D), C.c_size_t,
                                        C.c_int, P(_abi.KxPriceResult), P(D)]
        L.ko_price_american_detail.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(D), C.c_size_t,
                                               C.c_int, C.c_int, P(_abi.KxPriceResult), P(D), P(C.c_int32), P(D)]
        L.ko_price_american_basis.argtypes = [C.c_char_p, P(_abi.KxModel), P(_abi.KxMcConfig), P(D), C.c_size_t,
                                              C.c_int, C.c_int, P(_abi.KxPriceResult), P(D)]
        for f, n in [("ko_bs_call", 5), ("ko_bs_put", 5), ("ko_down_and_out_call", 6), ("ko_up_and_out_call", 6),
                     ("ko_norm_cdf_as", 1)]:
            fn = getattr(L, f)
            fn.restype = D
            fn.argtypes = [D] * n
        L.ko_value_on_path.argtypes = [C.c_char_p, P(D), P(D), C.c_size_t, C.c_char_p, D, P(D)]
        L.ko_bs_call_greeks.argtypes = [D] * 5 + [P(D)]
        L.ko_crr_american.restype = D
        L.ko_crr_american.argtypes = [D, D, D, D, D, C.c_int, C.c_int]
        L.ko_heston_call.restype = D
        L.ko_heston_call.argtypes = [D] * 9
        if threads:
            L.ko_set_threads(threads)

    # ---- helpers ----
    def _chk(self, st: int) -> None:
        if st != 0:
            raise OracleError(st, self.L.ko_last_error().decode())

    @staticmethod
    def cfg(n_paths, seed, spy, rate, shared=False) -> _abi.KxMcConfig:
        return _abi.KxMcConfig(n_paths=int(n_paths), seed=int(seed) & (2**64 - 1), steps_per_year=int(spy),
                               rng=_abi.KX_RNG_SHARED_DRAWS if shared else _abi.KX_RNG_PHILOX,
                               precision=_abi.KX_PREC_FP64, flags=0, rate=float(rate))

    def threads(self) -> int:
        return self.L.ko_max_threads()

    def set_threads(self, n: int) -> None:
        self.L.ko_set_threads(int(n))

    # ---- API ----
    def set_shared_draws(self, z: np.ndarray) -> None:
        z = np.ascontiguousarray(z, dtype=np.float64)
        self._chk(self.L.ko_set_shared_draws(z.ctypes.data_as(C.POINTER(C.c_double)), z.shape[0], z.shape[1]))

    def parse(self, js: str) -> None:
        self._chk(self.L.ko_parse(js.encode()))

    def plan(self, js: str) -> dict:
        info = _abi.KxPlanInfo()
        dates = (C.c_double * 4096)()
        buf = C.create_string_buffer(1 << 16)
        self._chk(self.L.ko_plan(js.encode(), C.byref(info), dates, 4096, buf, len(buf)))
        return dict(assets=buf.value.decode().split("\n") if info.n_assets else [],
                    fixed_dates=list(dates[: info.n_fixed_dates]), horizon=info.horizon,
                    needs_fine_grid=bool(info.needs_fine_grid))

    def time_grid(self, js: str, spy: int, force: bool = False) -> list[float]:
        n = C.c_size_t()
        out = (C.c_double * 200000)()
        self._chk(self.L.ko_time_grid(js.encode(), spy, int(force), out, 200000, C.byref(n)))
        return list(out[: n.value])

    def simulate(self, model, grid, n_paths, seed, shared=False) -> np.ndarray:
        g = np.ascontiguousarray(grid, dtype=np.float64)
        out = np.zeros((n_paths, len(g)))
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, 0, 0.0, shared)
        self._chk(self.L.ko_simulate(C.byref(cm), g.ctypes.data_as(C.POINTER(C.c_double)), len(g), n_paths,
                                     C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def normals(self, seed: int, path: int, n: int) -> np.ndarray:
        out = np.zeros(n)
        self._chk(self.L.ko_normals(seed, path, n, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def price(self, js: str, model, n_paths=100_000, seed=42, steps_per_year=50, rate=None, shared=False,
              per_path=False):
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, steps_per_year, _rate(model, rate), shared)
        r = _abi.KxPriceResult()
        pp = np.zeros(max(1, n_paths)) if per_path else None
        self._chk(self.L.ko_price(js.encode(), C.byref(cm), C.byref(cfg), C.byref(r),
                                  pp.ctypes.data_as(C.POINTER(C.c_double)) if per_path else None))
        return (Result(r), pp[:n_paths]) if per_path else Result(r)

    def price_vr(self, js: str, model, n_paths=100_000, seed=42, steps_per_year=50, antithetic=False,
                 control_variate=False, rate=None, shared=False) -> Result:
        """price_gbm with variance reduction (pricer.rs:108-230)."""
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, steps_per_year, _rate(model, rate), shared)
        r = _abi.KxPriceResult()
        flags = (1 if antithetic else 0) | (2 if control_variate else 0)
        self._chk(self.L.ko_price_vr(js.encode(), C.byref(cm), C.byref(cfg), flags, C.byref(r)))
        return Result(r)

    def price_on_grid(self, js: str, model, grid, n_paths, seed, rate=None, shared=False) -> Result:
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, 0, _rate(model, rate), shared)
        g = np.ascontiguousarray(grid, dtype=np.float64)
        r = _abi.KxPriceResult()
        self._chk(self.L.ko_price_on_grid(js.encode(), C.byref(cm), C.byref(cfg),
                                          g.ctypes.data_as(C.POINTER(C.c_double)), len(g), C.byref(r)))
        return Result(r)

    def price_batch(self, jss, model, n_paths=100_000, seed=42, steps_per_year=50, rate=None):
        arr = (C.c_char_p * len(jss))(*[j.encode() for j in jss])
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, steps_per_year, _rate(model, rate))
        out = (_abi.KxPriceResult * len(jss))()
        self._chk(self.L.ko_price_batch(len(jss), arr, C.byref(cm), C.byref(cfg), out))
        return [Result(r) for r in out]

    def greeks(self, js: str, model, n_paths=200_000, seed=42, steps_per_year=50, bumps=(1e-2, 1e-2, 1e-4),
               relative=False, shared=False) -> dict:
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, steps_per_year, _rate(model, None), shared)
        b = _abi.KxBumps(spot=bumps[0], vol=bumps[1], rate=bumps[2], relative=int(relative), smooth=0,
                         smoothing_width=0.0)
        g = _abi.KxGreeks()
        self._chk(self.L.ko_greeks(js.encode(), C.byref(cm), C.byref(cfg), C.byref(b), C.byref(g)))
        return {k: getattr(g, k) for k, _ in g._fields_}

    def greek_surface(self, js: str, asset: str, spots, vols, n_paths=100_000, seed=42, steps_per_year=50,
                      rate=0.0, bumps=(1e-2, 1e-2, 1e-4), relative=False) -> list:
        """greek_surface (surface.rs:104-137): a row-major list of greeks dicts,
        cell i * len(vols) + j for spots[i], vols[j]."""
        sp = (C.c_double * max(1, len(spots)))(*spots)
        vo = (C.c_double * max(1, len(vols)))(*vols)
        cfg = self.cfg(n_paths, seed, steps_per_year, rate)
        b = _abi.KxBumps(spot=bumps[0], vol=bumps[1], rate=bumps[2], relative=int(relative), smooth=0,
                         smoothing_width=0.0)
        out = (_abi.KxGreeks * max(1, len(spots) * len(vols)))()
        self._chk(self.L.ko_greek_surface(js.encode(), asset.encode(), sp, len(spots), vo, len(vols), C.byref(cfg),
                                          C.byref(b), out))
        return [{k: getattr(g, k) for k, _ in g._fields_} for g in out[: len(spots) * len(vols)]]

    def calib_gbm_prices(self, js: str, asset: str, spots, sigmas, n_paths=1000, seed=42, steps_per_year=252,
                         rate=0.0) -> np.ndarray:
        """gbm_prices (calibration.rs:72-90) per volatility: [len(sigmas), len(spots)]."""
        sp = np.ascontiguousarray(spots, dtype=np.float64)
        sg = np.ascontiguousarray(sigmas, dtype=np.float64)
        out = np.zeros(max(1, len(sp) * len(sg)))
        cfg = self.cfg(n_paths, seed, steps_per_year, rate)
        self._chk(self.L.ko_calib_gbm_prices(js.encode(), asset.encode(), sp.ctypes.data_as(C.POINTER(C.c_double)),
                                             len(sp), sg.ctypes.data_as(C.POINTER(C.c_double)), len(sg),
                                             C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[: len(sp) * len(sg)].reshape(len(sg), len(sp))

    def calib_heston_objective(self, js: str, asset: str, quotes, params, n_paths=1000, seed=42,
                               steps_per_year=252, rate=0.0) -> np.ndarray:
        """eval_obj_heston (calibration.rs:103-126) for each row of params."""
        q = np.ascontiguousarray(quotes, dtype=np.float64).reshape(-1, 2)
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(-1, 5)
        obj = np.zeros(max(1, len(p)))
        cfg = self.cfg(n_paths, seed, steps_per_year, rate)
        self._chk(self.L.ko_calib_heston_objective(js.encode(), asset.encode(),
                                                   q.ctypes.data_as(C.POINTER(C.c_double)), len(q),
                                                   p.ctypes.data_as(C.POINTER(C.c_double)), len(p), C.byref(cfg),
                                                   obj.ctypes.data_as(C.POINTER(C.c_double))))
        return obj[: len(p)]

    def mlmc_level_values(self, js: str, model, level: int, n: int, seed=42, rate=None) -> np.ndarray:
        """level_samples (mlmc.rs:276-305): P_l - P_(l-1) per coupled path."""
        cm = _model_c(model)
        cfg = self.cfg(0, seed, 0, _rate(model, rate))
        out = np.zeros(max(1, n))
        self._chk(self.L.ko_mlmc_level_values(js.encode(), C.byref(cm), C.byref(cfg), int(level), int(n),
                                              out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[:n]

    def mlmc_optimal_allocation(self, variances, costs, target) -> list:
        n = min(len(variances), len(costs))
        v = (C.c_double * max(1, n))(*variances[:n])
        c = (C.c_uint64 * max(1, n))(*costs[:n])
        out = (C.c_uint64 * max(1, n))()
        self._chk(self.L.ko_mlmc_optimal_allocation(v, c, n, float(target), out))
        return list(out[:n])

    def price_mlmc(self, js: str, model, n_levels=6, pilot_paths=2000, target_variance=1e-4, cost_per_step=1,
                   seed=42, rate=None) -> dict:
        """price_mlmc_detailed (mlmc.rs:107-215)."""
        cm = _model_c(model)
        cfg = self.cfg(0, seed, 0, _rate(model, rate))
        mc = _abi.KxMlmcCfg(n_levels=n_levels, cost_per_step=cost_per_step, pilot_paths=pilot_paths,
                            target_variance=target_variance)
        out = _abi.KxMlmcResult()
        self._chk(self.L.ko_price_mlmc(js.encode(), C.byref(cm), C.byref(cfg), C.byref(mc), C.byref(out)))
        k = out.n_levels + 1
        return {"price": Result(out.price), "level_means": list(out.level_means[:k]),
                "level_variances": list(out.level_variances[:k]), "level_costs": list(out.level_costs[:k]),
                "level_paths": list(out.level_paths[:k]), "total_cost": out.total_cost}

    def price_multi(self, js: str, model, n_paths=100_000, seed=42, steps_per_year=50, per_path=False):
        """price_gbm under CorrelatedGbmN (multi_asset.rs:107-170)."""
        mm = _as_struct(model._c(), _abi.KxMultiGbm)
        cfg = self.cfg(n_paths, seed, steps_per_year, model.rate)
        r = _abi.KxPriceResult()
        pp = np.zeros(max(1, n_paths)) if per_path else None
        self._chk(self.L.ko_price_multi(js.encode(), C.byref(mm), C.byref(cfg), C.byref(r),
                                        pp.ctypes.data_as(C.POINTER(C.c_double)) if per_path else None))
        return (Result(r), pp[:n_paths]) if per_path else Result(r)

    def price_american(self, js: str, model, dates, n_paths=100_000, seed=42, n_basis=3, shared=False,
                       per_path=False, basis="monomial"):
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, 50, _rate(model, None), shared)
        d = (C.c_double * len(dates))(*dates)
        r = _abi.KxPriceResult()
        pp = np.zeros(max(1, n_paths)) if per_path else None
        self._chk(self.L.ko_price_american_basis(js.encode(), C.byref(cm), C.byref(cfg), d, len(dates), n_basis,
                                                 1 if basis == "laguerre" else 0, C.byref(r),
                                                 pp.ctypes.data_as(C.POINTER(C.c_double)) if per_path else None))
        return (Result(r), pp[:n_paths]) if per_path else Result(r)

    def price_american_detail(self, js: str, model, dates, n_paths=100_000, seed=42, n_basis=3, shared=False,
                              basis="monomial"):
        """price_american_lsm with per-path detail: (result, realised values,
        exercise date index per path (-1: never exercised), decision margin
        per path: the smallest |exercise - continuation| over its regression
        decisions)."""
        cm = _model_c(model)
        cfg = self.cfg(n_paths, seed, 50, _rate(model, None), shared)
        d = (C.c_double * len(dates))(*dates)
        r = _abi.KxPriceResult()
        n = max(1, n_paths)
        pv, ex, mg = np.zeros(n), np.zeros(n, dtype=np.int32), np.zeros(n)
        self._chk(self.L.ko_price_american_detail(js.encode(), C.byref(cm), C.byref(cfg), d, len(dates), n_basis,
                                                  1 if basis == "laguerre" else 0, C.byref(r),
                                                  pv.ctypes.data_as(C.POINTER(C.c_double)),
                                                  ex.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  mg.ctypes.data_as(C.POINTER(C.c_double))))
        return Result(r), pv[:n_paths], ex[:n_paths], mg[:n_paths]

    def value_on_path(self, js: str, times, values, asset: str = "S", rate: float = 0.0) -> float:
        t = np.ascontiguousarray(times, dtype=np.float64)
        v = np.ascontiguousarray(values, dtype=np.float64)
        out = C.c_double()
        self._chk(self.L.ko_value_on_path(js.encode(), t.ctypes.data_as(C.POINTER(C.c_double)),
                                          v.ctypes.data_as(C.POINTER(C.c_double)), len(t), asset.encode(),
                                          float(rate), C.byref(out)))
        return out.value

    # ---- closed forms ----
    def bs_call(self, s, k, t, r, sigma): return self.L.ko_bs_call(s, k, t, r, sigma)
    def bs_put(self, s, k, t, r, sigma): return self.L.ko_bs_put(s, k, t, r, sigma)
    def norm_cdf_as(self, x): return self.L.ko_norm_cdf_as(x)

    def bs_call_greeks(self, s, k, t, r, sigma) -> dict:
        o = (C.c_double * 5)()
        self.L.ko_bs_call_greeks(s, k, t, r, sigma, o)
        return dict(price=o[0], delta=o[1], gamma=o[2], vega=o[3], rho=o[4])

    def down_and_out_call(self, s, k, h, r, sigma, t): return self.L.ko_down_and_out_call(s, k, h, r, sigma, t)
    def up_and_out_call(self, s, k, h, r, sigma, t): return self.L.ko_up_and_out_call(s, k, h, r, sigma, t)

    def crr_american(self, s0, k, t, r, sigma, n, is_call):
        return self.L.ko_crr_american(s0, k, t, r, sigma, n, int(is_call))

    def heston_call(self, s0, k, t, r, v0, kappa, theta, sigma_v, rho):
        return self.L.ko_heston_call(s0, k, t, r, v0, kappa, theta, sigma_v, rho)
