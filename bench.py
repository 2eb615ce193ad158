"""Benchmark of the compiled-contract pricing path (one JSON line on stdout).

Workload (N = 1): the up-and-out barrier call on GBM, call.until(S >= 200):
s0 = 180, K = 100, B = 200, sigma = 0.25, r = 0.05, T = 1, 365 steps a year
(366-point grid, barrier checked at every point), 4,000,000 paths, FP32 path
arithmetic with FP64 payoff sums, Philox normals. One "step" is one kx_price
call over that batch.

  value      nominal path-steps / s of the device work of a call (path kernel
             + reduction), tables already on the device, L2 flushed between
             steps (a 256 MB write);
  e2e        the same metric through the C ABI call kx_price from the host
             (lowering, table upload, kernels, result download) by wall clock;
  roofline   the path kernel's simulated steps/s against the ceiling measured
             in the same run: the bare simulation loop (Philox draw,
             Box-Muller, log-space update, no contract) on the same GPU.
             The kernel moves 8 bytes per path to HBM and is bound by
             instruction issue, not by HBM or tensor cores;
  cpu_baseline  the oracle (CPU restatement of the reference pricer) on a
             bounded sample of the same workload on this host's cores.

`--impl reference` times that CPU restatement alone (all host threads), the
reference's own CPU pricer being Rust that cannot be built here.
Multi-GPU: `--gpus N` starts N ranks under torch.distributed.run (or runs
as one rank of an outer torchrun). Weak scaling (default): every rank prices
its own batch on its own GPU with its own Philox stream, no collective on the
data path. Strong scaling (`--scaling strong`): one price of `--paths` paths,
each rank a chunk-aligned range of the same stream, the per-chunk statistics
gathered and merged (the single-GPU result). value = all ranks' path-steps /
the slowest rank's device time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="up-and-out barrier call on GBM, call.until(S>=200), 366-point daily grid",
                s0=180.0, strike=100.0, barrier=200.0, sigma=0.25, r=0.05, maturity=1.0, steps_per_year=365,
                n_paths=4_000_000, path_dtype="fp32", accumulate="fp64", rng="philox4x32-10")
METRIC = "path-steps/s"
UNIT = "path-steps/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws: int) -> None:
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(seconds: float = 12.0) -> dict:
    """The oracle on a bounded sample of the workload on this host."""
    import kontracts_gb300 as kx
    from oracle import Oracle
    orc = Oracle()
    w = WORKLOAD
    c = kx.up_and_out_call("S", w["strike"], w["barrier"], w["maturity"])
    m = kx.GBM(s0=w["s0"], sigma=w["sigma"], r=w["r"], asset="S")
    js = c.to_json()
    steps = len(c.time_grid(w["steps_per_year"])) - 1
    pilot = 20_000
    t = time.perf_counter()
    orc.price(js, m, n_paths=pilot, seed=42, steps_per_year=w["steps_per_year"])
    dt = time.perf_counter() - t
    n = int(min(w["n_paths"], max(pilot, pilot * seconds / max(dt, 1e-6))))
    t = time.perf_counter()
    ref = orc.price(js, m, n_paths=n, seed=42, steps_per_year=w["steps_per_year"])
    dt = time.perf_counter() - t
    return {"value": n * steps / dt, "unit": UNIT, "cores": orc.threads(), "kind": "port",
            "sample": f"{n} of {w['n_paths']} paths x {steps} steps, CPU restatement of the reference "
                      f"pricer (materialised paths + recursive cash-flow walk), {dt:.2f} s",
            "_n": n, "_price": ref.price, "_se": ref.std_error}


def accuracy(cb: dict) -> dict:
    """The GPU's FP32 price against the FP64 CPU run on the same draws (the
    oracle's Philox paths of the baseline sample) and against the closed form
    (Reiner-Rubinstein up-and-out with the Broadie-Glasserman-Kou shift for
    daily monitoring)."""
    import kontracts_gb300 as kx
    from oracle import Oracle
    w = WORKLOAD
    c = kx.up_and_out_call("S", w["strike"], w["barrier"], w["maturity"])
    m = kx.GBM(s0=w["s0"], sigma=w["sigma"], r=w["r"], asset="S")
    n = cb["_n"]
    g = c.price(m, n_paths=n, seed=42, steps_per_year=w["steps_per_year"], precision="fp32")
    dt = 1.0 / w["steps_per_year"]
    bgk = w["barrier"] * math.exp(0.5826 * w["sigma"] * math.sqrt(dt))
    cf = Oracle().up_and_out_call(w["s0"], w["strike"], bgk, w["r"], w["sigma"], w["maturity"])
    se = math.sqrt(g.std_error ** 2 + cb["_se"] ** 2)
    return {"paths": n, "draws": "Philox4x32-10 seed 42, paths 0..n-1 on both",
            "gpu_fp32_price": g.price, "gpu_std_error": g.std_error, "cpu_fp64_price": cb["_price"],
            "gpu_minus_cpu": g.price - cb["_price"], "gpu_minus_cpu_rel": (g.price - cb["_price"]) / cb["_price"],
            "closed_form_bgk": cf, "gpu_minus_closed_form_in_se": (g.price - cf) / g.std_error,
            "cpu_minus_closed_form_in_combined_se": (cb["_price"] - cf) / se}


# The workload's contract, call.until(S >= 200) on the call max(S - 100, 0) at
# T = 1, as the reference's serde JSON (Contract::to_json, src/ast.rs:210-217).
WORKLOAD_JSON = ('{"Until":[{"Ge":[{"Spot":"S"},{"Const":200.0}]},{"When":[{"At":1.0},{"Scale":[{"Max":'
                 '[{"Sub":[{"Spot":"S"},{"Const":100.0}]},{"Const":0.0}]},{"One":"USD"}]}]}]}')


def _config(n_paths: int, ws: int) -> dict:
    """The `config` of both arms' lines (identical for the same workload)."""
    return dict(WORKLOAD, n_paths=n_paths, l2="flushed between timed steps (256 MB write) on the GPU arm",
                parallelism=f"paths sharded over {ws} GPU(s), no collective" if ws > 1 else "1 GPU")


def run_reference(args, ws, rank) -> None:
    """The CPU restatement of the reference pricer (the reference is Rust and
    cannot be built here) on the same workload as the GPU arm: the same
    contract, model, grid and number of paths per step. It loads no engine
    code: the contract is its serde JSON, the grid the oracle's own."""
    if rank != 0:
        return
    from oracle import Oracle, _abi
    orc = Oracle()
    w = WORKLOAD
    m = _abi.KxModel(kind=_abi.KX_MODEL_GBM, heston_scheme=0, s0=w["s0"], mu=w["r"], sigma=w["sigma"],
                     asset=b"S")
    js = WORKLOAD_JSON
    spy = w["steps_per_year"]
    steps = len(orc.time_grid(js, spy)) - 1
    n = args.paths
    for i in range(args.warmup):
        orc.price(js, m, n_paths=n, seed=42 + 1000 + i, steps_per_year=spy, rate=w["r"])
    times = []
    for k in range(args.steps):
        t = time.perf_counter()
        orc.price(js, m, n_paths=n, seed=42 + 100 + k, steps_per_year=spy, rate=w["r"])
        times.append(time.perf_counter() - t)
    tot = sum(times)
    value = n * steps * args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox4x32-10 normals)",
        "config": _config(n, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": orc.threads(), "kind": "port",
                         "sample": f"the whole workload per step: {n} paths x {steps} steps, CPU restatement of "
                                   f"the reference pricer (materialised paths + recursive cash-flow walk), "
                                   f"OpenMP over paths; rank 0 only"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def price_greeks(c, m, n_paths, seed, spy) -> dict:
    """Price + delta/vega/rho of the workload: the pathwise adjoint (one reverse
    sweep per path, checkpoints every 16 steps, logistic barrier of the
    default width) against GPU CRN bump-and-reprice of the same smoothed
    payoff (seven reprices on the seed's normals as plain jobs of one lean
    launch, h = 1e-3 relative) and of the raw payoff.
    Equal standard error: the bump cost is scaled by the worst
    (SE_bump / SE_adjoint)^2 over the three Greeks (MC time ~ paths ~ SE^-2)."""
    import kontracts_gb300 as kx

    sim = {}

    def timed(fn, reps=3, key=None):
        best = None
        for _ in range(reps):
            out = fn()
            st = kx.last_launch_stats()
            t = (st["kernel_ms"] + st["reduce_ms"]) * 1e-3
            best = t if best is None or t < best else best
            if key:
                sim[key] = st["steps_simulated"]
        return out, best

    adj, t_adj = timed(lambda: c.adjoint(m, n_paths=n_paths, seed=seed, steps_per_year=spy, checkpoint_every=16))
    w = adj.smoothing_width
    bump, t_bump = timed(lambda: c.greeks(m, n_paths=n_paths, seed=seed, steps_per_year=spy,
                                          bumps=(1e-3, 1e-3, 1e-3), relative=True, smooth_width=w), key="smoothed")
    raw, t_raw = timed(lambda: c.greeks(m, n_paths=n_paths, seed=seed, steps_per_year=spy,
                                        bumps=(1e-3, 1e-3, 1e-3), relative=True), reps=1, key="raw")
    pairs = {"delta": (adj.d_s0, adj.se_s0, bump.delta, bump.delta_se, raw.delta, raw.delta_se),
             "vega": (adj.d_sigma, adj.se_sigma, bump.vega, bump.vega_se, raw.vega, raw.vega_se),
             "rho": (adj.d_r, adj.se_r, bump.rho, bump.rho_se, raw.rho, raw.rho_se)}
    se_scale = max((b_se / a_se) ** 2 for (_, a_se, _, b_se, _, _) in pairs.values())
    se_scale_raw = max((r_se / a_se) ** 2 for (_, a_se, _, _, _, r_se) in pairs.values())
    return {
        "workload": "same contract/model/paths as value; FP32 paths",
        "smoothing_width_logspot": w,
        "adjoint": {"seconds": t_adj, "price_greeks_per_s": 1.0 / t_adj, "price": adj.price,
                    **{k: v[0] for k, v in pairs.items()}, **{k + "_se": v[1] for k, v in pairs.items()}},
        "bump_smoothed": {"seconds": t_bump, "price_greeks_per_s": 1.0 / t_bump, "price": bump.price,
                          **{k: v[2] for k, v in pairs.items()}, **{k + "_se": v[3] for k, v in pairs.items()}},
        "bump_raw_payoff": {"seconds": t_raw, **{k: v[4] for k, v in pairs.items()},
                            **{k + "_se": v[5] for k, v in pairs.items()}},
        "rel_diff_adjoint_vs_bump": {k: abs(v[0] - v[2]) / max(abs(v[2]), 1e-12) for k, v in pairs.items()},
        "smoothed_over_raw_bump_time": t_bump / t_raw,
        # the smoothed payoff keeps paths alive past the barrier (their weight reaches exactly 0 only
        # far beyond it), so it simulates more steps; per simulated step the two bumps run alike
        "steps_simulated": {"bump_smoothed": sim.get("smoothed"), "bump_raw_payoff": sim.get("raw")},
        "smoothed_over_raw_time_per_simulated_step": (t_bump / sim["smoothed"]) / (t_raw / sim["raw"])
        if sim.get("smoothed") and sim.get("raw") else None,
        "equal_se_speedup_vs_bump_smoothed": t_bump * se_scale / t_adj,
        "equal_se_speedup_vs_bump_raw": t_raw * se_scale_raw / t_adj,
        "price_greeks_per_s_equal_se": {"adjoint": 1.0 / t_adj, "bump_smoothed": 1.0 / (t_bump * se_scale),
                                        "bump_raw_payoff": 1.0 / (t_raw * se_scale_raw)},
    }


def _dev_seconds(kx) -> float:
    st = kx.last_launch_stats()
    return (st["kernel_ms"] + st["reduce_ms"]) * 1e-3


_BARE = {}


def _bare_loop(what: int) -> float:
    """kx_measure_peak: 3 the bare Philox + Box-Muller + GBM step loop, 4 the
    Heston one (FP32 steps/s on this GPU, measured once per process)."""
    if what not in _BARE:
        import ctypes as C
        from kontracts_gb300 import _abi
        v = C.c_double()
        _BARE[what] = v.value if _abi.load().kx_measure_peak(what, C.byref(v)) == 0 else float("nan")
    return _BARE[what]


def _issue_roofline(sim_steps: float, kernel_s: float, what: int, unit_note: str) -> dict:
    """Simulated steps/s of the path kernel(s) against the bare step loop of the
    same model: the issue-bound roofline of the path kernels."""
    achieved = sim_steps / kernel_s / 1e9
    peak = _bare_loop(what) / 1e9
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gsteps/s",
            "frac": achieved / peak if peak == peak and peak > 0 else None,
            "peak_source": f"kx_measure_peak({what}) in this run", "note": unit_note}


def _hbm_peak() -> tuple:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"


def european_fp64(reps=5) -> dict:
    """Plain European call on GBM: s0 = K = 100, sigma 0.2, r 0.05, T 1, one
    step, 1,000,000 paths, FP64 paths, seed 42, against Black-Scholes
    (10.450583572185565)."""
    import kontracts_gb300 as kx
    c = kx.european_call("S", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.05, asset="S")
    best = None
    for _ in range(reps):
        r = c.price(m, n_paths=1_000_000, seed=42, steps_per_year=1, precision="fp64")
        t = _dev_seconds(kx)
        best = t if best is None or t < best else best
    bs = 10.450583572185565
    return {"workload": "European call, 1 step, 1M paths, FP64, seed 42", "seconds": best,
            "path_steps_per_s": 1_000_000 / best, "price": r.price, "std_error": r.std_error,
            "black_scholes": bs, "error_in_se": (r.price - bs) / r.std_error}


def variance_reduction(reps=3) -> dict:
    """The benchmark's up-and-out call (4,000,000 paths, daily grid, FP32)
    priced plain and with the reference's variance reduction (antithetic
    pairs, the at-the-money call as a control, both): device time, standard
    error, and the gain at equal standard error over plain pricing
    (time x SE^2, plain / mode)."""
    import kontracts_gb300 as kx
    c = kx.up_and_out_call("S", 100.0, 200.0, 1.0)
    m = kx.GBM(s0=180.0, sigma=0.25, r=0.05, asset="S")
    out = {"workload": "up-and-out call, s0 180, K 100, B 200, sigma 0.25, r 0.05, T 1, 365 steps/yr, 4M paths, FP32"}
    base = None
    for name, anti, cv in (("plain", False, False), ("antithetic", True, False), ("control_variate", False, True),
                           ("antithetic_control_variate", True, True)):
        best = None
        for _ in range(reps):
            r = c.price(m, n_paths=4_000_000, seed=42, steps_per_year=365, antithetic=anti, control_variate=cv)
            t = _dev_seconds(kx)
            best = t if best is None or t < best else best
        row = {"seconds": best, "price": r.price, "std_error": r.std_error, "n_paths": r.n_paths}
        if base is None:
            base = (best, r.std_error)
        else:
            row["equal_se_gain"] = (base[0] * base[1] ** 2) / (best * r.std_error ** 2)
        out[name] = row
    return out


def greek_surface_grid(reps=3, cpu_seconds=4.0) -> dict:
    """A trader's spot x vol surface (greek_surface, surface.rs:104-137):
    11 spots (80..120) x 9 vols (0.10..0.42) of an up-and-out call (K 100,
    B 130, T 1) on a daily grid (252 steps a year), 100,000 paths per cell,
    FP32 paths, default bumps (1e-2, 1e-2, 1e-4), seed 42. Each cell is seven
    CRN reprices; the 99 cells x 7 reprices run as one path launch. The
    oracle (the reference's cell loop restated, all host threads) prices a
    bounded sample of the same cells for the CPU rate. `adjoint`: the same
    grid by one pathwise-adjoint portfolio launch (no gamma), at equal
    standard error against the bump surface (median over cells of
    (SE_bump / SE_adjoint)^2, the worse of delta and vega)."""
    import kontracts_gb300 as kx
    from oracle import Oracle
    c = kx.up_and_out_call("S", 100.0, 130.0, 1.0)
    spots = [80.0 + 4.0 * i for i in range(11)]
    vols = [0.10 + 0.04 * j for j in range(9)]
    n, spy = 100_000, 252
    steps = len(c.time_grid(spy)) - 1
    best, launches, roof = None, 0, None
    for _ in range(reps):
        s = kx.greek_surface(c, "S", spots, vols, n_paths=n, seed=42, steps_per_year=spy, rate=0.05)
        t = _dev_seconds(kx)
        st = kx.last_launch_stats()
        launches = st["kernel_launches"]
        if best is None or t < best:
            best = t
            roof = _issue_roofline(st["steps_simulated"], st["kernel_ms"] * 1e-3, 3,
                                   "simulated scenario-steps of the 693 reprices (knocked-out paths stop)")
    t0 = time.perf_counter()
    kx.greek_surface(c, "S", spots, vols, n_paths=n, seed=42, steps_per_year=spy, rate=0.05)
    wall = time.perf_counter() - t0
    # the same grid as one pathwise-adjoint portfolio launch (delta / vega / rho of the smoothed payoff)
    best_a = None
    for _ in range(reps):
        a = kx.greek_surface(c, "S", spots, vols, n_paths=n, seed=42, steps_per_year=spy, rate=0.05,
                             method="adjoint")
        t = _dev_seconds(kx)
        best_a = t if best_a is None or t < best_a else best_a
    import numpy as np
    se_ratio = {q: float(np.median((getattr(s, q + "_se") / getattr(a, q + "_se")) ** 2)) for q in ("delta", "vega")}
    cells = len(spots) * len(vols)
    scen_steps = cells * 7 * n * steps
    # CPU: the oracle on a sample of cells and paths, scaled to cells/s at n paths
    orc = Oracle()
    pn = 20_000
    t0 = time.perf_counter()
    orc.greek_surface(c.to_json(), "S", spots[5:6], vols[3:4], n_paths=pn, seed=42, steps_per_year=spy, rate=0.05)
    dt = time.perf_counter() - t0
    k = max(1, min(cells, int(cpu_seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    orc.greek_surface(c.to_json(), "S", spots[:1], vols[:k] if k <= len(vols) else vols, n_paths=pn, seed=42,
                      steps_per_year=spy, rate=0.05)
    cdt = time.perf_counter() - t0
    kc = min(k, len(vols))
    cpu_cells_per_s = kc * pn / n / cdt
    return {"workload": "greek surface, 11 spots x 9 vols, up-and-out call K 100 B 130 T 1, 252 steps/yr, "
                        "100k paths per cell, FP32, default bumps", "cells": cells,
            "seconds": best, "wall_seconds_e2e": wall, "gpu_launches": launches,
            "cells_per_s": cells / best, "scenario_path_steps_per_s": scen_steps / best, "roofline": roof,
            "delta_atm_0.26": float(s.delta[5, 4]), "gamma_atm_0.26": float(s.gamma[5, 4]),
            "vega_atm_0.26": float(s.vega[5, 4]),
            "cpu_baseline": {"cells_per_s": cpu_cells_per_s, "cores": orc.threads(), "kind": "port",
                             "sample": f"{kc} cells x {pn} paths x {steps} steps x 7 reprices, {cdt:.2f} s"},
            "gpu_over_cpu_cells_per_s": cells / best / cpu_cells_per_s,
            "adjoint": {"seconds": best_a, "cells_per_s": cells / best_a,
                        "median_se2_ratio_bump_over_adjoint": se_ratio,
                        "equal_se_speedup_vs_bump": best * max(se_ratio.values()) / best_a,
                        "delta_atm_0.26": float(a.delta[5, 4]), "vega_atm_0.26": float(a.vega[5, 4])}}


def heston_calibration(cpu_seconds=6.0) -> dict:
    """calibrate_heston_cmaes (calibration.rs:441-465) as the reference tests
    it: three call quotes (spots 90 / 100 / 110, K 100, T 1, r 0.05) priced
    under (v0, kappa, theta, sigma_v, rho) = (0.04, 2, 0.04, 0.3, -0.5) on the
    calibration's own paths (3,000 paths, seed 42, 252 steps a year), 40
    generations of 40 candidates. Each generation's 120 Heston prices are one
    path launch. FP64 paths (the reference's precision) and FP32. CPU: the
    oracle's eval_obj_heston over one generation's population, all host
    threads, scaled to the 40 generations."""
    import numpy as np

    import kontracts_gb300 as kx
    from kontracts_gb300 import calibration as cal
    from oracle import Oracle
    c = kx.european_call("underlying", 100.0, 1.0)
    hp = [0.04, 2.0, 0.04, 0.3, -0.5]
    quotes = [(s, c.price(kx.heston(s, *hp, 0.05, asset="underlying"), n_paths=3000, seed=42, steps_per_year=252,
                          precision="fp64").price) for s in (90.0, 100.0, 110.0)]
    out = {"workload": "Heston CMA-ES calibration, 3 call quotes, 3000 paths x 252 steps, 40 generations x 40 "
                       "candidates (the reference's calibrate_heston_reproduces_prices)"}
    for prec in ("fp64", "fp32"):
        cfg = cal.FastCalibrationConfig(n_paths=3000, max_iterations=40, precision=prec)
        cal.calibrate_heston_cmaes(c, quotes, 0.05, cal.FastCalibrationConfig(n_paths=3000, max_iterations=2,
                                                                             precision=prec))  # tune + warm
        t0 = time.perf_counter()
        res = cal.calibrate_heston_cmaes(c, quotes, 0.05, cfg)
        wall = time.perf_counter() - t0
        err = max(abs(c.price(kx.heston(s, *res.parameters, 0.05, asset="underlying"), n_paths=3000, seed=42,
                              steps_per_year=252, precision="fp64").price - q) / q for s, q in quotes)
        out[prec] = {"wall_seconds": wall, "generations": res.iterations, "objective": res.objective,
                     "parameters": res.parameters, "max_rel_price_error": err,
                     "generations_per_s": res.iterations / wall}
    # the oracle on one generation (40 candidates x 3 quotes), repeated to ~cpu_seconds
    orc = Oracle()
    rng = np.random.default_rng(1)
    pop = [[float(rng.uniform(lo, hi)) for lo, hi in zip(cal.HESTON_LOWER, cal.HESTON_UPPER)] for _ in range(40)]
    t0 = time.perf_counter()
    k = 0
    while True:
        orc.calib_heston_objective(c.to_json(), "underlying", quotes, pop, n_paths=3000, steps_per_year=252,
                                   rate=0.05)
        k += 1
        if time.perf_counter() - t0 > cpu_seconds or k >= 40:
            break
    per_gen = (time.perf_counter() - t0) / k
    out["cpu_baseline"] = {"seconds_per_generation": per_gen, "generations_per_s": 1.0 / per_gen,
                           "cores": orc.threads(), "kind": "port",
                           "sample": f"{k} generations of 40 candidates x 3 quotes x 3000 paths x 252 steps"}
    out["gpu_fp64_over_cpu_generations_per_s"] = out["fp64"]["generations_per_s"] * per_gen
    return out


def mlmc_heston() -> dict:
    """price_mlmc_detailed (mlmc.rs:107-215) on a European call under Heston
    (s0 100, v0 0.04, kappa 1.5, theta 0.04, sigma_v 0.3, rho -0.7, r 0.05,
    T 1): 9 levels (2^0 .. 2^8 steps), 2,000 pilot paths, target standard
    error 0.005, seed 11; per phase one k_mlmc_pairs launch for the fine and
    coarse paths of all levels. Against the oracle (the reference's level loop restated, all
    host threads) on the same configuration, and against plain Monte Carlo on
    the GPU at the finest grid and the same standard error (the reference's
    mlmc_cheaper_than_standard_mc comparison)."""
    import kontracts_gb300 as kx
    from oracle import Oracle
    c = kx.european_call("S", 100.0, 1.0)
    h = kx.heston(100.0, 0.04, 1.5, 0.04, 0.3, -0.7, 0.05, asset="S")
    cfg = kx.MlmcConfig(n_levels=8, pilot_paths=2000, target_variance=0.005 ** 2)
    out = {"workload": "Heston call MLMC, levels 0..8, pilot 2000, target SE 0.005, seed 11"}
    for prec in ("fp64", "fp32"):
        kx.price_mlmc_detailed(c, h, kx.MlmcConfig(n_levels=8, pilot_paths=2000, target_variance=0.05 ** 2),
                               seed=11, precision=prec)  # tune + warm
        t0 = time.perf_counter()
        d = kx.price_mlmc_detailed(c, h, cfg, seed=11, precision=prec)
        wall = time.perf_counter() - t0
        if prec == "fp32":
            st = kx.last_launch_stats()
            out["roofline"] = _issue_roofline(st["steps_simulated"], st["kernel_ms"] * 1e-3, 4,
                                              "simulated Heston steps of both phases' fine and coarse launches")
        out[prec] = {"wall_seconds": wall, "price": d.price.price, "std_error": d.price.std_error,
                     "level_paths": d.level_paths, "total_cost_steps": d.total_cost,
                     "path_steps_per_s": d.total_cost / wall}
    orc = Oracle()
    t0 = time.perf_counter()
    r = orc.price_mlmc(c.to_json(), h, n_levels=8, pilot_paths=2000, target_variance=0.005 ** 2, seed=11)
    cpu = time.perf_counter() - t0
    out["cpu_baseline"] = {"wall_seconds": cpu, "price": r["price"].price, "cores": orc.threads(), "kind": "port",
                           "path_steps_per_s": r["total_cost"] / cpu, "sample": "the whole configuration"}
    out["gpu_fp64_vs_cpu_price_diff"] = out["fp64"]["price"] - r["price"].price
    out["gpu_fp64_over_cpu_wall"] = cpu / out["fp64"]["wall_seconds"]
    # plain Monte Carlo on the 2^8-step grid at the same standard error, on the GPU (FP64)
    pilot = c.price(h, n_paths=30_000, seed=99, steps_per_year=256, precision="fp64")
    n_std = int((pilot.sample_std / 0.005) ** 2) + 1
    t0 = time.perf_counter()
    std = c.price(h, n_paths=n_std, seed=99, steps_per_year=256, precision="fp64")
    t_std = time.perf_counter() - t0
    out["plain_mc_same_se_fp64"] = {"n_paths": n_std, "wall_seconds": t_std, "price": std.price,
                                    "std_error": std.std_error, "cost_steps": n_std * 256}
    out["mlmc_speedup_over_plain_mc_fp64"] = t_std / out["fp64"]["wall_seconds"]
    return out


def multi_asset_basket(reps=3) -> dict:
    """A knock-out basket call on 5 correlated GBM factors (CorrelatedGbmN,
    multi_asset.rs): s0 100, sigma 0.15..0.35, pairwise correlation 0.4, r
    0.03; payoff max(basket - 100, 0) at T 1 unless the equally weighted
    basket reaches 130 on the daily grid (252 steps); 1,000,000 paths, FP32
    and FP64. CPU: the oracle on a bounded sample."""
    import kontracts_gb300 as kx
    from oracle import Oracle
    S = kx.S
    n_f = 5
    fac = [(f"S{i}", 100.0, 0.03, 0.15 + 0.05 * i) for i in range(n_f)]
    corr = [[1.0 if i == j else 0.4 for j in range(n_f)] for i in range(n_f)]
    m = kx.CorrelatedGbmN(fac, corr, rate=0.03)
    basket = (S("S0") + S("S1") + S("S2") + S("S3") + S("S4")) / 5.0
    c = kx.until(basket >= 130.0, kx.scale((basket - 100.0).clip(0.0), kx.one()) @ kx.at(1.0))
    n, spy = 1_000_000, 252
    steps = len(c.time_grid(spy)) - 1
    out = {"workload": "knock-out basket call, 5 correlated GBM factors, daily grid, 1M paths"}
    for prec in ("fp32", "fp64"):
        c.price(m, n_paths=n, seed=42, steps_per_year=spy, precision=prec)  # tune + warm
        best = None
        for _ in range(reps):
            r = c.price(m, n_paths=n, seed=42, steps_per_year=spy, precision=prec)
            t = _dev_seconds(kx)
            best = t if best is None or t < best else best
        st = kx.last_launch_stats()
        sim = st["steps_simulated"]
        if prec == "fp32":
            out["roofline"] = _issue_roofline(sim * n_f, st["kernel_ms"] * 1e-3, 3,
                                              "factor-steps (each one normal and one GBM step, as the bare loop) "
                                              "of the last run")
        out[prec] = {"seconds": best, "price": r.price, "std_error": r.std_error,
                     "nominal_path_steps_per_s": n * steps / best, "simulated_path_steps_per_s": sim / best,
                     "factor_steps_per_s": sim * n_f / best}
    orc = Oracle()
    ns = 200_000
    t0 = time.perf_counter()
    o = orc.price_multi(c.to_json(), m, n_paths=ns, seed=42, steps_per_year=spy)
    cpu = time.perf_counter() - t0
    out["cpu_baseline"] = {"nominal_path_steps_per_s": ns * steps / cpu, "cores": orc.threads(), "kind": "port",
                           "sample": f"{ns} paths x {steps} steps, {cpu:.2f} s", "price": o.price}
    out["gpu_fp32_over_cpu"] = out["fp32"]["nominal_path_steps_per_s"] / out["cpu_baseline"]["nominal_path_steps_per_s"]
    return out


def heston_book(reps=3) -> dict:
    """Heston benchmark shape: 32 strikes (evenly spaced in [80, 120]) x T in
    {0.5, 1, 2}, full truncation, 252 steps a year, 2,000,000 paths, FP32, all
    96 contracts on one shared simulation (price_batch); plus the pathwise
    adjoint sensitivities (s0, v0, kappa, theta, sigma_v, rho) of the T = 1,
    K = 100 call with a checkpoint every 16 steps, of all 96 calls each on its
    own paths (portfolio adjoint), and of all 96 calls on the book's shared
    simulation (tangent mode)."""
    import kontracts_gb300 as kx
    h = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="S", scheme="full_truncation")
    ks = [80.0 + 40.0 * i / 31 for i in range(32)]
    book = [kx.european_call("S", k, t) for t in (0.5, 1.0, 2.0) for k in ks]
    n = 2_000_000
    best = None
    for _ in range(reps):
        res = kx.price_batch(book, h, n_paths=n, seed=42, steps_per_year=252)
        t = _dev_seconds(kx)
        best = t if best is None or t < best else best
    steps = n * 504
    # roofline: the simulation's steps/s against the bare Heston loop (Philox, Box-Muller, the
    # full-truncation step; kx_measure_peak(4)) measured in the same process
    import ctypes as C
    from kontracts_gb300 import _abi
    pk = C.c_double()
    peak = pk.value if _abi.load().kx_measure_peak(4, C.byref(pk)) == 0 else float("nan")
    adj = None
    for _ in range(2):
        a = kx.european_call("S", 100.0, 1.0).adjoint(h, n_paths=n, seed=7, steps_per_year=252, checkpoint_every=16)
        ta = _dev_seconds(kx)
        adj = (a, ta) if adj is None or ta < adj[1] else adj
    a, ta = adj
    # the whole book: price and the seven Heston sensitivities of every contract by one portfolio
    # adjoint launch, each contract on its own 1M paths
    nb = 1_000_000
    tb = None
    for _ in range(2):
        _, sens = kx.price_portfolio(book, [h] * len(book), [nb] * len(book), list(range(len(book))),
                                     steps_per_year=252, greeks=True)
        t = _dev_seconds(kx)
        tb = t if tb is None or t < tb else tb
    book_adj = {"workload": "price + (s0, v0, kappa, theta, sigma_v, rho, r) sensitivities of all 96 calls, "
                            "one portfolio adjoint launch, 1M paths per contract, FP32",
                "seconds": tb, "contracts_per_s": len(book) / tb,
                "path_steps_per_s": sum(nb * (len(c.time_grid(252)) - 1) for c in book) / tb,
                "d_s0_T1_K100": sens[32 + 15].d_s0, "d_v0_T1_K100": sens[32 + 15].d_v0}
    # the same price + sensitivities of all 96 calls on the book's one shared 2M-path simulation
    # (kx_price_batch_sens: the tangents of y and v carried forward, one pass for the whole book)
    ts = None
    for _ in range(reps):
        res_s, sens_s = kx.price_batch(book, h, n_paths=n, seed=42, steps_per_year=252, greeks=True)
        t = _dev_seconds(kx)
        ts = t if ts is None or t < ts else ts
    book_sens = {"workload": "price + (s0, v0, kappa, theta, sigma_v, rho, r) sensitivities of all 96 calls on the "
                             "book's shared 2M-path simulation (kx_price_batch_sens, tangent mode), FP32",
                 "seconds": ts, "contracts_per_s": len(book) / ts, "over_price_only": ts / best,
                 "prices_equal_price_batch": all(a_.price == b_.price for a_, b_ in zip(res_s, res)),
                 "d_s0_T1_K100": sens_s[32 + 15].d_s0, "d_v0_T1_K100": sens_s[32 + 15].d_v0,
                 "d_kappa_T1_K100": sens_s[32 + 15].d_kappa, "se_v0_T1_K100": sens_s[32 + 15].se_v0}
    return {"workload": "96 Heston calls (32 strikes x 3 maturities) on one 2M-path simulation, full truncation, "
                        "252 steps/yr, FP32", "seconds": best, "path_steps_per_s": steps / best,
            "contracts_per_s": len(book) / best, "price_T1_K100": res[32 + 15].price,
            "roofline": {"bound": "issue", "achieved": steps / best / 1e9, "peak": peak / 1e9, "unit": "Gsteps/s",
                         "frac": steps / best / peak if peak == peak and peak > 0 else None,
                         "peak_source": "measured in this run: kx_measure_peak(4), the bare Philox4x32-10 + "
                                        "Box-Muller + Heston full-truncation step loop",
                         "note": "time includes the 96 payoffs on the shared simulation"},
            "adjoint_T1_K100": {"seconds": ta, "price": a.price, "d_s0": a.d_s0, "d_v0": a.d_v0,
                                "d_kappa": a.d_kappa, "d_theta": a.d_theta, "d_sigma_v": a.d_sigma_v,
                                "d_rho": a.d_rho, "se_v0": a.se_v0, "checkpoint_every": 16},
            "adjoint_book_96": book_adj, "sens_book_96_shared": book_sens}


def book_256(reps=5) -> dict:
    """The 256-contract book (tests/golden/portfolio_256.json: seeded 50/30/20
    European / up-and-out / arithmetic-Asian calls, uneven paths and steps):
    (1) prices by replaying the book's CUDA graph; (2) price + delta + vega of
    every contract by the pathwise adjoint (one launch) against GPU CRN
    bump-and-reprice of the same smoothed payoffs (h = 1e-3 relative), the
    bump cost scaled to the adjoint's standard errors (time ~ SE^-2), per
    contract by its worse Greek."""
    import kontracts_gb300 as kx
    fx = json.load(open(os.path.join(ROOT, "tests", "golden", "portfolio_256.json")))["contracts"]
    cs = [kx.Contract.from_json(c["json"]) for c in fx]
    ms = [kx.GBM(s0=c["s0"], sigma=c["sigma"], r=c["r"], asset="S") for c in fx]
    ns = [int(c["n_paths"]) for c in fx]
    seeds = [int(c["seed"]) for c in fx]
    t0 = time.perf_counter()
    book = kx.Book(cs, ms, ns, seeds, steps_per_year=252, tune=True)
    create_s = time.perf_counter() - t0
    info = book.info()
    best = None
    for _ in range(reps):
        book.price()
        t = kx.last_launch_stats()["kernel_ms"] * 1e-3
        best = t if best is None or t < best else best
    t0 = time.perf_counter()
    for _ in range(reps):
        book.price()
    e2e = (time.perf_counter() - t0) / reps
    out = {"workload": "256-contract book, FP32 paths, 252 steps/yr", "n_paths": info["n_paths"],
           "path_steps": info["path_steps"], "book_create_s": create_s, "tuning": info,
           "graph_seconds": best, "path_steps_per_s": info["path_steps"] / best, "contracts_per_s": 256 / best,
           "e2e_seconds": e2e, "e2e_contracts_per_s": 256 / e2e}
    book.close()
    # steps the price simulates (knocked-out paths stop) against the sensitivities' (smoothed
    # barriers never knock out; every step once for the forward-mode kernel, twice for a reverse
    # sweep: the forward pass and the recomputation of each segment)
    kx.price_portfolio(cs, ms, ns, seeds, steps_per_year=252)
    sim_price = kx.last_launch_stats()["steps_simulated"]
    # price + delta + vega: adjoint (one launch per kernel group) vs CRN bump per contract
    _, sens = kx.price_portfolio(cs, ms, ns, seeds, steps_per_year=252, greeks=True)
    t_adj = _dev_seconds(kx)
    sim_adj = kx.last_launch_stats()["steps_simulated"]
    out["steps_simulated"] = {"price": sim_price, "adjoint": sim_adj}
    out["adjoint_over_graph_time_per_simulated_step"] = (t_adj / sim_adj) / (best / sim_price)
    by_kind = {}
    for kind in sorted({c["kind"] for c in fx}):
        ix = [i for i, c in enumerate(fx) if c["kind"] == kind]
        kx.price_portfolio([cs[i] for i in ix], [ms[i] for i in ix], [ns[i] for i in ix], [seeds[i] for i in ix],
                           steps_per_year=252, greeks=True)
        by_kind[kind] = {"contracts": len(ix), "adjoint_seconds": _dev_seconds(kx)}
    t_bump_eq, t_bump, worst = 0.0, 0.0, []
    t_raw = 0.0
    for c, m, n, sd, g in zip(cs, ms, ns, seeds, sens):
        b = c.greeks(m, n_paths=n, seed=sd, steps_per_year=252, bumps=(1e-3, 1e-3, 1e-3), relative=True,
                     smooth_width=g.smoothing_width)
        tb = _dev_seconds(kx)
        scale = max((b.delta_se / max(g.se_s0, 1e-300)) ** 2, (b.vega_se / max(g.se_sigma, 1e-300)) ** 2)
        t_bump += tb
        t_bump_eq += tb * scale
        worst.append(max(abs(g.d_s0 - b.delta) / max(abs(b.delta), 1e-8), abs(g.d_sigma - b.vega) / max(abs(b.vega), 1e-8)))
        c.greeks(m, n_paths=n, seed=sd, steps_per_year=252, bumps=(1e-3, 1e-3, 1e-3), relative=True)
        t_raw += _dev_seconds(kx)
    # accuracy of the adjoint against CRN differences of the same smoothed payoff: FP64 paths,
    # 20,000 per contract, bumps of 1e-6 relative (no FP32 noise, negligible truncation)
    _, s64 = kx.price_portfolio(cs, ms, [20_000] * len(cs), seeds, steps_per_year=252, precision="fp64", greeks=True)
    acc = []
    for c, m, sd, g in zip(cs, ms, seeds, s64):
        b = c.greeks(m, n_paths=20_000, seed=sd, steps_per_year=252, bumps=(1e-6, 1e-6, 1e-6), relative=True,
                     smooth_width=g.smoothing_width, precision="fp64")
        acc += [abs(g.d_s0 - b.delta) / max(abs(b.delta), 1e-8), abs(g.d_sigma - b.vega) / max(abs(b.vega), 1e-8)]
    out["price_delta_vega"] = {"adjoint_seconds": t_adj, "bump_seconds": t_bump, "bump_seconds_equal_se": t_bump_eq,
                               "raw_payoff_bump_seconds": t_raw, "smoothed_over_raw_bump_time": t_bump / t_raw,
                               "equal_se_speedup": t_bump_eq / t_adj,
                               "adjoint_over_graph_price": t_adj / best,
                               "adjoint_by_kind": by_kind,
                               "fp32_h1e-3_median_rel_diff_adjoint_vs_bump": sorted(worst)[len(worst) // 2],
                               "fp64_h1e-6_max_rel_diff_adjoint_vs_bump": max(acc),
                               "fp64_h1e-6_median_rel_diff_adjoint_vs_bump": sorted(acc)[len(acc) // 2],
                               "rel_diff_note": "timing pair: FP32 paths, bumps 1e-3 relative (the FP32 noise and the "
                                                "truncation of such bumps dominate near-zero Greeks); accuracy pair: "
                                                "FP64, 20,000 paths per contract, bumps 1e-6, over all 512 Greeks"}
    return out


def lsm_cases(reps=2) -> dict:
    """American puts by Longstaff-Schwartz: s0 in {36, 40, 44}, K = 40,
    sigma in {0.2, 0.4}, r = 0.06, T in {1, 2}, 50 dates a year, 1,000,000
    paths stored FP32, 4 weighted-Laguerre functions. HBM roofline: bytes per
    path and date = 4 (forward store of S) + 16 (backward: read S at the
    decision and regression dates, read and write the FP32 value), plus 8 per
    path for the FP64 per-path result."""
    import kontracts_gb300 as kx
    peak, src = _hbm_peak()
    n = 1_000_000
    cases, tot_s, tot_bytes, batch = [], 0.0, 0.0, []
    for s0 in (36.0, 40.0, 44.0):
        for sig in (0.2, 0.4):
            for t in (1.0, 2.0):
                nd = int(50 * t)
                ds = [t * i / nd for i in range(1, nd + 1)]
                put = kx.scale((kx.const_(40.0) - kx.S("S")).clip(0.0), kx.one())
                m = kx.GBM(s0=s0, sigma=sig, r=0.06, asset="S")
                batch.append((put, m, ds, n, 42))
                best = None
                for _ in range(reps):
                    r = put.price_american(m, ds, n_paths=n, seed=42, n_basis=4, basis="laguerre")
                    st = kx.last_launch_stats()
                    ts = st["kernel_ms"] * 1e-3
                    best = ts if best is None or ts < best else best
                byts = n * (4.0 * nd + 16.0 * nd + 8.0)
                cases.append({"s0": s0, "sigma": sig, "T": t, "price": r.price, "se": r.std_error, "seconds": best,
                              "hbm_gbs": byts / best / 1e9})
                tot_s += best
                tot_bytes += byts
    # the same 12 problems in one batched call (one backward launch per date for all of them)
    bt, same = None, True
    for _ in range(reps):
        res = kx.price_american_batch(batch, n_basis=4, basis="laguerre")
        ts = kx.last_launch_stats()["kernel_ms"] * 1e-3
        bt = ts if bt is None or ts < bt else bt
    same = all(r.price == c["price"] and r.std_error == c["se"] for r, c in zip(res, cases))
    ach = tot_bytes / bt / 1e9
    return {"workload": "12 LSM American puts, 1M paths FP32 in HBM, 4 weighted-Laguerre functions",
            "seconds_total_single_calls": tot_s, "seconds_total_batched": bt, "batched_equals_single": same,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "peak_source": src, "timed": "batched call"},
            "cases": cases}


def run_ours(args, ws, rank, local) -> None:
    import torch

    import kontracts_gb300 as kx
    from kontracts_gb300 import _abi
    import ctypes as C

    lib = _abi.load()
    w = WORKLOAD
    n_paths = args.paths
    c = kx.up_and_out_call("S", w["strike"], w["barrier"], w["maturity"])
    m = kx.GBM(s0=w["s0"], sigma=w["sigma"], r=w["r"], asset="S")
    steps_per_path = len(c.time_grid(w["steps_per_year"])) - 1
    if args.scaling == "strong":
        # one price of n_paths paths over the ranks: each prices its chunk-aligned range of the
        # same stream, the chunk statistics are gathered and merged (the single-GPU result)
        from kontracts_gb300 import sharded
        seed = 42
        price = lambda s: sharded.price_sharded(c, m, n_paths, seed=s, steps_per_year=w["steps_per_year"],
                                                precision="fp32")
        job_paths = n_paths
    else:
        seed = 42 + 1000003 * rank
        price = lambda s: c.price(m, n_paths=n_paths, seed=s, steps_per_year=w["steps_per_year"],
                                  precision="fp32")
        job_paths = ws * n_paths
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    for i in range(args.warmup):
        r = price(seed + i)
    peaks = {}
    for what, name in ((0, "mufu"), (1, "fp32_fma"), (2, "imad_hi"), (3, "bare_path_steps"),
                       (4, "bare_heston_steps")):
        v = C.c_double()
        if lib.kx_measure_peak(what, C.byref(v)) == 0:
            peaks[name] = v.value
    # ---- timed region: device time of each call, L2 flushed in between ----
    clocks = Clocks(local)
    _barrier(ws)
    torch.cuda.synchronize()
    dev_ms, ker_ms, sim_steps, launches, rank_steps = 0.0, 0.0, 0, 0, 0
    results = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r = price(seed + 100 + k)
        st = kx.last_launch_stats()
        dev_ms += st["kernel_ms"] + st["reduce_ms"]
        ker_ms += st["kernel_ms"]
        sim_steps += st["steps_simulated"]
        rank_steps += st["path_steps"]  # this rank's nominal path-steps
        launches += st["kernel_launches"]
        results.append(r)
    torch.cuda.synchronize()
    _barrier(ws)
    clk = clocks.stop()
    dev_ms_max = _barrier_max(dev_ms, ws)
    nominal = job_paths * steps_per_path  # all ranks' path-steps of one step
    value = nominal * args.steps / (dev_ms_max * 1e-3)
    # ---- e2e: the C-ABI call from the host, wall clock ----
    _barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for k in range(args.steps):
        price(seed + 500 + k)
        st = kx.last_launch_stats()
        h2d += st["h2d_bytes"]
        d2h += st["d2h_bytes"]
    e2e_s = _barrier_max(time.perf_counter() - t0, ws)
    e2e = {"value": nominal * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
           "ms_per_step": 1e3 * e2e_s / args.steps}
    # ---- roofline of the path kernel: simulated steps/s against the bare simulation loop ----
    achieved = sim_steps / (ker_ms * 1e-3) / 1e9
    peak = peaks.get("bare_path_steps", float("nan")) / 1e9
    # DRAM bytes per launch: ncu's dram__bytes_read.sum + dram__bytes_write.sum of the path kernel
    # on the 1M-path case (profiles/k_lean_static_up_and_out.md: 23,296 + 0 bytes), scaled by the
    # number of paths; the per-path values (8 B/path) stay in L2 during the launch.
    rank_paths = rank_steps // max(1, steps_per_path * args.steps)  # paths of one launch on this rank
    traffic = 23296.0 / 1_000_000 * rank_paths
    kname = {1: "k_paths<float,GBM>", 2: "k_lean<float,GBM>", 3: "k_lean<float,GBM,static schedule>"}.get(
        kx.last_launch_stats()["path_kernel"], "?")
    roofline = {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gsteps/s",
                "frac": achieved / peak if peak == peak and peak > 0 else None, "traffic": traffic,
                "peak_source": "measured in this run: kx_measure_peak(3), the bare Philox4x32-10 + Box-Muller "
                               "+ GBM step loop (no contract, no scheduling) on this GPU",
                "kernel": kname, "algorithmic_bytes_per_path": 8,
                "achieved_hbm_gbs": 8.0 * rank_paths * args.steps / (ker_ms * 1e-3) / 1e9,
                "steps_simulated_fraction": sim_steps / max(1, rank_steps),
                "mufu_results_per_s_share": 2.0 * sim_steps / (ker_ms * 1e-3) / peaks.get("mufu", float("nan")),
                "measured_peaks_per_s": dict(peaks)}
    # the per-pipe form of the same roofline: frozen algorithmic ops per simulated step (2 MUFU
    # results, 5 32x32 high multiplies of Philox, 7 FP32 operations) over each pipe's peak measured
    # in this run; the binding pipe's share is the fraction
    rate = sim_steps / (ker_ms * 1e-3)
    shares = {"xu": 2.0 * rate / peaks.get("mufu", float("nan")),
              "imad_hi": 5.0 * rate / peaks.get("imad_hi", float("nan")),
              "fp32": 7.0 * rate / peaks.get("fp32_fma", float("nan"))}
    roofline["pipe_shares"] = shares
    roofline["pipe_bound"] = max(shares, key=lambda k: shares[k] if shares[k] == shares[k] else -1.0)
    roofline["bare_loop_pipe_shares"] = {
        "xu": 2.0 * peaks.get("bare_path_steps", float("nan")) / peaks.get("mufu", float("nan")),
        "imad_hi": 5.0 * peaks.get("bare_path_steps", float("nan")) / peaks.get("imad_hi", float("nan")),
        "fp32": 7.0 * peaks.get("bare_path_steps", float("nan")) / peaks.get("fp32_fma", float("nan"))}
    greeks = None if args.no_greeks else price_greeks(c, m, n_paths, seed, w["steps_per_year"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": args.scaling,
        "vs_baseline": None,
        "dtype": "f32 paths / f64 sums", "data": "synthetic (Philox4x32-10 normals generated in registers)",
        "config": _config(n_paths, ws),
        "price": results[-1].price, "std_error": results[-1].std_error,
        "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
    }
    if greeks is not None:
        line["price_greeks"] = greeks
    if rank == 0 and not args.no_extra:
        line["other_configs"] = {"european_fp64": european_fp64(), "heston_book_96": heston_book(),
                                 "book_256": book_256(), "lsm_12": lsm_cases(),
                                 "variance_reduction": variance_reduction(),
                                 "greek_surface_99": greek_surface_grid(),
                                 "heston_calibration": heston_calibration(), "mlmc_heston": mlmc_heston(),
                                 "multi_asset_basket": multi_asset_basket()}
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.cpu_seconds)
        line["accuracy"] = accuracy(cb)
        line["cpu_baseline"] = {k: v for k, v in cb.items() if not k.startswith("_")}
    if rank == 0:
        print(json.dumps(line), flush=True)


def _launch(n: int) -> int:
    """Start n ranks of this command under torch.distributed.run (one node,
    rendezvous on 127.0.0.1); rank 0 prints the line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def _pin_device(local: int) -> None:
    """Give rank `local` its own GPU: the library prices on device 0 of the
    process, so the rank sees only the local-th device of the visible list."""
    vis = [x.strip() for x in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if x.strip()]
    os.environ["CUDA_VISIBLE_DEVICES"] = vis[local % len(vis)] if vis else str(local)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--paths", type=int, default=WORKLOAD["n_paths"],
                    help="paths per rank (weak scaling) or in all (strong)")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="weak: every rank prices its own batch; strong: one price split over the ranks "
                         "(chunk statistics gathered, the single-GPU result)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-greeks", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the Heston book, 256-contract book and LSM lines")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = _dist()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(_launch(args.gpus))
    if ws > 1:
        _pin_device(local)
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        lib = os.path.join(ROOT, "kontracts_gb300", "libkontract_gpu.so")
        if not os.path.exists(lib):
            import __graft_entry__
            __graft_entry__.build()
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
