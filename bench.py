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
Multi-GPU (torchrun, N > 1): every rank prices its own batch on its own GPU
with its own Philox stream (weak scaling, no collective on the data path);
value = all ranks' path-steps / the slowest rank's time.
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
    orc.price(js, m, n_paths=n, seed=42, steps_per_year=w["steps_per_year"])
    dt = time.perf_counter() - t
    return {"value": n * steps / dt, "unit": UNIT, "cores": orc.threads(), "kind": "port",
            "sample": f"{n} of {w['n_paths']} paths x {steps} steps, CPU restatement of the reference "
                      f"pricer (materialised paths + recursive cash-flow walk), {dt:.2f} s"}


def run_reference(args, ws, rank) -> None:
    if rank != 0:
        return
    import kontracts_gb300 as kx
    from oracle import Oracle
    orc = Oracle()
    w = WORKLOAD
    c = kx.up_and_out_call("S", w["strike"], w["barrier"], w["maturity"])
    m = kx.GBM(s0=w["s0"], sigma=w["sigma"], r=w["r"], asset="S")
    js = c.to_json()
    steps = len(c.time_grid(w["steps_per_year"])) - 1
    n = args.ref_paths
    for _ in range(args.warmup):
        orc.price(js, m, n_paths=max(1000, n // 10), seed=42, steps_per_year=w["steps_per_year"])
    times = []
    for k in range(args.steps):
        t = time.perf_counter()
        orc.price(js, m, n_paths=n, seed=42 + k, steps_per_year=w["steps_per_year"])
        times.append(time.perf_counter() - t)
    tot = sum(times)
    value = n * steps * args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox normals)",
        "config": dict(WORKLOAD, sample_paths=n),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": orc.threads(), "kind": "port",
                         "sample": f"{n} of {w['n_paths']} paths x {steps} steps per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def price_greeks(c, m, n_paths, seed, spy) -> dict:
    """Price + delta/vega/rho of the workload: the pathwise adjoint (one reverse
    sweep per path, checkpoints every 16 steps, logistic barrier of the
    default width) against GPU CRN bump-and-reprice of the same smoothed
    payoff (seven scenarios sharing each path's normals, h = 1e-3 relative).
    Equal standard error: the bump cost is scaled by the worst
    (SE_bump / SE_adjoint)^2 over the three Greeks (MC time ~ paths ~ SE^-2)."""
    import kontracts_gb300 as kx

    def timed(fn, reps=3):
        best = None
        for _ in range(reps):
            out = fn()
            st = kx.last_launch_stats()
            t = (st["kernel_ms"] + st["reduce_ms"]) * 1e-3
            best = t if best is None or t < best else best
        return out, best

    adj, t_adj = timed(lambda: c.adjoint(m, n_paths=n_paths, seed=seed, steps_per_year=spy, checkpoint_every=16))
    w = adj.smoothing_width
    bump, t_bump = timed(lambda: c.greeks(m, n_paths=n_paths, seed=seed, steps_per_year=spy,
                                          bumps=(1e-3, 1e-3, 1e-3), relative=True, smooth_width=w))
    raw, t_raw = timed(lambda: c.greeks(m, n_paths=n_paths, seed=seed, steps_per_year=spy,
                                        bumps=(1e-3, 1e-3, 1e-3), relative=True), reps=1)
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
        "equal_se_speedup_vs_bump_smoothed": t_bump * se_scale / t_adj,
        "equal_se_speedup_vs_bump_raw": t_raw * se_scale_raw / t_adj,
        "price_greeks_per_s_equal_se": {"adjoint": 1.0 / t_adj, "bump_smoothed": 1.0 / (t_bump * se_scale),
                                        "bump_raw_payoff": 1.0 / (t_raw * se_scale_raw)},
    }


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
    seed = 42 + 1000003 * rank
    steps_per_path = len(c.time_grid(w["steps_per_year"])) - 1
    price = lambda s: c.price(m, n_paths=n_paths, seed=s, steps_per_year=w["steps_per_year"], precision="fp32")
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    for i in range(args.warmup):
        r = price(seed + i)
    peaks = {}
    for what, name in ((0, "mufu"), (1, "fp32_fma"), (2, "imad_hi"), (3, "bare_path_steps")):
        v = C.c_double()
        if lib.kx_measure_peak(what, C.byref(v)) == 0:
            peaks[name] = v.value
    # ---- timed region: device time of each call, L2 flushed in between ----
    clocks = Clocks(local)
    _barrier(ws)
    torch.cuda.synchronize()
    dev_ms, ker_ms, sim_steps, launches = 0.0, 0.0, 0, 0
    results = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        r = price(seed + 100 + k)
        st = kx.last_launch_stats()
        dev_ms += st["kernel_ms"] + st["reduce_ms"]
        ker_ms += st["kernel_ms"]
        sim_steps += st["steps_simulated"]
        launches += st["kernel_launches"]
        results.append(r)
    torch.cuda.synchronize()
    _barrier(ws)
    clk = clocks.stop()
    dev_ms_max = _barrier_max(dev_ms, ws)
    nominal = n_paths * steps_per_path
    value = ws * nominal * args.steps / (dev_ms_max * 1e-3)
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
    e2e = {"value": ws * nominal * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
           "ms_per_step": 1e3 * e2e_s / args.steps}
    # ---- roofline of the path kernel: simulated steps/s against the bare simulation loop ----
    achieved = sim_steps / (ker_ms * 1e-3) / 1e9
    peak = peaks.get("bare_path_steps", float("nan")) / 1e9
    prof = os.path.join(ROOT, "profiles", "k_lean_up_and_out_traffic.json")
    traffic = None
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("dram_bytes_per_launch_full_workload")
        except Exception:
            traffic = None
    kname = {1: "k_paths<float,GBM>", 2: "k_lean<float,GBM>"}.get(kx.last_launch_stats()["path_kernel"], "?")
    roofline = {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Gsteps/s",
                "frac": achieved / peak if peak == peak and peak > 0 else None, "traffic": traffic,
                "peak_source": "measured in this run: kx_measure_peak(3), the bare Philox4x32-10 + Box-Muller "
                               "+ GBM step loop (no contract, no scheduling) on this GPU",
                "kernel": kname, "algorithmic_bytes_per_path": 8,
                "achieved_hbm_gbs": 8.0 * n_paths * args.steps / (ker_ms * 1e-3) / 1e9,
                "steps_simulated_fraction": sim_steps / (nominal * args.steps),
                "mufu_results_per_s_share": 2.0 * sim_steps / (ker_ms * 1e-3) / peaks.get("mufu", float("nan")),
                "measured_peaks_per_s": dict(peaks)}
    greeks = None if args.no_greeks else price_greeks(c, m, n_paths, seed, w["steps_per_year"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 paths / f64 sums", "data": "synthetic (Philox4x32-10 normals generated in registers)",
        "config": dict(WORKLOAD, n_paths=n_paths, l2="flushed between timed steps (256 MB write)",
                       parallelism=f"paths sharded over {ws} GPU(s), no collective"),
        "price": results[-1].price, "std_error": results[-1].std_error,
        "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
    }
    if greeks is not None:
        line["price_greeks"] = greeks
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--paths", type=int, default=WORKLOAD["n_paths"])
    ap.add_argument("--ref-paths", type=int, default=400_000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-greeks", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = _dist()
    if ws > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
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
