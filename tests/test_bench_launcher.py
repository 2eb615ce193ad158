"""bench.py's multi-rank launcher on the CPU: `--gpus 2` starts two ranks
under torch.distributed.run (gloo rendezvous on 127.0.0.1); with the CPU arm
(`--impl reference`) rank 0 alone prices and prints one JSON line that names
both ranks, and the arm runs the configuration the GPU arm runs."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args: str) -> list[dict]:
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    env.setdefault("OMP_NUM_THREADS", "2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_two_rank_launch_prints_one_line():
    lines = _bench("--gpus", "2", "--impl", "reference", "--steps", "1", "--warmup", "3", "--paths", "20000")
    assert len(lines) == 1, lines
    ln = lines[0]
    assert ln["impl"] == "reference" and ln["n_gpus"] == 2
    assert ln["config"]["n_paths"] == 20000 and ln["steps"] == 1 and ln["warmup"] == 3
    assert ln["value"] > 0 and ln["e2e"]["value"] == ln["value"]
    assert ln["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_no_engine_code():
    # the CPU arm prices through the oracle alone: no engine package, no engine library
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', "
            "'--paths', '5000']; runpy.run_path('bench.py', run_name='__main__'); "
            "import os; maps = open('/proc/self/maps').read(); "
            "assert 'libkontract_gpu' not in maps, 'engine library loaded'; "
            "assert not any(m == 'kontracts_gb300' or m.startswith('kontracts_gb300.') for m in sys.modules), "
            "'engine package imported'")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    ln = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][0])
    assert ln["n_gpus"] == 1 and ln["config"]["n_paths"] == 5000
