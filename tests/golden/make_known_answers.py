"""Writes tests/golden/known_answers.json: the known-answer values the
reference's own tests pin for the pricing path, with the file:line each comes
from, and the serde JSON wire format of the contracts those tests build.

The reference crate cannot be built here (no Rust toolchain), so nothing is
executed: every number below is read from the reference's test sources and
every JSON string is the serde externally-tagged encoding of the AST of
src/ast.rs:34-206 for the contract the cited test constructs (f64 written in
serde_json/ryu form, e.g. 1.0, 0.5). Run: python tests/golden/make_known_answers.py
"""
import json
import math
import os

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")


def call(asset, k, t):  # tests/compiler.rs:10-15 and friends
    return ('{"When":[{"At":%s},{"Scale":[{"Max":[{"Sub":[{"Spot":"%s"},{"Const":%s}]},{"Const":0.0}]},'
            '{"One":"USD"}]}]}' % (t, asset, k))


UO = '{"Until":[{"Ge":[{"Spot":"AAPL"},{"Const":200.0}]},%s]}' % call("AAPL", "150.0", "1.0")

known = {
    "source": "LePhilippeDucTai/kontracts tests (read as text)",
    "z95": {"value": 1.959963984540054, "ref": "src/pricer.rs:74"},
    "bs_call_atm": {"s0": 100.0, "k": 100.0, "sigma": 0.2, "r": 0.05, "t": 1.0,
                    "value": 10.450583572185565, "ref": "tests/diagnostics.rs:64"},
    # sigma = 0 exact prices (tests/pricer.rs:58-106; model Gbm("AAPL", 100, 0.05, 0); cfg n=16, seed 1, spy 4)
    "sigma_zero": [
        {"json": '"Zero"', "rate": 0.05, "price": 0.0, "tol": 0.0, "ref": "tests/pricer.rs:58-62"},
        {"json": '{"One":"USD"}', "rate": 0.05, "price": 1.0, "tol": 1e-12, "ref": "tests/pricer.rs:64-68"},
        {"json": '{"Give":{"One":"USD"}}', "rate": 0.05, "price": -1.0, "tol": 1e-12, "ref": "tests/pricer.rs:70-74"},
        {"json": '{"And":[{"One":"USD"},{"And":[{"One":"USD"},{"One":"USD"}]}]}', "rate": 0.0, "price": 3.0,
         "tol": 1e-12, "ref": "tests/pricer.rs:76-81"},
        {"json": '{"Scale":[{"Const":7.5},{"One":"USD"}]}', "rate": 0.0, "price": 7.5, "tol": 1e-12,
         "ref": "tests/pricer.rs:83-88"},
        {"json": '{"When":[{"At":1.0},{"One":"USD"}]}', "rate": 0.05, "price": math.exp(-0.05), "tol": 1e-12,
         "ref": "tests/pricer.rs:90-96"},
        {"json": '{"Scale":[{"Spot":"AAPL"},{"When":[{"At":1.0},{"One":"USD"}]}]}', "rate": 0.05, "price": 100.0,
         "tol": 1e-9, "ref": "tests/pricer.rs:98-106"},
    ],
    # first-touch / knock-out exact cases (tests/barriers.rs:104-153)
    "barrier_exact": [
        {"json": '{"Until":[{"Le":[{"Spot":"AAPL"},{"Const":200.0}]},%s]}' % call("AAPL", "100.0", "1.0"),
         "s0": 100.0, "sigma": 0.2, "mu": 0.05, "rate": 0.05, "n_paths": 1000, "seed": 1, "spy": 10,
         "price": 0.0, "tol": 0.0, "ref": "tests/barriers.rs:104-120"},
        {"json": '{"Anytime":[{"Ge":[{"Spot":"AAPL"},{"Const":105.0}]},{"When":[{"At":2.0},{"One":"USD"}]}]}',
         "s0": 100.0, "sigma": 0.0, "mu": 0.05, "rate": 0.05, "n_paths": 8, "seed": 1, "spy": 12,
         "price": math.exp(-0.1), "tol": 1e-9, "ref": "tests/barriers.rs:122-138"},
        {"json": '{"Anytime":[{"Ge":[{"Spot":"AAPL"},{"Const":200.0}]},{"When":[{"At":2.0},{"One":"USD"}]}]}',
         "s0": 100.0, "sigma": 0.0, "mu": 0.05, "rate": 0.05, "n_paths": 8, "seed": 1, "spy": 12,
         "price": 0.0, "tol": 0.0, "ref": "tests/barriers.rs:140-153"},
    ],
    # compiler plans (tests/compiler.rs:19-122)
    "plans": [
        {"json": '{"When":[{"At":1.0},{"One":"USD"}]}', "assets": [], "fixed_dates": [1.0], "horizon": 1.0,
         "needs_fine_grid": False, "grids": {"50": [0.0, 1.0]}, "ref": "tests/compiler.rs:19-29"},
        {"json": call("AAPL", "150.0", "1.0"), "assets": ["AAPL"], "fixed_dates": [1.0], "horizon": 1.0,
         "needs_fine_grid": False, "ref": "tests/compiler.rs:31-38"},
        {"json": UO, "assets": ["AAPL"], "fixed_dates": [1.0], "horizon": 1.0, "needs_fine_grid": True,
         "grid_len": {"12": 13}, "ref": "tests/compiler.rs:40-57"},
        {"json": '{"When":[{"At":1.0},{"Scale":[{"Add":[{"Spot":"MSFT"},{"Spot":"AAPL"}]},{"One":"USD"}]}]}',
         "assets": ["AAPL", "MSFT"], "fixed_dates": [1.0], "horizon": 1.0, "needs_fine_grid": False,
         "ref": "tests/compiler.rs:59-66"},
        {"json": '{"And":[{"When":[{"At":0.5},{"One":"USD"}]},{"Until":[{"Ge":[{"Spot":"AAPL"},{"Const":150.0}]},%s]}]}'
                 % call("AAPL", "120.0", "1.0"),
         "assets": ["AAPL"], "fixed_dates": [0.5, 1.0], "horizon": 1.0, "needs_fine_grid": True,
         "grid_contains": {"10": 0.5}, "ref": "tests/compiler.rs:68-82"},
        {"json": '"Zero"', "assets": [], "fixed_dates": [], "horizon": 0.0, "needs_fine_grid": False,
         "grids": {"12": [0.0]}, "ref": "tests/compiler.rs:86-94"},
        {"json": '{"Anytime":[{"Le":[{"Spot":"AAPL"},{"Const":80.0}]},{"When":[{"At":2.0},{"One":"USD"}]}]}',
         "assets": ["AAPL"], "fixed_dates": [2.0], "horizon": 2.0, "needs_fine_grid": True,
         "ref": "tests/compiler.rs:96-103"},
        {"json": '{"And":[{"When":[{"At":1.0},{"One":"USD"}]},{"When":[{"At":1.0},{"One":"EUR"}]}]}',
         "assets": [], "fixed_dates": [1.0], "horizon": 1.0, "needs_fine_grid": False,
         "ref": "tests/compiler.rs:114-121"},
    ],
    "malformed": [{"json": '{"When":[{"At":-1.0},{"One":"USD"}]}', "status": "MalformedContract",
                   "ref": "tests/compiler.rs:106-112"}],
    "garbage": [{"json": "{ not valid json", "ref": "tests/ast.rs:100"},
                {"json": '"Unknown"', "ref": "tests/ast.rs:101"}],
    # hand-built paths (tests/j26_temporal_obs.rs:24-88): value = obs at the last step (rate 0)
    "on_path": [
        {"json": '{"When":[{"At":1.0},{"Scale":[{"Average":{"obs":{"Spot":"S"},"from_year":0.25,"to_year":0.75}},'
                 '{"One":"USD"}]}]}',
         "times": [0.0, 0.25, 0.5, 0.75, 1.0], "values": [1.0, 2.0, 3.0, 4.0, 5.0], "value": 3.0, "tol": 1e-12,
         "ref": "tests/j26_temporal_obs.rs:61-71"},
        {"json": '{"When":[{"At":1.0},{"Scale":[{"Average":{"obs":{"Const":7.0},"from_year":null,"to_year":null}},'
                 '{"One":"USD"}]}]}',
         "times": [0.0, 0.25, 0.5, 0.75, 1.0], "values": [100.0, 105.0, 98.0, 102.0, 110.0], "value": 7.0,
         "tol": 1e-14, "ref": "tests/j26_temporal_obs.rs:23-34"},
        {"json": '{"When":[{"At":0.75},{"Scale":[{"RunningMax":{"Spot":"S"}},{"One":"USD"}]}]}',
         "times": [0.0, 0.25, 0.5, 0.75, 1.0], "values": [1.0, 2.0, 3.0, 4.0, 5.0], "value": 4.0, "tol": 1e-14,
         "ref": "tests/j26_temporal_obs.rs:36-47"},
        {"json": '{"When":[{"At":0.5},{"Scale":[{"RunningMin":{"Spot":"S"}},{"One":"USD"}]}]}',
         "times": [0.0, 0.25, 0.5, 0.75, 1.0], "values": [5.0, 4.0, 3.0, 2.0, 1.0], "value": 3.0, "tol": 1e-14,
         "ref": "tests/j26_temporal_obs.rs:49-59"},
    ],
    # the ten round-trip contracts of tests/ast.rs:77-97 in serde form
    "roundtrip": [
        '"Zero"', '{"One":"USD"}', '{"Give":{"One":"EUR"}}', '{"And":[{"One":"USD"},{"Give":{"One":"EUR"}}]}',
        '{"Or":[{"One":"USD"},{"One":"EUR"}]}', '{"Scale":[{"Const":100.0},{"One":"USD"}]}',
        '{"Scale":[{"Spot":"AAPL"},{"One":"USD"}]}', '{"When":[{"At":1.0},{"One":"USD"}]}',
        call("AAPL", "150.0", "1.0"), UO,
    ],
}

if __name__ == "__main__":
    with open(OUT, "w") as f:
        json.dump(known, f, indent=1)
    print("wrote", OUT)
