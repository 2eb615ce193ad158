"""Writes tests/golden/portfolio_256.json: the uneven book of 256 GBM contracts
priced in one persistent launch (seeded synthetic inputs, numpy
default_rng(42)). Mix 50/30/20: 128 European, 77 up-and-out barrier and
51 arithmetic-Asian calls (256 * 0.3 = 76.8 and 256 * 0.2 = 51.2 rounded).
s0 = 100, K ~ U[80, 120], sigma ~ U[0.1, 0.5], r = 0.03, barrier = s0 * U[1.1, 1.5],
T ~ U[0.25, 2] with 252 steps a year, n_paths = round(exp(U[ln 65536, ln 1048576])),
seed of contract i = 1000 + i. Run: python tests/golden/make_portfolio.py
"""
import json
import math
import os

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "portfolio_256.json")


def fmt(x):  # serde_json float text for the JSON strings
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from kontracts_gb300 import _fmt_f64
    return _fmt_f64(x)


def call_json(k, t):
    return ('{"When":[{"At":%s},{"Scale":[{"Max":[{"Sub":[{"Spot":"S"},{"Const":%s}]},{"Const":0.0}]},'
            '{"One":"USD"}]}]}' % (fmt(t), fmt(k)))


def main():
    rng = np.random.default_rng(42)
    kinds = ["euro"] * 128 + ["up_and_out"] * 77 + ["asian"] * 51
    rng.shuffle(kinds)
    book = []
    for i, kind in enumerate(kinds):
        k = float(rng.uniform(80, 120))
        sigma = float(rng.uniform(0.1, 0.5))
        b = 100.0 * float(rng.uniform(1.1, 1.5))
        t = float(rng.uniform(0.25, 2.0))
        n = int(round(math.exp(rng.uniform(math.log(65536), math.log(1048576)))))
        if kind == "euro":
            js = call_json(k, t)
        elif kind == "up_and_out":
            js = '{"Until":[{"Ge":[{"Spot":"S"},{"Const":%s}]},%s]}' % (fmt(b), call_json(k, t))
        else:
            js = ('{"When":[{"At":%s},{"Scale":[{"Max":[{"Sub":[{"Average":{"obs":{"Spot":"S"},"from_year":null,'
                  '"to_year":null}},{"Const":%s}]},{"Const":0.0}]},{"One":"USD"}]}]}' % (fmt(t), fmt(k)))
        book.append(dict(kind=kind, json=js, s0=100.0, sigma=sigma, r=0.03, strike=k, barrier=b, maturity=t,
                         n_paths=n, seed=1000 + i))
    meta = dict(steps_per_year=252, generator="numpy default_rng(42)", n=len(book),
                total_paths=sum(c["n_paths"] for c in book))
    with open(OUT, "w") as f:
        json.dump(dict(meta=meta, contracts=book), f, indent=0)
    print("wrote", OUT, meta)


if __name__ == "__main__":
    main()
