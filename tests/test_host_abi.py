"""CPU tests of the engine's host side and C ABI (no GPU needed): the library
loads and exports every symbol include/kontract_gpu.h declares, the ctypes
structures match the C layout, and the engine's parser / compiler / grid agree
exactly with the oracle's."""
import ctypes as C
import json
import os
import random
import re
import subprocess
import tempfile

import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kontract_gpu.h")
GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "known_answers.json")))


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    text = open(HEADER).read()
    decls = set(re.findall(r"\b(kx_[a-z_0-9]+)\s*\(", text))
    assert len(decls) >= 16
    for name in decls:
        assert hasattr(lib, name), name
    assert set(_abi.SIGNATURES) == decls
    assert lib.kx_abi_version() == 1


STRUCTS = {
    "kx_model": _abi.KxModel, "kx_mc_config": _abi.KxMcConfig, "kx_price_result": _abi.KxPriceResult,
    "kx_bumps": _abi.KxBumps, "kx_greeks": _abi.KxGreeks, "kx_adjoint_cfg": _abi.KxAdjointCfg,
    "kx_sens": _abi.KxSens, "kx_launch_stats": _abi.KxLaunchStats, "kx_plan_info": _abi.KxPlanInfo,
    "kx_book_info": _abi.KxBookInfo, "kx_chunk_stats": _abi.KxChunkStats,
}


def test_struct_layouts_match_header():
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "l.c"), os.path.join(d, "l")
        open(src, "w").write("\n".join(lines))
        subprocess.run(["gcc", "-o", exe, src], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = {}
    for ln in out.splitlines():
        s, f, v = ln.split()
        got[(s, f)] = int(v)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


@pytest.mark.parametrize("js", GOLD["roundtrip"])
def test_dsl_writes_serde_json(js):
    c = kx.Contract.from_json(js)
    assert c.to_json() == js


def test_dsl_builds_reference_contracts():
    # tests/ast.rs:77-97 built with the Python DSL reproduce the serde strings
    built = [
        kx.zero(), kx.one("USD"), kx.give(kx.one("EUR")), kx.one("USD") + kx.give(kx.one("EUR")),
        kx.one("USD").or_(kx.one("EUR")), kx.scale(100.0, kx.one("USD")), kx.scale(kx.S("AAPL"), kx.one("USD")),
        kx.one("USD") @ kx.at(1.0), kx.european_call("AAPL", 150.0, 1.0), kx.up_and_out_call("AAPL", 150.0, 200.0, 1.0),
    ]
    for c, js in zip(built, GOLD["roundtrip"]):
        assert c.to_json() == js


def test_garbage_is_serde_error():
    for case in GOLD["garbage"]:
        with pytest.raises(kx.KontractError) as e:
            kx.Contract.from_json(case["json"])
        assert e.value.status == "Serde"
    for bad in ['{"When":[{"At":1.0}]}', '{"Spot":"X"}', '{"One":"USD","Zero":null}', '{"Scale":[{"Foo":1},"Zero"]}',
                '{"When":[{"At":1e999},"Zero"]}', '"Zero" x']:
        h = C.c_void_p()
        assert _abi.load().kx_compile(bad.encode(), C.byref(h)) == _abi.KX_SERDE, bad


def test_or_and_negative_dates_fail_late_like_the_reference():
    # Contract::from_json accepts them; compile()/price_gbm reject them.
    orc = kx.Contract.from_json('{"Or":[{"One":"USD"},{"One":"USD"}]}')
    assert orc.plan()["assets"] == []  # compile() walks `or` (compiler.rs:101-104)
    neg = kx.Contract.from_json(GOLD["malformed"][0]["json"])
    with pytest.raises(kx.KontractError) as e:
        neg.plan()
    assert e.value.status == "MalformedContract"


def test_serde_accepts_struct_variant_as_sequence_and_unit_as_map(orc):
    js = '{"When":[{"At":1},{"Scale":[{"Average":[{"Spot":"S"},0.5,null]},{"Zero":null}]}]}'
    kx.Contract.from_json(js)
    orc.parse(js)


# ---- compiler / grid parity with the oracle --------------------------------
def _random_obs(rng, depth, assets):
    r = rng.random()
    if depth <= 0 or r < 0.3:
        return kx.S(rng.choice(assets)) if rng.random() < 0.6 else kx.const_(round(rng.uniform(-5, 150), 3))
    k = rng.choice(["add", "sub", "mul", "max", "min", "neg", "avg", "avgw", "rmax", "rmin"])
    a = _random_obs(rng, depth - 1, assets)
    if k == "neg":
        return -a
    if k == "avg":
        return kx.average(a)
    if k == "avgw":
        t0 = round(rng.uniform(0, 1.5), 3)
        return kx.average_over(a, t0, t0 + round(rng.uniform(0, 1), 3))
    if k == "rmax":
        return kx.running_max(a)
    if k == "rmin":
        return kx.running_min(a)
    b = _random_obs(rng, depth - 1, assets)
    return {"add": a + b, "sub": a - b, "mul": a * b, "max": a.max(b), "min": a.min(b)}[k]


def _random_cond(rng, depth, assets):
    r = rng.random()
    if depth <= 0 or r < 0.4:
        if rng.random() < 0.4:
            return kx.at(round(rng.uniform(0, 2.5), 4))
        a, b = _random_obs(rng, 1, assets), _random_obs(rng, 1, assets)
        return rng.choice([a >= b, a > b, a <= b, a < b])
    k = rng.choice(["and", "or", "not"])
    a = _random_cond(rng, depth - 1, assets)
    if k == "not":
        return ~a
    b = _random_cond(rng, depth - 1, assets)
    return a & b if k == "and" else a | b


def _random_contract(rng, depth, assets):
    r = rng.random()
    if depth <= 0 or r < 0.2:
        return kx.one("USD") if rng.random() < 0.8 else kx.zero()
    k = rng.choice(["give", "and", "scale", "when", "anytime", "until"])
    a = _random_contract(rng, depth - 1, assets)
    if k == "give":
        return kx.give(a)
    if k == "and":
        return a + _random_contract(rng, depth - 1, assets)
    if k == "scale":
        return kx.scale(_random_obs(rng, 2, assets), a)
    cond = _random_cond(rng, 2, assets)
    return {"when": kx.when, "anytime": kx.anytime, "until": kx.until}[k](cond, a)


@pytest.mark.parametrize("seed", range(40))
def test_random_contracts_plan_and_grid_match_oracle(orc, seed):
    rng = random.Random(seed)
    c = _random_contract(rng, 5, ["AAPL", "MSFT"])
    js = c.to_json()
    c2 = kx.Contract.from_json(js)
    assert c2.to_json() == js
    p = c2.plan()
    q = orc.plan(js)
    for k in ("assets", "fixed_dates", "horizon", "needs_fine_grid"):
        assert p[k] == q[k], k
    for spy in (1, 12, 50, 365):
        for force in (False, True):
            assert c2.time_grid(spy, force) == orc.time_grid(js, spy, force)


@pytest.mark.parametrize("case", GOLD["plans"], ids=lambda c: c["ref"])
def test_engine_plans_match_reference(case):
    p = kx.Contract.from_json(case["json"]).plan()
    for k in ("assets", "fixed_dates", "horizon", "needs_fine_grid"):
        assert p[k] == case[k]


def test_lowered_table_shape():
    uo = kx.up_and_out_call("AAPL", 100.0, 200.0, 1.0).plan()
    assert (uo["n_triggers"], uo["n_flows"], uo["n_accumulators"]) == (2, 1, 0)
    asian = (kx.scale((kx.average(kx.S("S")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0)).plan()
    assert (asian["n_triggers"], asian["n_flows"], asian["n_accumulators"]) == (1, 1, 1)


def test_pricing_without_device_fails_loudly():
    lib = _abi.load()
    n = C.c_int32()
    if lib.kx_device_info(None, 0, C.byref(n), None, None) == _abi.KX_OK:
        pytest.skip("a CUDA device is present")
    with pytest.raises(kx.KontractError) as e:
        kx.european_call("X", 100.0, 1.0).price(kx.GBM(100, 0.2, 0.05, asset="X"), n_paths=10)
    assert e.value.status == "NoDevice"


def test_measure_peak_rejects_unknown_loops():
    import ctypes as C
    lib = _abi.load()
    v = C.c_double()
    assert lib.kx_measure_peak(5, C.byref(v)) == _abi.KX_INVALID_ARGUMENT
    assert lib.kx_measure_peak(-1, C.byref(v)) == _abi.KX_INVALID_ARGUMENT


def test_book_sensitivities_validate_the_book_on_the_host():
    """kx_price_batch_sens checks its book before it needs a device: a
    path-dependent contract is refused (Unsupported) wherever it runs, NULL
    arrays are invalid, an empty book is a no-op; a book of Europeans then
    needs the device (NoDevice here when there is none)."""
    lib = _abi.load()
    m = kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.5, 0.05, asset="X")
    with pytest.raises(kx.KontractError) as e:
        kx.price_batch([kx.european_call("X", 100.0, 1.0), kx.up_and_out_call("X", 100.0, 130.0, 1.0)], m,
                       n_paths=100, greeks=True)
    assert e.value.status == "Unsupported"
    assert kx.price_batch([], m, greeks=True) == ([], [])
    out, sens = _abi.KxPriceResult(), _abi.KxSens()
    assert lib.kx_price_batch_sens(1, None, None, None, C.byref(out), C.byref(sens)) == _abi.KX_INVALID_ARGUMENT
    n = C.c_int32()
    if lib.kx_device_info(None, 0, C.byref(n), None, None) != _abi.KX_OK:
        with pytest.raises(kx.KontractError) as e:
            kx.price_batch([kx.european_call("X", 100.0, 1.0)], m, n_paths=100, greeks=True)
        assert e.value.status == "NoDevice"
