"""The C ABI from C: tests/c_abi/abi_smoke.c is compiled with gcc against
include/kontract_gpu.h and linked with the engine's library, as a Rust or
other FFI binding would link it. Without a GPU the pricing calls must return
KX_NO_DEVICE (no CPU fallback); with one, they must return what the Python
binding returns for the same arguments."""
import os
import subprocess

import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi", "abi_smoke.c")
LIBDIR = os.path.join(ROOT, "kontracts_gb300")


def _run(tmp_path) -> dict:
    _abi.load()  # the library is built
    exe = str(tmp_path / "abi_smoke")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), "-o", exe,
                    SRC, "-L", LIBDIR, "-lkontract_gpu", f"-Wl,-rpath,{LIBDIR}", "-lm"], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout
    return {ln.split()[0]: ln.split()[1:] for ln in out.splitlines()}


def test_c_caller_compiles_and_links(tmp_path):
    r = _run(tmp_path)
    assert r["abi_version"] == ["0", "1"]
    assert r["compile"] == ["0"] and r["compile_put"] == ["0"]
    assert r["compile_bad"] == [str(_abi.KX_SERDE), "null"]
    assert r["plan"][:2] == ["0", "1"] and float(r["plan"][2]) == 1.0 and r["plan"][3] == "1"
    assert r["grid"] == ["0", "366"]
    for call in ("price", "adjoint", "lsm"):
        assert int(r[call][0]) in (_abi.KX_OK, _abi.KX_NO_DEVICE), (call, r[call])
    assert r["chunk_moments"] == ["0", "4", "2.5", "5"]  # host code: no device needed


@pytest.mark.gpu
def test_c_caller_matches_python_binding(tmp_path):
    r = _run(tmp_path)
    uo = kx.up_and_out_call("S", 100.0, 200.0, 1.0)
    m = kx.GBM(s0=180.0, sigma=0.25, r=0.05, asset="S")
    assert r["price"][0] == "0"
    p = uo.price(m, n_paths=200_000, seed=42, steps_per_year=365, precision="fp32")
    assert float(r["price"][1]) == p.price and float(r["price"][2]) == p.std_error and r["price"][3] == "200000"
    assert r["adjoint"][0] == "0"
    a = uo.adjoint(m, n_paths=200_000, seed=42, steps_per_year=365, checkpoint_every=16)
    assert [float(x) for x in r["adjoint"][1:]] == [a.price, a.d_s0, a.d_sigma, a.d_r, a.smoothing_width]
    assert r["lsm"][0] == "0"
    put = kx.scale((kx.const_(40.0) - kx.S("S")).clip(0.0), kx.one())
    lp = put.price_american(kx.GBM(s0=36.0, sigma=0.2, r=0.06, asset="S"), [(i + 1) / 50.0 for i in range(50)],
                            n_paths=100_000, seed=7, n_basis=4, precision="fp64")
    assert float(r["lsm"][1]) == lp.price and float(r["lsm"][2]) == lp.std_error
    # an unknown asset: the reference's UnknownAsset, no payload
    assert r["unknown_asset"] == [str(_abi.KX_UNKNOWN_ASSET), "1", "1"]
