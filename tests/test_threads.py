"""First calls from two threads at once. The library's device context is set
up lazily by the first call that needs it; two threads making their first
calls together must not both set it up (two streams, torn fields). Each case
runs in a fresh interpreter, so the calls really are the first of the
process; ctypes releases the GIL around foreign calls, so the two calls run
concurrently."""
import os
import subprocess
import sys
import textwrap

import pytest

from kontracts_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = textwrap.dedent("""
    import ctypes as C, sys, threading
    sys.path.insert(0, {root!r})
    import kontracts_gb300 as kx
    from kontracts_gb300 import _abi
    lib = _abi.load()
    go = threading.Barrier(2)
    out = [None, None]
""")


def _run(body: str) -> str:
    code = PRELUDE.format(root=ROOT) + textwrap.dedent(body)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_two_threads_first_device_queries_agree():
    # on a machine without a GPU both threads get KX_NO_DEVICE, with one a
    # device both get its description; never a crash or a mixed answer
    out = _run("""
        def q(i):
            name = C.create_string_buffer(256)
            sm, ma, mi = C.c_int32(), C.c_int32(), C.c_int32()
            go.wait()
            st = lib.kx_device_info(name, 256, C.byref(sm), C.byref(ma), C.byref(mi))
            out[i] = (st, name.value, sm.value, ma.value, mi.value)
        ts = [threading.Thread(target=q, args=(i,)) for i in range(2)]
        [t.start() for t in ts]; [t.join() for t in ts]
        assert out[0] == out[1], out
        assert out[0][0] in (_abi.KX_OK, _abi.KX_NO_DEVICE), out
        print(out[0][0])
    """)
    assert out.strip() in (str(_abi.KX_OK), str(_abi.KX_NO_DEVICE))


@pytest.mark.gpu
def test_two_threads_first_prices_at_once_match_one_thread():
    _run("""
        c = kx.up_and_out_call("X", 100.0, 150.0, 1.0)
        m = kx.GBM(s0=100.0, sigma=0.25, r=0.03, asset="X")
        def p(i):
            go.wait()
            out[i] = c.price(m, n_paths=200_000, seed=11, steps_per_year=252, precision="fp32")
        ts = [threading.Thread(target=p, args=(i,)) for i in range(2)]
        [t.start() for t in ts]; [t.join() for t in ts]
        one = c.price(m, n_paths=200_000, seed=11, steps_per_year=252, precision="fp32")
        for r in out:
            assert r.price == one.price and r.std_error == one.std_error, (r.price, one.price)
    """)
