"""kx_price_fixed_scratch: the pricing call that allocates no device memory.
Called through the C ABI and compared with kx_price on the same arguments,
twice in a row (the first call of the process does the set-up). Collected
last so that it runs both after the other tests and, alone, in a fresh
process."""
import ctypes as C

import numpy as np
import pytest

import kontracts_gb300 as kx
from kontracts_gb300 import _abi

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the two calls run the same kernels on the same paths


def _fixed(contract, model, n_paths, seed, spy, precision, per_path=False):
    h = kx._Handle(contract.to_json())
    cm = model._c()
    cfg = kx._cfg(n_paths, seed, spy, model.rate, precision, False)
    out = _abi.KxPriceResult()
    pv = np.zeros(n_paths, dtype=np.float64) if per_path else None
    ptr = pv.ctypes.data_as(C.POINTER(C.c_double)) if per_path else None
    st = kx._lib().kx_price_fixed_scratch(h.h, C.byref(cm), C.byref(cfg), C.byref(out), ptr)
    return st, kx.PriceResult(out), pv


def _close(a, b):
    return abs(a - b) <= TOL * max(1.0, abs(b))


CASES = [
    ("up_and_out_fp32", lambda: kx.up_and_out_call("X", 100.0, 200.0, 1.0),
     lambda: kx.GBM(s0=180.0, sigma=0.25, r=0.05, asset="X"), 1 << 20, 365, "fp32"),
    ("asian_fp64", lambda: kx.scale((kx.average(kx.S("X")) - 100.0).clip(0.0), kx.one()) @ kx.at(1.0),
     lambda: kx.GBM(s0=100.0, sigma=0.3, r=0.02, asset="X"), 50_000, 52, "fp64"),
    ("heston_call_fp32", lambda: kx.european_call("X", 100.0, 1.0),
     lambda: kx.heston(100.0, 0.04, 2.0, 0.04, 0.3, -0.7, 0.03, asset="X"), 200_000, 252, "fp32"),
]


@pytest.mark.parametrize("name,mk_c,mk_m,n,spy,prec", CASES, ids=[c[0] for c in CASES])
def test_fixed_scratch_matches_kx_price_twice(name, mk_c, mk_m, n, spy, prec):
    c, m = mk_c(), mk_m()
    ref = c.price(m, n_paths=n, seed=7, steps_per_year=spy, precision=prec)
    for _ in range(2):
        st, r, _ = _fixed(c, m, n, 7, spy, prec)
        assert st == 0, kx._lib().kx_last_error_message()
        assert _close(r.price, ref.price), (r.price, ref.price)
        assert _close(r.std_error, ref.std_error)
        assert r.n_paths == n


def test_fixed_scratch_per_path_values():
    c = kx.until(kx.S("X") <= 85.0, kx.european_put("X", 100.0, 0.5))
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.01, asset="X")
    _, pv = c.price(m, n_paths=20_000, seed=3, steps_per_year=252, precision="fp64", per_path=True)
    for _ in range(2):
        st, _, pv2 = _fixed(c, m, 20_000, 3, 252, "fp64", per_path=True)
        assert st == 0
        assert np.allclose(pv2, np.asarray(pv), rtol=TOL, atol=TOL)


def test_fixed_scratch_call_leaves_free_device_memory_unchanged():
    # the property the entry point exists for: after a first call (set-up),
    # a call takes no device memory, so the device's free memory is the same
    # before and after it, even for a launch kx_price has not sized its
    # buffers for yet
    torch = pytest.importorskip("torch")
    c = kx.up_and_out_call("X", 100.0, 150.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.3, r=0.02, asset="X")
    for prec in ("fp32", "fp64"):  # set-up, and the lazy loading of both kernels' code
        st, _, _ = _fixed(c, m, 1000, 5, 52, prec)
        assert st == 0, kx._lib().kx_last_error_message()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for n, prec in ((1 << 20, "fp32"), (300_000, "fp64")):
        st, r, _ = _fixed(c, m, n, 9, 252, prec)
        assert st == 0 and r.n_paths == n
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_fixed_scratch_rejects_sizes_beyond_its_limits():
    c = kx.european_call("X", 100.0, 1.0)
    m = kx.GBM(s0=100.0, sigma=0.2, r=0.01, asset="X")
    st, _, _ = _fixed(c, m, (1 << 20) + 1, 1, 52, "fp32")
    assert st == _abi.KX_INVALID_ARGUMENT
    assert "fixed scratch limit" in kx._lib().kx_last_error_message().decode()
    # 8192 grid points at most: 40 years daily is 14601 points
    lng = kx.up_and_out_call("X", 100.0, 300.0, 40.0)
    st, _, _ = _fixed(lng, m, 1000, 1, 365, "fp32")
    assert st == _abi.KX_INVALID_ARGUMENT
    assert "fixed scratch limit" in kx._lib().kx_last_error_message().decode()
    # a valid call still works after the rejections
    st, r, _ = _fixed(c, m, 10_000, 1, 52, "fp32")
    assert st == 0 and r.n_paths == 10_000
