"""kontracts_gb300 — GB300 (sm_103a) Monte-Carlo engine for the `kontract`
contract algebra, with the call surface of the reference Python binding
(python/kontract/__init__.py, src/bindings.rs).

    from kontracts_gb300 import S, one, at, USD, GBM
    call = ((S("AAPL") - 100.0).clip(0.0) * one(USD)) @ at(1.0)
    res = call.price(GBM(s0=100, sigma=0.2, r=0.05, asset="AAPL"), n_paths=200_000)
    print(res.price, res.std_error)

Contracts serialise to the reference's serde JSON (Contract.to_json /
from_json, src/ast.rs:210-217); pricing goes through the C ABI of
libkontract_gpu.so (include/kontract_gpu.h). There is no CPU fallback: without
the built library or a CUDA device, pricing raises.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import threading
from typing import Any, Sequence

from . import _abi

__version__ = "0.2.3+gb300"

USD, EUR, GBP, JPY = "USD", "EUR", "GBP", "JPY"


class KontractError(ValueError):
    """Raised for every engine error (the reference raises ValueError,
    src/bindings.rs:50-52). `.status` is the kx_status name; `.payload` the
    date of TimeOutOfRange or the index of StepOutOfRange (error.rs:11-15),
    else None."""

    def __init__(self, status: int, message: str, payload=None):
        self.code = status
        self.status = _abi.STATUS_NAMES.get(status, str(status))
        self.payload = payload
        super().__init__(f"{self.status}: {message}")


_lock = threading.Lock()


def _lib():
    return _abi.load()


def _check(st: int) -> None:
    if st != _abi.KX_OK:
        lib = _lib()
        msg = lib.kx_last_error_message().decode("utf-8", "replace")
        t, k = C.c_double(), C.c_uint64()
        lib.kx_last_error_payload(C.byref(t), C.byref(k))
        payload = t.value if st == _abi.KX_TIME_OUT_OF_RANGE else k.value if st == _abi.KX_STEP_OUT_OF_RANGE else None
        raise KontractError(st, msg, payload)


# ---------------------------------------------------------------------------
# serde_json number formatting (ryu, as used by serde_json): shortest
# round-trip digits, decimal notation for 1e-5 <= |x| < 1e16, else d.ddde±x.
# ---------------------------------------------------------------------------
def _fmt_f64(x: float) -> str:
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return "null"  # serde_json writes non-finite floats as null
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign = "-" if x < 0 else ""
    r = repr(abs(x))
    if "e" in r:
        mant, ex = r.split("e")
        exp10 = int(ex)
    else:
        mant, exp10 = r, 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    # position of the decimal point relative to the digit string
    point = len(ip) + exp10 - (len(ip + fp) - len((ip + fp).lstrip("0")))
    digits = digits.rstrip("0") or "0"
    length = len(digits)
    kk = point
    exponent = kk - length
    if 0 <= exponent and kk <= 16:
        return sign + digits + "0" * exponent + ".0"
    if 0 < kk <= 16:
        return sign + digits[:kk] + "." + digits[kk:]
    if -5 < kk <= 0:
        return sign + "0." + "0" * (-kk) + digits
    e = kk - 1
    if length == 1:
        return f"{sign}{digits}e{e}"
    return f"{sign}{digits[0]}.{digits[1:]}e{e}"


def _dump(v: Any) -> str:
    """serde_json.to_string of our value tree (dict/list/str/float/bool/None)."""
    if v is None:
        return "null"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, float)):
        return _fmt_f64(v)
    if isinstance(v, str):
        return json.dumps(v, ensure_ascii=False)
    if isinstance(v, list):
        return "[" + ",".join(_dump(x) for x in v) + "]"
    if isinstance(v, dict):
        return "{" + ",".join(json.dumps(k) + ":" + _dump(x) for k, x in v.items()) + "}"
    raise TypeError(f"cannot serialise {type(v)}")


# ---------------------------------------------------------------------------
# AST (src/ast.rs) — values are kept in serde's externally tagged shape.
# ---------------------------------------------------------------------------
def _obs(x: Any) -> "Observable":
    if isinstance(x, Observable):
        return x
    if isinstance(x, (int, float)) and not isinstance(x, bool):
        return Observable({"Const": float(x)})
    raise TypeError("expected a number or an Observable")


class Observable:
    """A real-valued process (ast.rs:34-71)."""

    __slots__ = ("_v",)

    def __init__(self, v: Any):
        self._v = v

    def _bin(self, tag: str, other: Any, swap: bool = False) -> "Observable":
        o = _obs(other)
        a, b = (o, self) if swap else (self, o)
        return Observable({tag: [a._v, b._v]})

    def __add__(self, o): return self._bin("Add", o)
    def __radd__(self, o): return self._bin("Add", o, swap=True)
    def __sub__(self, o): return self._bin("Sub", o)
    def __rsub__(self, o): return self._bin("Sub", o, swap=True)
    def __mul__(self, o):
        if isinstance(o, Contract):
            return Contract({"Scale": [self._v, o._v]})
        return self._bin("Mul", o)
    def __rmul__(self, o): return self._bin("Mul", o, swap=True)
    def __truediv__(self, o): return self._bin("Div", o)
    def __rtruediv__(self, o): return self._bin("Div", o, swap=True)
    def __neg__(self): return Observable({"Neg": self._v})

    def max(self, o) -> "Observable": return self._bin("Max", o)
    def min(self, o) -> "Observable": return self._bin("Min", o)
    def clip(self, floor: float) -> "Observable": return self._bin("Max", float(floor))  # ast.rs:339
    def average(self) -> "Observable": return average(self)
    def average_over(self, from_year: float, to_year: float) -> "Observable":
        return average_over(self, from_year, to_year)
    def running_max(self) -> "Observable": return running_max(self)
    def running_min(self) -> "Observable": return running_min(self)
    def scale(self, c: "Contract") -> "Contract": return Contract({"Scale": [self._v, c._v]})

    def __ge__(self, o): return Condition({"Ge": [self._v, _obs(o)._v]})
    def __gt__(self, o): return Condition({"Gt": [self._v, _obs(o)._v]})
    def __le__(self, o): return Condition({"Le": [self._v, _obs(o)._v]})
    def __lt__(self, o): return Condition({"Lt": [self._v, _obs(o)._v]})
    def ge(self, o): return self.__ge__(o)
    def gt(self, o): return self.__gt__(o)
    def le(self, o): return self.__le__(o)
    def lt(self, o): return self.__lt__(o)

    def __eq__(self, other):  # structural equality (not a condition, as in the reference)
        return isinstance(other, Observable) and _dump(self._v) == _dump(other._v)

    __hash__ = None

    def __repr__(self):
        return f"Observable({_dump(self._v)})"


class Condition:
    """A boolean process (ast.rs:142-161)."""

    __slots__ = ("_v",)

    def __init__(self, v: Any):
        self._v = v

    def __and__(self, o: "Condition"): return Condition({"And": [self._v, o._v]})
    def __or__(self, o: "Condition"): return Condition({"Or": [self._v, o._v]})
    def __invert__(self): return Condition({"Not": self._v})

    def __eq__(self, other):
        return isinstance(other, Condition) and _dump(self._v) == _dump(other._v)

    __hash__ = None

    def __repr__(self):
        return f"Condition({_dump(self._v)})"


class PriceResult:
    """Mirror of PriceResult (src/pricer.rs:58-87)."""

    __slots__ = ("price", "sample_std", "std_error", "ci95_low", "ci95_high", "n_paths")

    def __init__(self, r: _abi.KxPriceResult):
        self.price = r.price
        self.sample_std = r.sample_std
        self.std_error = r.std_error
        self.ci95_low = r.ci95_low
        self.ci95_high = r.ci95_high
        self.n_paths = int(r.n_paths)

    def paths_for_tolerance(self, tol: float) -> int:  # pricer.rs:81-86
        if tol <= 0.0 or self.sample_std == 0.0:
            return 0
        return int(math.ceil((1.959963984540054 * self.sample_std / tol) ** 2))

    def __repr__(self):
        return (f"PriceResult(price={self.price:.6f}, std_error={self.std_error:.3g}, "
                f"ci95=[{self.ci95_low:.6f}, {self.ci95_high:.6f}], n_paths={self.n_paths})")


class Greeks:
    """Mirror of Greeks (src/greeks.rs:43-54) plus the CRN standard errors."""

    __slots__ = ("price", "delta", "gamma", "vega", "rho",
                 "price_se", "delta_se", "gamma_se", "vega_se", "rho_se")

    def __init__(self, g: _abi.KxGreeks):
        for k in self.__slots__:
            setattr(self, k, getattr(g, k))

    def __repr__(self):
        return (f"Greeks(price={self.price:.6f}, delta={self.delta:.6f}, gamma={self.gamma:.6f}, "
                f"vega={self.vega:.6f}, rho={self.rho:.6f})")


class Sensitivities:
    """Pathwise-adjoint price and sensitivities (kx_sens): d_s0, d_sigma, d_r
    for GBM; d_s0, d_v0, d_kappa, d_theta, d_sigma_v, d_rho, d_r for Heston;
    each with its standard error (se_*)."""

    __slots__ = tuple(n for n, _ in _abi.KxSens._fields_)

    def __init__(self, s: _abi.KxSens):
        for k in self.__slots__:
            setattr(self, k, getattr(s, k))

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k in self.__slots__}

    def __repr__(self):
        return (f"Sensitivities(price={self.price:.6f}, d_s0={self.d_s0:.6f}, d_sigma={self.d_sigma:.6f}, "
                f"d_r={self.d_r:.6f}, d_v0={self.d_v0:.6f}, d_kappa={self.d_kappa:.6f}, "
                f"d_theta={self.d_theta:.6f}, d_sigma_v={self.d_sigma_v:.6f}, d_rho={self.d_rho:.6f})")


class GBM:
    """GBM(s0, sigma, r, q=0.0, asset="ASSET"): drift r - q, discount r
    (src/bindings.rs:478-522)."""

    def __init__(self, s0: float, sigma: float, r: float, q: float = 0.0, asset: str = "ASSET"):
        self.s0, self.sigma, self.r, self.q, self.asset = float(s0), float(sigma), float(r), float(q), asset

    def _c(self) -> _abi.KxModel:
        return _abi.KxModel(kind=_abi.KX_MODEL_GBM, s0=self.s0, mu=self.r - self.q, sigma=self.sigma,
                            asset=self.asset.encode())

    @property
    def rate(self) -> float:
        return self.r

    def __repr__(self):
        return f"GBM(asset={self.asset!r}, s0={self.s0}, sigma={self.sigma}, r={self.r}, q={self.q})"


class Model:
    """Generic model handle (the reference's `Model`, bindings.rs:529-540)."""

    def __init__(self, label: str, cmodel: _abi.KxModel, rate: float, params: dict):
        self.label, self._cm, self.rate, self.params = label, cmodel, float(rate), params

    def _c(self) -> _abi.KxModel:
        return self._cm

    def __repr__(self):
        return f"Model({self.label}, rate={self.rate})"


class CorrelatedGbmN:
    """Correlated GBM factors (src/multi_asset.rs:49-105): `factors` is a list
    of (name, s0, mu, sigma) as GbmFactor::new (src/fx.rs:160-169) and `corr`
    their n x n correlation. `rate` discounts the flows (McConfig.rate)."""

    def __init__(self, factors: Sequence[tuple], corr: Sequence[Sequence[float]], rate: float = 0.0):
        self.factors = [(str(n), float(s0), float(mu), float(sg)) for n, s0, mu, sg in factors]
        self.corr = [[float(x) for x in row] for row in corr]
        self.rate = float(rate)
        k = len(self.factors)
        if k > _abi.KX_MAX_ASSETS:
            raise ValueError(f"at most {_abi.KX_MAX_ASSETS} factors")
        if len(self.corr) != k or any(len(r) != k for r in self.corr):
            raise KontractError(_abi.KX_MALFORMED_CONTRACT,
                                f"CorrelatedGbmN: the correlation matrix must be {k}x{k}")  # multi_asset.rs:69-73

    def _c(self) -> _abi.KxMultiGbm:
        k = len(self.factors)
        m = _abi.KxMultiGbm(n_assets=k)
        self._names = [n.encode() for n, _, _, _ in self.factors]  # keep the bytes alive
        for i, (n, s0, mu, sg) in enumerate(self.factors):
            m.names[i] = self._names[i]
            m.s0[i], m.mu[i], m.sigma[i] = s0, mu, sg
            for j in range(k):
                m.corr[i * k + j] = self.corr[i][j]
        return m


def heston(spot: float, v0: float, kappa: float, theta: float, sigma_v: float, rho: float, r: float,
           asset: str = "ASSET", scheme: str = "reference") -> Model:
    """Heston model (src/bindings.rs:547-567). `scheme`: "reference" (Euler
    step then v = max(v, 0), simulator.rs:517-534) or "full_truncation"."""
    sc = {"reference": _abi.KX_HESTON_REFERENCE_FLOOR,
          "full_truncation": _abi.KX_HESTON_FULL_TRUNCATION}[scheme]
    cm = _abi.KxModel(kind=_abi.KX_MODEL_HESTON, heston_scheme=sc, s0=float(spot), v0=float(v0),
                      kappa=float(kappa), theta=float(theta), sigma_v=float(sigma_v), rho=float(rho),
                      r=float(r), asset=asset.encode())
    return Model("Heston", cm, r, dict(spot=spot, v0=v0, kappa=kappa, theta=theta, sigma_v=sigma_v,
                                       rho=rho, r=r, asset=asset, scheme=scheme))


_PREC = {"fp32": _abi.KX_PREC_FP32, "fp64": _abi.KX_PREC_FP64, "fp32_kahan": _abi.KX_PREC_FP32_KAHAN}


def _cfg(n_paths: int, seed: int, spy: int, rate: float, precision: str, shared_draws: bool) -> _abi.KxMcConfig:
    if n_paths < 0:
        raise ValueError("n_paths must be non-negative")
    return _abi.KxMcConfig(n_paths=int(n_paths), seed=int(seed) & (2**64 - 1), steps_per_year=int(spy),
                           rng=_abi.KX_RNG_SHARED_DRAWS if shared_draws else _abi.KX_RNG_PHILOX,
                           precision=_PREC[precision], flags=0, rate=float(rate))


class _Handle:
    """Owns a compiled kx_program."""

    def __init__(self, js: str):
        h = C.c_void_p()
        _check(_lib().kx_compile(js.encode(), C.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                _lib().kx_program_free(self.h)
        except Exception:
            pass


class Contract:
    """A contract of the algebra (ast.rs:187-206)."""

    __slots__ = ("_v", "_h")

    def __init__(self, v: Any):
        self._v = v
        self._h = None

    # --- combinators (bindings.rs:255-311) ---
    def __matmul__(self, cond: Condition) -> "Contract": return Contract({"When": [cond._v, self._v]})
    def __add__(self, o: "Contract") -> "Contract": return Contract({"And": [self._v, o._v]})
    def __neg__(self) -> "Contract": return Contract({"Give": self._v})
    def when(self, cond: Condition) -> "Contract": return self @ cond
    def until(self, cond: Condition) -> "Contract": return Contract({"Until": [cond._v, self._v]})
    def anytime(self, cond: Condition) -> "Contract": return Contract({"Anytime": [cond._v, self._v]})
    def or_(self, o: "Contract") -> "Contract": return Contract({"Or": [self._v, o._v]})
    def and_(self, o: "Contract") -> "Contract": return self + o
    def give(self) -> "Contract": return -self

    def to_json(self) -> str:
        return _dump(self._v)

    @staticmethod
    def from_json(s: str) -> "Contract":
        try:
            v = json.loads(s)
        except json.JSONDecodeError as e:
            raise KontractError(_abi.KX_SERDE, str(e)) from None
        c = Contract(v)
        c._handle()  # full validation by the engine's parser + compiler
        return c

    def _handle(self) -> _Handle:
        if self._h is None:
            self._h = _Handle(self.to_json())
        return self._h

    def __eq__(self, other):
        return isinstance(other, Contract) and self.to_json() == other.to_json()

    __hash__ = None

    def __repr__(self):
        return f"Contract({self.to_json()})"

    # --- plan / grid ---
    def plan(self) -> dict:
        info = _abi.KxPlanInfo()
        dates = (C.c_double * 4096)()
        buf = C.create_string_buffer(1 << 16)
        _check(_lib().kx_program_plan(self._handle().h, C.byref(info), dates, 4096, buf, len(buf)))
        assets = buf.value.decode().split("\n") if info.n_assets else []
        return dict(assets=assets, fixed_dates=list(dates[: info.n_fixed_dates]), horizon=info.horizon,
                    needs_fine_grid=bool(info.needs_fine_grid), n_triggers=info.n_triggers,
                    n_flows=info.n_flows, n_accumulators=info.n_accumulators)

    def time_grid(self, steps_per_year: int, force_fine: bool = False) -> list[float]:
        n = C.c_size_t()
        _check(_lib().kx_time_grid(self._handle().h, steps_per_year, int(force_fine), None, 0, C.byref(n)))
        out = (C.c_double * max(1, n.value))()
        _check(_lib().kx_time_grid(self._handle().h, steps_per_year, int(force_fine), out, n.value, C.byref(n)))
        return list(out[: n.value])

    # --- pricing (bindings.rs:350-467) ---
    def price(self, model, n_paths: int = 100_000, seed: int = 42, steps_per_year: int = 50,
              antithetic: bool = False, control_variate: bool = False, *, precision: str = "fp32",
              shared_draws: bool = False, per_path: bool = False):
        """Price under `model` (GBM or Model), as Contract.price of the
        reference. Returns a PriceResult (and the per-path discounted values
        as a list when per_path=True). antithetic / control_variate: the
        reference's variance reduction (pricer.rs:108-230): antithetic pairs
        for GBM models, the at-the-money call as a control (no per-path
        values then)."""
        if isinstance(model, CorrelatedGbmN):
            if antithetic or control_variate:
                raise KontractError(_abi.KX_UNSUPPORTED, "variance reduction needs a one-asset model")
            mm = model._c()
            cfg = _cfg(n_paths, seed, steps_per_year, model.rate, precision, shared_draws)
            res = _abi.KxPriceResult()
            pp = (C.c_double * max(1, int(n_paths)))() if per_path else None
            with _lock:
                _check(_lib().kx_price_multi(self._handle().h, C.byref(mm), C.byref(cfg), C.byref(res), pp))
            if per_path:
                return PriceResult(res), list(pp[: int(n_paths)])
            return PriceResult(res)
        if not isinstance(model, (GBM, Model)):
            raise TypeError("expected a GBM, Model or CorrelatedGbmN")
        cm = model._c()
        cfg = _cfg(n_paths, seed, steps_per_year, model.rate, precision, shared_draws)
        cfg.flags = (_abi.KX_VR_ANTITHETIC if antithetic else 0) | (_abi.KX_VR_CONTROL_VARIATE if control_variate else 0)
        res = _abi.KxPriceResult()
        pp = (C.c_double * max(1, int(n_paths)))() if per_path else None
        with _lock:
            _check(_lib().kx_price(self._handle().h, C.byref(cm), C.byref(cfg), C.byref(res), pp))
        if per_path:
            return PriceResult(res), list(pp[: int(n_paths)])
        return PriceResult(res)

    def greeks(self, model: GBM, n_paths: int = 200_000, seed: int = 42, steps_per_year: int = 50, *,
               bumps: tuple | None = None, relative: bool = False, precision: str = "fp32",
               shared_draws: bool = False, smooth_width: float = 0.0) -> Greeks:
        """Bump-and-reprice Greeks with common random numbers (greeks.rs:60-98).
        `bumps` = (spot, vol, rate), absolute unless relative=True; default
        (1e-2, 1e-2, 1e-4) as BumpSizes::default (greeks.rs:31-39)."""
        if not isinstance(model, GBM):
            raise TypeError("greeks need a GBM model")
        hs, hv, hr = bumps if bumps is not None else (1e-2, 1e-2, 1e-4)
        b = _abi.KxBumps(spot=hs, vol=hv, rate=hr, relative=int(relative), smooth=int(smooth_width > 0),
                         smoothing_width=float(smooth_width))
        cm = model._c()
        cfg = _cfg(n_paths, seed, steps_per_year, model.r, precision, shared_draws)
        out = _abi.KxGreeks()
        with _lock:
            _check(_lib().kx_greeks_bump(self._handle().h, C.byref(cm), C.byref(cfg), C.byref(b), C.byref(out)))
        return Greeks(out)

    def adjoint(self, model, n_paths: int = 200_000, seed: int = 42, steps_per_year: int = 50, *,
                checkpoint_every: int = 16, smoothing_width: float = 0.0, precision: str = "fp32",
                shared_draws: bool = False) -> Sensitivities:
        """Pathwise-adjoint sensitivities in one reverse sweep per path
        (kx_greeks_adjoint). Barrier untils are smoothed by a logistic of
        `smoothing_width` in log-spot (<= 0: 0.5 sigma sqrt(dt))."""
        if not isinstance(model, (GBM, Model)):
            raise TypeError("expected a GBM or Model")
        cm = model._c()
        cfg = _cfg(n_paths, seed, steps_per_year, model.rate, precision, shared_draws)
        ac = _abi.KxAdjointCfg(checkpoint_every=int(checkpoint_every), reserved=0,
                               smoothing_width=float(smoothing_width))
        out = _abi.KxSens()
        with _lock:
            _check(_lib().kx_greeks_adjoint(self._handle().h, C.byref(cm), C.byref(cfg), C.byref(ac), C.byref(out)))
        return Sensitivities(out)

    def price_american(self, model, exercise_dates: Sequence[float], n_paths: int = 100_000, seed: int = 42,
                       n_basis: int = 3, *, precision: str = "fp32", shared_draws: bool = False,
                       basis: str = "monomial", per_path: bool = False):
        """Longstaff-Schwartz American pricing (lsm.rs:80-124); `self` is the
        exercised payoff, e.g. (K - S).clip(0) * one(USD). basis: "monomial"
        (the reference's) or "laguerre" (weighted Laguerre functions of S/s0).
        per_path=True also returns every path's discounted realised value
        (a numpy array)."""
        if basis not in ("monomial", "laguerre"):
            raise ValueError("basis must be 'monomial' or 'laguerre'")
        if not isinstance(model, (GBM, Model)):
            raise TypeError("expected a GBM or Model")
        cm = model._c()
        cfg = _cfg(n_paths, seed, 50, model.rate, precision, shared_draws)
        d = (C.c_double * max(1, len(exercise_dates)))(*[float(x) for x in exercise_dates])
        out = _abi.KxPriceResult()
        pp = None
        if per_path:
            import numpy as np
            pp = np.zeros(max(1, int(n_paths)))
        with _lock:
            _check(_lib().kx_price_american_lsm_paths(self._handle().h, C.byref(cm), C.byref(cfg), d,
                                                      len(exercise_dates), int(n_basis),
                                                      _abi.KX_LSM_LAGUERRE if basis == "laguerre" else _abi.KX_LSM_MONOMIAL,
                                                      C.byref(out),
                                                      pp.ctypes.data_as(C.POINTER(C.c_double)) if per_path else None))
        if per_path:
            return PriceResult(out), pp[: int(n_paths)]
        return PriceResult(out)


def price_american_batch(cases: Sequence[tuple], n_basis: int = 3, *, precision: str = "fp32",
                         basis: str = "monomial") -> list[PriceResult]:
    """Several Longstaff-Schwartz problems in one call (no reference
    counterpart). Each case is (payoff, model, exercise_dates, n_paths, seed);
    result i equals payoff_i.price_american(model_i, dates_i, n_paths_i,
    seed_i, n_basis, precision=..., basis=...) bit for bit."""
    if basis not in ("monomial", "laguerre"):
        raise ValueError("basis must be 'monomial' or 'laguerre'")
    n = len(cases)
    if n == 0:
        return []
    hs = (C.c_void_p * n)()
    models = (_abi.KxModel * n)()
    cfgs = (_abi.KxMcConfig * n)()
    dates = (C.POINTER(C.c_double) * n)()
    nd = (C.c_size_t * n)()
    keep = []
    for i, (payoff, model, ex, n_paths, seed) in enumerate(cases):
        if not isinstance(model, (GBM, Model)):
            raise TypeError("expected a GBM or Model")
        hs[i] = payoff._handle().h.value
        models[i] = model._c()
        cfgs[i] = _cfg(n_paths, seed, 50, model.rate, precision, False)
        d = (C.c_double * max(1, len(ex)))(*[float(x) for x in ex])
        keep.append(d)
        dates[i] = C.cast(d, C.POINTER(C.c_double))
        nd[i] = len(ex)
    out = (_abi.KxPriceResult * n)()
    with _lock:
        _check(_lib().kx_price_american_lsm_batch(n, hs, models, cfgs, dates, nd, int(n_basis),
                                                  _abi.KX_LSM_LAGUERRE if basis == "laguerre" else _abi.KX_LSM_MONOMIAL,
                                                  out))
    return [PriceResult(r) for r in out]


def _fmt_display(x: float) -> str:
    """Rust's `{}` of an f64: the shortest round-trip digits in plain decimal
    notation (no exponent), no fractional part for integral values, and NaN /
    inf / -inf for the non-finite ones."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    import decimal
    t = format(decimal.Decimal(repr(x)), "f")
    if "." in t:
        t = t.rstrip("0").rstrip(".")
    return t


def _rust_round(x: float) -> int:
    """f64::round (half away from zero) followed by `as i32` (NaN -> 0,
    saturating)."""
    if math.isnan(x):
        return 0
    if math.isinf(x):
        return 2**31 - 1 if x > 0 else -(2**31)
    a = abs(x)
    r = math.floor(a)
    if a - r >= 0.5:
        r += 1
    r = int(r) if x >= 0 else -int(r)
    return max(-(2**31), min(2**31 - 1, r))


class GreekSurface:
    """Mirror of GreekSurface (src/surface.rs:17-35): the axes `spots` and
    `vols` and the matrices price, delta, gamma, vega of shape
    [len(spots), len(vols)] (row i = spots[i], column j = vols[j]), plus rho
    and each estimator's standard error (`<name>_se`), as numpy arrays."""

    QUANTITIES = ("price", "delta", "gamma", "vega", "rho",
                  "price_se", "delta_se", "gamma_se", "vega_se", "rho_se")

    def __init__(self, spots: Sequence[float], vols: Sequence[float], cells: Sequence[Any]):
        import numpy as np
        self.spots = [float(s) for s in spots]
        self.vols = [float(v) for v in vols]
        shape = (len(self.spots), len(self.vols))
        for q in self.QUANTITIES:
            setattr(self, q, np.array([getattr(g, q) for g in cells], dtype=np.float64).reshape(shape))

    def to_csv(self, quantity) -> str:
        """surface.rs:38-62: header `spot\\vol,<vols>`, then one row per spot."""
        head = "spot\\vol" + "".join("," + _fmt_display(v) for v in self.vols) + "\n"
        rows = "".join(_fmt_display(s) + "".join("," + _fmt_display(quantity[i][j]) for j in range(len(self.vols)))
                       + "\n" for i, s in enumerate(self.spots))
        return head + rows

    def to_pgm(self, quantity) -> str:
        """surface.rs:64-97: P2 (ASCII) grayscale, min -> 0 and max -> 255."""
        rows, cols = len(quantity), (len(quantity[0]) if len(quantity) else 0)
        lo, hi = math.inf, -math.inf
        for i in range(rows):
            for j in range(cols):
                x = float(quantity[i][j])
                if not math.isnan(x):  # f64::min / f64::max ignore NaN
                    lo, hi = min(lo, x), max(hi, x)
        span = 1.0 if abs(hi - lo) < 1e-300 else hi - lo
        out = [f"P2\n{cols} {rows}\n255\n"]
        for i in range(rows):
            out.append("".join(f"{max(0, min(255, _rust_round((float(quantity[i][j]) - lo) / span * 255.0)))} "
                               for j in range(cols)) + "\n")
        return "".join(out)

    def __repr__(self):
        return f"GreekSurface({len(self.spots)} spots x {len(self.vols)} vols)"


def _adjoint_surface(contract, asset, spots, vols, n_paths, seed, steps_per_year, rate, precision) -> GreekSurface:
    if not spots or not vols:
        raise KontractError(_abi.KX_INCONSISTENT_PATH, "empty surface grid")  # surface.rs:113-117
    cells = [(float(s), float(v)) for s in spots for v in vols]
    models = [GBM(s0=s, sigma=v, r=rate, asset=asset) for s, v in cells]
    res, sens = price_portfolio([contract] * len(cells), models, [n_paths] * len(cells), seed, steps_per_year,
                                precision=precision, greeks=True)
    nan = float("nan")

    class _Cell:
        pass
    out = []
    for r, g in zip(res, sens):
        c = _Cell()
        c.price, c.price_se = r.price, r.std_error
        c.delta, c.delta_se = g.d_s0, g.se_s0
        c.vega, c.vega_se = g.d_sigma, g.se_sigma
        c.rho, c.rho_se = g.d_r, g.se_r
        c.gamma = c.gamma_se = nan
        out.append(c)
    return GreekSurface(spots, vols, out)


def greek_surface(contract: Contract, asset: str, spots: Sequence[float], vols: Sequence[float],
                  n_paths: int = 100_000, seed: int = 42, steps_per_year: int = 50, rate: float = 0.0, *,
                  bumps: tuple | None = None, relative: bool = False, precision: str = "fp32",
                  method: str = "bump") -> GreekSurface:
    """greek_surface (src/surface.rs:104-137): bump-and-reprice Greeks
    (greeks_gbm) at every cell of spots x vols, all cells on the same seed.
    The arguments after `vols` are McConfig's fields (default McConfig,
    pricer.rs:44-54) and BumpSizes (default (1e-2, 1e-2, 1e-4)). One path
    launch values every cell and its seven reprices.

    method="adjoint" (no reference counterpart): every cell is a contract of
    one pathwise-adjoint portfolio launch (kx_price_portfolio with
    sensitivities): price with the hard barriers, delta / vega / rho of the
    barrier-smoothed payoff, gamma NaN (a pathwise first derivative only)."""
    if method == "adjoint":
        return _adjoint_surface(contract, asset, spots, vols, n_paths, seed, steps_per_year, rate, precision)
    if method != "bump":
        raise ValueError("method must be 'bump' or 'adjoint'")
    hs, hv, hr = bumps if bumps is not None else (1e-2, 1e-2, 1e-4)
    b = _abi.KxBumps(spot=hs, vol=hv, rate=hr, relative=int(relative), smooth=0, smoothing_width=0.0)
    cfg = _cfg(n_paths, seed, steps_per_year, rate, precision, False)
    ns, nv = len(spots), len(vols)
    sp = (C.c_double * max(1, ns))(*[float(x) for x in spots])
    vo = (C.c_double * max(1, nv))(*[float(x) for x in vols])
    out = (_abi.KxGreeks * max(1, ns * nv))()
    with _lock:
        _check(_lib().kx_greek_surface(contract._handle().h, asset.encode(), sp, ns, vo, nv, C.byref(cfg),
                                       C.byref(b), out))
    return GreekSurface(spots, vols, [Greeks(g) for g in out[: ns * nv]])


def fit_gbm_volatility(contract: Contract, maturities: Sequence[float], market_prices: Sequence[tuple], rate: float,
                       n_paths: int = 2000) -> float:
    """The reference binding's fit_gbm_volatility (src/bindings.rs:1014-1038):
    the fitted GBM volatility for (spot, price) quotes
    (kontracts_gb300.calibration.fit_gbm_volatility with n_paths)."""
    from . import calibration
    cfg = calibration.FastCalibrationConfig(n_paths=int(n_paths))
    return calibration.fit_gbm_volatility(contract, maturities, market_prices, rate, cfg).parameters[0]


def price_batch(contracts: Sequence[Contract], model, n_paths: int = 100_000, seed: int = 42,
                steps_per_year: int = 50, *, precision: str = "fp32", greeks: bool = False):
    """price_batch_gbm (src/pricer.rs:250-294): every contract on the same paths.
    With greeks=True (a book of Europeans: each contract pays one call, put or
    constant at a fixed date) also returns every contract's pathwise
    Sensitivities, from one forward pass over the shared paths."""
    if not contracts:
        return ([], []) if greeks else []
    hs = (C.c_void_p * len(contracts))(*[c._handle().h.value for c in contracts])
    cm = model._c()
    cfg = _cfg(n_paths, seed, steps_per_year, model.rate, precision, False)
    out = (_abi.KxPriceResult * len(contracts))()
    if greeks:
        sens = (_abi.KxSens * len(contracts))()
        with _lock:
            _check(_lib().kx_price_batch_sens(len(contracts), hs, C.byref(cm), C.byref(cfg), out, sens))
        return [PriceResult(r) for r in out], [Sensitivities(s) for s in sens]
    with _lock:
        _check(_lib().kx_price_batch_shared(len(contracts), hs, C.byref(cm), C.byref(cfg), out))
    return [PriceResult(r) for r in out]


def price_portfolio(contracts: Sequence[Contract], models: Sequence[Any], n_paths: Sequence[int],
                    seeds: Sequence[int] | int = 42, steps_per_year: int = 252, *,
                    precision: str = "fp32", greeks: bool = False):
    """An uneven book in one persistent launch: contract i priced under
    models[i] with n_paths[i] paths (no reference counterpart). With
    greeks=True also returns per-contract pathwise Sensitivities (barriers
    smoothed for the derivatives; the prices keep the hard barriers)."""
    n = len(contracts)
    if isinstance(seeds, int):
        seeds = [seeds] * n
    hs = (C.c_void_p * n)(*[c._handle().h.value for c in contracts])
    ms = (_abi.KxModel * n)(*[m._c() for m in models])
    cfgs = (_abi.KxMcConfig * n)(*[_cfg(n_paths[i], seeds[i], steps_per_year, models[i].rate, precision, False)
                                   for i in range(n)])
    out = (_abi.KxPriceResult * n)()
    sens = (_abi.KxSens * n)() if greeks else None
    with _lock:
        _check(_lib().kx_price_portfolio(n, hs, ms, cfgs, out, sens))
    res = [PriceResult(r) for r in out]
    if greeks:
        return res, [Sensitivities(s) for s in sens]
    return res


class Book:
    """A book of contracts priced by replaying one CUDA graph (no reference
    counterpart): contract i under models[i] with n_paths[i] paths and
    seeds[i]. Built once (lowering, tables uploaded, launch shape tuned when
    tune=True, graph captured); price() replays it; set_models() prices the
    same paths under new model parameters. Prices equal Contract.price's."""

    def __init__(self, contracts: Sequence[Contract], models: Sequence[Any], n_paths: Sequence[int],
                 seeds: Sequence[int] | int = 42, steps_per_year: int | Sequence[int] = 252, *,
                 precision: str = "fp32", tune: bool = True):
        n = len(contracts)
        if isinstance(seeds, int):
            seeds = [seeds] * n
        if isinstance(steps_per_year, int):
            steps_per_year = [steps_per_year] * n
        self._contracts = list(contracts)
        self._handles = [c._handle() for c in contracts]  # keep the programs alive
        self._rates = [m.rate for m in models]
        hs = (C.c_void_p * n)(*[h.h.value for h in self._handles])
        ms = (_abi.KxModel * n)(*[m._c() for m in models])
        cfgs = (_abi.KxMcConfig * n)(*[_cfg(n_paths[i], seeds[i], steps_per_year[i], models[i].rate, precision, False)
                                       for i in range(n)])
        self.n = n
        self._b = C.c_void_p()
        with _lock:
            _check(_lib().kx_book_create(n, hs, ms, cfgs, _abi.KX_BOOK_TUNE if tune else 0, C.byref(self._b)))

    def price(self) -> list[PriceResult]:
        out = (_abi.KxPriceResult * self.n)()
        with _lock:
            _check(_lib().kx_book_price(self._b, out))
        return [PriceResult(r) for r in out]

    def set_models(self, models: Sequence[Any]) -> None:
        """New parameters for every contract's model (same kinds and rates
        as at creation)."""
        if [m.rate for m in models] != self._rates:
            raise ValueError("a book keeps each contract's discount rate")
        ms = (_abi.KxModel * self.n)(*[m._c() for m in models])
        with _lock:
            _check(_lib().kx_book_set_models(self._b, ms))

    def info(self) -> dict:
        i = _abi.KxBookInfo()
        _check(_lib().kx_book_get_info(self._b, C.byref(i)))
        g = i.n_groups
        return {"n_contracts": i.n_contracts, "n_groups": g, "n_paths": i.n_paths, "path_steps": i.path_steps,
                "tune_ms": i.tune_ms,
                "groups": [{"kernel": {1: "k_paths", 2: "k_lean", 3: "k_lean/static", 4: "k_lean/static+average"}.get(i.group_kernel[q], "?"),
                            "minb": i.group_minb[q], "item_paths": i.group_item_paths[q],
                            "contracts": i.group_contracts[q]} for q in range(min(g, 4))]}

    def close(self) -> None:
        if self._b:
            _lib().kx_book_free(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_shared_draws(z) -> None:
    """Register host normals (n_paths x draws_per_path, C-contiguous float64
    or float32 numpy array) for shared_draws=True pricing."""
    import numpy as np
    z = np.ascontiguousarray(z)
    if z.ndim != 2:
        raise ValueError("draws must be 2-D (n_paths x draws_per_path)")
    if z.dtype == np.float64:
        st = _lib().kx_set_shared_draws(z.ctypes.data_as(C.POINTER(C.c_double)), None, z.shape[0], z.shape[1])
    elif z.dtype == np.float32:
        st = _lib().kx_set_shared_draws(None, z.ctypes.data_as(C.POINTER(C.c_float)), z.shape[0], z.shape[1])
    else:
        raise TypeError("draws must be float64 or float32")
    _check(st)


def last_launch_stats() -> dict:
    s = _abi.KxLaunchStats()
    _check(_lib().kx_last_launch_stats(C.byref(s)))
    return {k: getattr(s, k) for k, _ in s._fields_}


# ---------------------------------------------------------------------------
# DSL constructors (src/ast.rs:224-335, bindings.rs)
# ---------------------------------------------------------------------------
def zero() -> Contract: return Contract("Zero")
def one(ccy: str = USD) -> Contract: return Contract({"One": ccy})
def give(c: Contract) -> Contract: return -c
def spot(name: str) -> Observable: return Observable({"Spot": name})
def S(name: str) -> Observable: return spot(name)
def const_(x: float) -> Observable: return Observable({"Const": float(x)})
def at(t: float) -> Condition: return Condition({"At": float(t)})
def bool_(b: bool) -> Condition: return Condition({"Bool": bool(b)})
def scale(o, c: Contract) -> Contract: return Contract({"Scale": [_obs(o)._v, c._v]})
def when(cond: Condition, c: Contract) -> Contract: return Contract({"When": [cond._v, c._v]})
def anytime(cond: Condition, c: Contract) -> Contract: return Contract({"Anytime": [cond._v, c._v]})
def until(cond: Condition, c: Contract) -> Contract: return Contract({"Until": [cond._v, c._v]})
def and_(a: Contract, b: Contract) -> Contract: return a + b
def or_(a: Contract, b: Contract) -> Contract: return a.or_(b)


def average(o) -> Observable:
    return Observable({"Average": {"obs": _obs(o)._v, "from_year": None, "to_year": None}})


def average_over(o, from_year: float, to_year: float) -> Observable:
    return Observable({"Average": {"obs": _obs(o)._v, "from_year": float(from_year), "to_year": float(to_year)}})


def running_max(o) -> Observable: return Observable({"RunningMax": _obs(o)._v})
def running_min(o) -> Observable: return Observable({"RunningMin": _obs(o)._v})


# --- products catalogue (src/products.rs) ---
def zero_coupon_bond(ccy: str, t: float) -> Contract:
    return one(ccy) @ at(t)


def european_call(asset: str, k: float, t: float, ccy: str = USD) -> Contract:
    return scale((spot(asset) - const_(k)).max(const_(0.0)), one(ccy)) @ at(t)


def european_put(asset: str, k: float, t: float, ccy: str = USD) -> Contract:
    return scale((const_(k) - spot(asset)).max(const_(0.0)), one(ccy)) @ at(t)


def forward(asset: str, k: float, t: float, ccy: str = USD) -> Contract:
    return scale(spot(asset) - const_(k), one(ccy)) @ at(t)


def straddle(asset: str, k: float, t: float, ccy: str = USD) -> Contract:
    return european_call(asset, k, t, ccy) + european_put(asset, k, t, ccy)


def bull_call_spread(asset: str, k_low: float, k_high: float, t: float, ccy: str = USD) -> Contract:
    return european_call(asset, k_low, t, ccy) + give(european_call(asset, k_high, t, ccy))


def cash_or_nothing_call(asset: str, k: float, payout: float, t: float, ccy: str = USD) -> Contract:
    return when(at(t), when(spot(asset) >= const_(k), scale(const_(payout), one(ccy))))


def up_and_out_call(asset: str, k: float, barrier: float, t: float, ccy: str = USD) -> Contract:
    return until(spot(asset) >= const_(barrier), european_call(asset, k, t, ccy))


def down_and_out_call(asset: str, k: float, barrier: float, t: float, ccy: str = USD) -> Contract:
    return until(spot(asset) <= const_(barrier), european_call(asset, k, t, ccy))


__all__ = [
    "__version__", "KontractError", "Observable", "Condition", "Contract", "GBM", "Model", "PriceResult",
    "Greeks", "Sensitivities", "zero", "one", "give", "S", "spot", "const_", "at", "bool_", "scale", "when", "anytime",
    "until", "and_", "or_", "USD", "EUR", "GBP", "JPY", "average", "average_over", "running_max",
    "running_min", "heston", "zero_coupon_bond", "european_call", "european_put", "forward", "straddle",
    "bull_call_spread", "cash_or_nothing_call", "up_and_out_call", "down_and_out_call", "price_batch",
    "price_american_batch", "GreekSurface", "greek_surface", "fit_gbm_volatility", "CorrelatedGbmN",
    "price_portfolio", "set_shared_draws", "last_launch_stats",
]

from .mlmc import (MlmcConfig, MlmcResult, estimate_variance_at_level, optimal_allocation,  # noqa: E402
                   price_mlmc, price_mlmc_detailed)

__all__ += ["MlmcConfig", "MlmcResult", "price_mlmc", "price_mlmc_detailed", "estimate_variance_at_level",
            "optimal_allocation"]
