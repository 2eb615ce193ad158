"""Per-path parity of FP32 path arithmetic against the FP64 oracle.

The reference computes in FP64; the engine's FP32 mode rounds every step of a
path to FP32, so its simulated spot differs from the FP64 one by about 1e-7
relative (at most 16 FP32 ulps on a 365-step path, measured). The required
agreement is 1e-5 relative, checked on every path in one of two forms:

  forward error   |pv_gpu - pv_ref| <= 1e-5 |pv_ref| (+ 1e-9 absolute for
                  paths worth 0), or
  backward error  pv_gpu lies between the oracle's values of the same path
                  (same normals) started from s0 (1 - 1e-5) and s0 (1 + 1e-5),
                  widened by 1e-5 of their size: the FP32 result is the exact
                  reference result for a spot perturbed by at most 1e-5.

The second form is what a path next to a kink needs: a call whose spot ends
0.1 % above the strike has a payoff 1000 times more sensitive to the spot
than to itself, so a 1e-7 relative spot difference is a 1e-4 relative payoff
difference; a barrier decision taken within 1e-7 of the barrier can flip.
Such paths are not excused: each must still equal the reference's value for
a spot within 1e-5. Both GBM and Heston spots scale with s0 (their log-spot
dynamics do not depend on it), so the perturbed runs move the whole path.
"""
from __future__ import annotations

import numpy as np

REL = 1e-5


def perturbed_oracle(orc, js, model, rel=REL, **kw):
    """The oracle's per-path values of the contract started from s0 (1 - rel)
    and s0 (1 + rel), on the same draws."""
    out = []
    src = model._c()
    for f in (1.0 - rel, 1.0 + rel):
        cm = type(src)()  # a copy: some models hand out their own structure
        for name, _ in src._fields_:
            setattr(cm, name, getattr(src, name))
        cm.s0 = src.s0 * f
        _, pv = orc.price(js, cm, rate=model.rate, per_path=True, **kw)
        out.append(np.asarray(pv))
    return out


def fp32_check(pv, ref, ref_dn, ref_up, rel=REL):
    """(passed mask, forward mask): forward = within rel of the FP64 value;
    passed = forward or inside the perturbed-spot envelope."""
    pv, ref = np.asarray(pv), np.asarray(ref)
    fwd = np.abs(pv - ref) <= rel * np.abs(ref) + 1e-9
    lo = np.minimum(np.minimum(ref_dn, ref_up), ref)
    hi = np.maximum(np.maximum(ref_dn, ref_up), ref)
    slack = rel * np.maximum(np.abs(lo), np.abs(hi)) + 1e-9
    back = (pv >= lo - slack) & (pv <= hi + slack)
    return fwd | back, fwd
