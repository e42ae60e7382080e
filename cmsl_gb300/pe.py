"""Remanent polarization and coercive field of a recorded P-E loop.

The reference prints the loop (HZO_Code_github/src/evolve.cu:391-400) and
leaves its analysis to the user; these are the quantities the FP32-refined
path is held to against FP64:

* Pr+ / Pr-: the average polarization at the E = 0 crossings of the loop
  with the field decreasing / increasing, interpolated linearly between the
  two rows around the crossing; Pr = (Pr+ - Pr-) / 2;
* Ec+ / Ec-: the field at the P = 0 crossings with the polarization
  increasing / decreasing, interpolated the same way; Ec = (Ec+ - Ec-) / 2.

When a loop crosses more than once in one direction (several periods), the
last crossing is used.
"""
from __future__ import annotations

import math

import numpy as np


def _crossings(x: np.ndarray, y: np.ndarray, falling: bool) -> list[float]:
    """y interpolated where x crosses 0 (falling: from > 0 to <= 0)."""
    out = []
    for i in range(x.size - 1):
        a, b = x[i], x[i + 1]
        hit = (a > 0.0 >= b) if falling else (a < 0.0 <= b)
        if hit:
            t = a / (a - b)
            out.append(float(y[i] + t * (y[i + 1] - y[i])))
    return out


def loop_metrics(E, P) -> dict:
    """Pr and Ec of one recorded loop: E and P are the rows' field and
    average polarization in the order they were written."""
    E = np.asarray(E, np.float64)
    P = np.asarray(P, np.float64)
    if E.shape != P.shape or E.ndim != 1:
        raise ValueError("E and P must be 1-D arrays of the same length")
    pr_p = _crossings(E, P, falling=True)
    pr_m = _crossings(E, P, falling=False)
    ec_m = _crossings(P, E, falling=True)
    ec_p = _crossings(P, E, falling=False)
    nan = math.nan
    m = {"Pr_plus": pr_p[-1] if pr_p else nan, "Pr_minus": pr_m[-1] if pr_m else nan,
         "Ec_plus": ec_p[-1] if ec_p else nan, "Ec_minus": ec_m[-1] if ec_m else nan}
    m["Pr"] = 0.5 * (m["Pr_plus"] - m["Pr_minus"])
    m["Ec"] = 0.5 * (m["Ec_plus"] - m["Ec_minus"])
    return m


def relative_errors(test: dict, ref: dict, keys=("Pr", "Ec", "Pr_plus", "Pr_minus", "Ec_plus", "Ec_minus")) -> dict:
    """|test - ref| / |ref| per key."""
    out = {}
    for k in keys:
        r = ref[k]
        out[k] = abs(test[k] - r) / abs(r) if r not in (0.0,) and math.isfinite(r) else math.nan
    return out


def field_errors(test, ref) -> dict:
    """Max-abs and relative-L2 differences of stacked field arrays."""
    t = np.concatenate([np.ravel(a) for a in test])
    r = np.concatenate([np.ravel(a) for a in ref])
    d = t - r
    nr = float(np.linalg.norm(r))
    return {"max_abs": float(np.abs(d).max()), "rel_l2": float(np.linalg.norm(d)) / nr if nr > 0 else math.nan,
            "max_ref": float(np.abs(r).max())}
