"""Error measures of a result against the oracle (test infrastructure, the checker's side).

Two measures, both reported for every parity claim:

* norm-wise: max over the two quantity classes (node voltages, branch currents) of
  max|x - x_ref| / max|x_ref| over that class;
* element-wise, in the form of the reference's own convergence test
  (crates/krets-solver/src/solver.rs:96-103: |x - x_prev| <= reltol * scale + atol, atol
  1e-6 for voltages and 1e-12 for currents, reltol 1e-3): every value must satisfy
  |x - x_ref| <= 1e-9 * |x_ref| + floor, where the floors are those absolute tolerances
  scaled by the same factor as the relative one (1e-9 / 1e-3): 1e-12 V and 1e-18 A.
  It is returned as max |x - x_ref| / (|x_ref| + floor / 1e-9), so that "<= 1e-9" is the
  test; values far below the floor (a ladder section the wavefront has not reached) count
  only through their absolute error.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-9
FLOOR_V = 1e-6 * (RTOL / 1e-3)     # the reference's voltage atol scaled to 1e-9: 1e-12 V
FLOOR_I = 1e-12 * (RTOL / 1e-3)    # the reference's current atol scaled to 1e-9: 1e-18 A


def normwise_err(x, ref, cur_mask) -> float:
    """max over {voltages, currents} of max|x - ref| / max|ref| (arrays [..., n])."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    if not (np.all(np.isfinite(x)) and np.all(np.isfinite(ref))):
        return np.inf
    worst = 0.0
    for m in (cur_mask, ~cur_mask):
        if not m.any():
            continue
        r = np.abs(ref[..., m]).max()
        d = np.abs(x[..., m] - ref[..., m]).max()
        worst = max(worst, d / r if r > 0 else d)
    return float(worst)


def elementwise_err(x, ref, cur_mask) -> float:
    """max over every value of |x - ref| / (|ref| + floor / 1e-9), floor 1e-12 V or 1e-18 A
    by the unknown's class (arrays [..., n], real or complex)."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    if not (np.all(np.isfinite(x)) and np.all(np.isfinite(ref))):
        return np.inf
    worst = 0.0
    for m, floor in ((cur_mask, FLOOR_I), (~cur_mask, FLOOR_V)):
        if not m.any():
            continue
        r = ref[..., m]
        e = np.abs(x[..., m] - r) / (np.abs(r) + floor / RTOL)
        worst = max(worst, float(e.max()))
    return worst


def both(x, ref, cur_mask) -> tuple[float, float]:
    return normwise_err(x, ref, cur_mask), elementwise_err(x, ref, cur_mask)
