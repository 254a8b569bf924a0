"""Error measures of a result against the oracle (test infrastructure, the checker's side).

Two measures, both reported for every parity claim:

* norm-wise: max over the two quantity classes (node voltages, branch currents) of
  max|x - x_ref| / max|x_ref| over that class;
* element-wise, in the form of the reference's own convergence test
  (crates/krets-solver/src/solver.rs:96-103: |x - x_prev| <= reltol * scale + atol):
  every value must satisfy |x - x_ref| <= 1e-9 * |x_ref| + floor.  The floor is the
  larger of
    - the reference's absolute tolerances (1e-6 V, 1e-12 A at reltol 1e-3) scaled by the
      same factor as the relative one, 1e-9 / 1e-3: 1e-12 V and 1e-18 A, and
    - 1e-12 of the largest magnitude in the value's class: FP64 rounding noise.  A value
      that is zero in exact arithmetic (a current through a branch that carries none,
      a node the wavefront has not reached) comes out of any two FP64 eliminations as
      noise of a few ulps of the class's largest values, different in each; the
      reference's own results carry that noise too.
  It is returned as max |x - x_ref| / (|x_ref| + floor / 1e-9), so that "<= 1e-9" is the
  test: every value larger than 1e-3 of its class's scale (or than 1e-3 V, 1e-9 A) is
  held to 1e-9 relative, and smaller values to the floor absolutely.
"""
from __future__ import annotations

import numpy as np

RTOL = 1e-9
FLOOR_V = 1e-6 * (RTOL / 1e-3)     # the reference's voltage atol scaled to 1e-9: 1e-12 V
FLOOR_I = 1e-12 * (RTOL / 1e-3)    # the reference's current atol scaled to 1e-9: 1e-18 A
NOISE = 1e-12                      # FP64 rounding noise, relative to the class's largest value


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
    """max over every value of |x - ref| / (|ref| + floor / 1e-9), the floor by the
    unknown's class: max(1e-12 V or 1e-18 A, 1e-12 x the class's largest |ref|)
    (arrays [..., n], real or complex)."""
    x = np.asarray(x)
    ref = np.asarray(ref)
    if not (np.all(np.isfinite(x)) and np.all(np.isfinite(ref))):
        return np.inf
    worst = 0.0
    for m, atol in ((cur_mask, FLOOR_I), (~cur_mask, FLOOR_V)):
        if not m.any():
            continue
        r = ref[..., m]
        floor = max(atol, NOISE * float(np.abs(r).max()))
        e = np.abs(x[..., m] - r) / (np.abs(r) + floor / RTOL)
        worst = max(worst, float(e.max()))
    return worst


def both(x, ref, cur_mask) -> tuple[float, float]:
    return normwise_err(x, ref, cur_mask), elementwise_err(x, ref, cur_mask)
