"""CPU checks of the oracle's extensions (no reference counterpart): the FP64 adjoint's
gradients — R, C, L and the source-waveform scale — against central finite differences of
the oracle's own transient loss.  The GPU adjoint is held to this oracle elsewhere."""
import numpy as np
import pytest

from krets_gb300.generators import rc_ladder_step, rlc_ladder
from krets_gb300.table import element_table


def _loss(O, t, n, h, steps, method, out):
    x = O.tran(t, n, h, steps, method=method, lag=False)
    return float(np.sum(x[1:, out] ** 2))


def _scaled(t, e, alpha):
    t = t.copy()
    t["value"][e] *= alpha
    if t["wave"][e] in (1, 2):
        t["wp"][e][0] *= alpha
        t["wp"][e][1] *= alpha
    return t


@pytest.mark.parametrize("case", ["rc_tr", "rc_be", "rlc_tr"])
def test_oracle_adjoint_matches_finite_differences(oracle_lib, case):
    if case.startswith("rc"):
        c, out, h, steps = rc_ladder_step(10, seed=7), "V(n10)", 1e-9, 120
    else:
        c, out, h, steps = rlc_ladder(6, rise="50p", width="1n"), "V(n6)", 2e-11, 100
    method = "be" if case.endswith("be") else "tr"
    t = element_table(c)
    n = c.size
    o = c.index_map[out]
    L, g = oracle_lib.adjoint_tran(t, n, h, steps, o, method=method)
    assert abs(L - _loss(oracle_lib, t, n, h, steps, method, o)) <= 1e-13 * L
    rel = 1e-5
    for e in range(len(t)):
        kind = int(t["kind"][e])
        if kind in (1, 2, 3):
            d = rel * t["value"][e]
            tp, tm = t.copy(), t.copy()
            tp["value"][e] += d
            tm["value"][e] -= d
            fd = (_loss(oracle_lib, tp, n, h, steps, method, o) - _loss(oracle_lib, tm, n, h, steps, method, o)) / (2 * d)
        elif kind in (4, 5):
            fd = (_loss(oracle_lib, _scaled(t, e, 1 + rel), n, h, steps, method, o)
                  - _loss(oracle_lib, _scaled(t, e, 1 - rel), n, h, steps, method, o)) / (2 * rel)
        else:
            continue
        assert abs(g[e] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.max(np.abs(g))), (e, kind, g[e], fd)
