"""Small cases of the main kernels for profiler captures (one launch each, a few GB on
the device at most), run as

    python -m krets_gb300.profile_cases tran|multi|adjoint

  tran     k_tran_dfd: 304 instances of the 200-section RLC ladder, TR 1 ps, 1000 steps
  multi    k_multi_tran (global class): the 152 largest of the first 600 uneven
           netlists, operating point + 100 BE steps at 1 ns
  adjoint  k_adjoint_dfd: 152 instances of the 1000-section RC ladder, TR 1 ns,
           300 steps, checkpoint every 100
"""
from __future__ import annotations

import sys

import numpy as np

from . import _lib


def tran():
    from .generators import monte_carlo_values, rlc_ladder
    from .table import element_table
    c = rlc_ladder(200)
    t = element_table(c)
    n_inst, steps = 304, 1000
    vals = monte_carlo_values(c, n_inst, sigma=0.1, seed=3)
    g = _lib.GpuCircuit(t, c.size)
    out = _lib.DeviceArray((n_inst, steps + 1, c.size))
    dv = _lib.DeviceArray(vals.shape).upload(vals)
    g.batch_tran(dv, 1e-12, steps, "tr", lag=False, precision=_lib.PREC_DF, out=out, n_inst=n_inst)
    return g.timing()


def multi():
    from .generators import uneven_table
    tabs = [uneven_table(i) for i in range(600)]
    big = sorted(range(600), key=lambda i: -tabs[i][1])[:152]
    m = _lib.MultiCircuit([tabs[i][0] for i in big], [tabs[i][1] for i in big], method="be", h=1e-9)
    out = _lib.DeviceArray(m.total(100))
    m.tran(100, out=out)
    return m.timing()


def adjoint():
    from .generators import rc_ladder_step
    from .table import element_table
    c = rc_ladder_step(1000)
    t = element_table(c)
    vals = np.tile(t["value"], (152, 1))
    g = _lib.GpuCircuit(t, c.size)
    g.adjoint_tran(vals, 1e-9, 300, c.index_map["V(n20)"], checkpoint_every=100)
    return g.timing()


CASES = {"tran": tran, "multi": multi, "adjoint": adjoint}

if __name__ == "__main__":
    k, c = CASES[sys.argv[1]]()
    print(f"{sys.argv[1]}: kernel {k:.3f} ms, call {c:.3f} ms")
