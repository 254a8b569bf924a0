"""Small cases of the main kernels for profiler captures (one launch each, a few GB on
the device at most), run as

    python -m krets_gb300.profile_cases tran|multi|adjoint|kernels|op|ac|dense

  tran     k_tran_dfd: 2048 instances of the 200-section RLC ladder, TR 1 ps, 200 steps,
           the configuration the autotuner picks for it on GB300 (64 threads per instance,
           factors in global memory, 14 instances per SM: one wave), fixed here so that the
           first k_tran_dfd launch is the measured one
  multi    k_multi_tran (global class): the 152 largest of the first 600 uneven
           netlists, operating point + 100 BE steps at 1 ns
  adjoint  k_adjoint_dfd: 152 instances of the 1000-section RC ladder, TR 1 ns,
           300 steps, checkpoint every 100
  kernels  every other kernel once or a few times, at small sizes: plain OP / DC sweep /
           transient (20 steps), batched OP, DC, AC (FP64 and mixed), transient (FP64,
           mixed, double-float; nonlinear FP64 and mixed), adaptive transient, 64 small
           uneven netlists
  op       k_op: the plain operating point of the 1001-unknown ladder, three times
  ac       k_ac_batch<1>: the 4096-point AC sweep of the 500-section RC ladder (complex64
           factor, complex128 refinement), twice
  dense    k_multi_tran set-up (operating point and transient factorisations) and 100 BE
           steps of one circuit whose LU is a dense block of m - 1 rows, m = 96 .. 352
"""
from __future__ import annotations

import sys

import numpy as np

from . import _lib


def tran():
    from .generators import monte_carlo_values, rlc_ladder
    from .table import element_table
    import os
    os.environ.setdefault("KRETS_GROUP", "64")
    os.environ.setdefault("KRETS_DFD_LU", "global")
    c = rlc_ladder(200)
    t = element_table(c)
    n_inst, steps = 2048, 200
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


def kernels():
    from . import parse_circuit_description
    from .analyses import AcAnalysis, Decade, generate_frequencies
    from .generators import config1_circuit, monte_carlo_values, rc_ladder_ac, rlc_ladder, uneven_table
    from .table import element_table
    c = config1_circuit()
    g = _lib.GpuCircuit(element_table(c), c.size)
    g.op()
    g.batch_op(monte_carlo_values(c, 64, seed=1))
    d = parse_circuit_description("V1 in 0 1\nR1 in a 1000\nD1 a 0 DMOD\nR2 a b 2200\nD2 b 0 DMOD\n"
                                  "R3 b 0 10000\n.model DMOD D (is=1e-12)\n")
    td = element_table(d)
    gd = _lib.GpuCircuit(td, d.size)
    gd.dc(0, -0.5, 3.0, 0.05)
    gd.batch_dc(monte_carlo_values(d, 16, seed=2), 0, -0.5, 3.0, 0.05)
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):   # nonlinear: Newton per step
        gd.batch_tran(monte_carlo_values(d, 16, seed=5), 1e-9, 50, "be", precision=prec)
    a = rc_ladder_ac(500)
    ga = _lib.GpuCircuit(element_table(a), a.size)
    f = np.array(generate_frequencies(AcAnalysis(Decade(455), 1.0, 1e9)))[::16]
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        ga.batch_ac(None, f, precision=prec)
    r = rlc_ladder(200)
    tr = element_table(r)
    gr = _lib.GpuCircuit(tr, r.size)
    gr.tran(1e-12, 20, "tr")
    vals = monte_carlo_values(r, 152, seed=3)
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED, _lib.PREC_DF):
        out = _lib.DeviceArray((152, 201, r.size))
        gr.batch_tran(vals, 1e-12, 200, "tr", lag=False, precision=prec, out=out)
        del out
    s = rlc_ladder(20)
    gs = _lib.GpuCircuit(element_table(s), s.size)
    gs.batch_tran_adaptive(monte_carlo_values(s, 8, seed=4), 1e-12, 2e-9, "tr", lte_tol=1e-4, h_min=1e-18)
    tabs = [uneven_table(i) for i in range(64)]
    m = _lib.MultiCircuit([t for t, _ in tabs], [n for _, n in tabs], method="be", h=1e-9)
    out = _lib.DeviceArray(m.total(200))
    m.tran(200, out=out)
    gr.flush_l2()
    return m.timing()


def op():
    from .generators import config1_circuit
    from .table import element_table
    c = config1_circuit()
    g = _lib.GpuCircuit(element_table(c), c.size)
    for _ in range(3):
        g.op()
    return g.timing()


def ac():
    from .analyses import AcAnalysis, Decade, generate_frequencies
    from .generators import rc_ladder_ac
    from .table import element_table
    c = rc_ladder_ac()
    g = _lib.GpuCircuit(element_table(c), c.size)
    f = np.array(generate_frequencies(AcAnalysis(Decade(455), 1.0, 1e9)))
    out = _lib.DeviceArray((1, len(f), c.size, 2))
    for _ in range(2):
        g.batch_ac(None, f, precision=_lib.PREC_MIXED, out=out)
    return g.timing()


def dense():
    from .generators import dense_block_table
    rows = []
    for m in (96, 128, 192, 256, 352):
        t, n = dense_block_table(m)
        meta = _lib.symbolic_export(t, n, _lib.MODE_TRAN, "be", 1e-9, ordering=0x1ff)["meta"]
        mc = _lib.MultiCircuit([t], [n], method="be", h=1e-9)
        times = []
        for steps in (0, 0, 100, 100):
            out = _lib.DeviceArray(mc.total(steps))
            mc.tran(steps, out=out)
            times.append(mc.timing()[0])
            del out
        setup, with_steps = min(times[:2]), min(times[2:])
        rows.append((m, int(meta[8]), setup, (with_steps - setup) / 100))
        print(f"m {m}: dense block {int(meta[8])}, set-up + OP {setup:.3f} ms, "
              f"per BE step {(with_steps - setup) / 100 * 1e3:.1f} us", flush=True)
        mc.close()
    return rows[-1][2], rows[-1][2]


CASES = {"tran": tran, "multi": multi, "adjoint": adjoint, "kernels": kernels, "op": op, "ac": ac, "dense": dense}

if __name__ == "__main__":
    k, c = CASES[sys.argv[1]]()
    print(f"{sys.argv[1]}: kernel {k:.3f} ms, call {c:.3f} ms")
