"""NMOS with resolved node lookups (KRETS_FLAG_NMOS_RESOLVED).  The reference looks the
NMOS terminals up by bare node name and stamps nothing (stampable.rs:842-844); with the
flag the device stamps the reference's own entries (stampable.rs:846-866, rhs :870-899)
with the level-1 model of nmosfet.rs:51-103.  The reference cannot run here, so the
oracle's stamp is pinned against an independent dense restatement of those lines; the GPU
is then held to the oracle (1e-9, as the other parity tests)."""
import json
from pathlib import Path

import numpy as np
import pytest

from krets_gb300 import parse_circuit_description
from krets_gb300.table import element_table, is_current_mask

GOLDEN = Path(__file__).parent / "golden" / "reference_cases.json"

# lambda = 0: with lambda > 0 the level-1 i_d of nmosfet.rs jumps at the linear/saturation
# boundary (the (1 + lambda v_ds) factor only in saturation), and Newton may cycle there
# until maximum_iterations -- on the oracle as on the device -- for some parameter sets
COMMON_SOURCE = """* NMOS common-source stage, gate pulse, capacitive load
VDD vdd 0 DC 2
VIN g 0 DC 0 PULSE(0 2 1e-9 1e-9 1e-9 5e-9 2e-8)
RD vdd d 2000
MN1 d g 0 0 NMOD
CD d 0 1e-12
RL d out 500
CL out 0 2e-12
.model NMOD NMOS (vto=0.5 kp=2e-4 lambda=0 w=4e-6 l=1e-6)
"""


def _inverter():
    fx = json.loads(GOLDEN.read_text())["parquet"]["inverter_dc"]
    return parse_circuit_description(fx["netlist"])


def _nmos_lin(wp, vg, vs, vd):
    """nmosfet.rs:51-103 (beta = kp * (w / l), models/nmosfet.rs:41-43)."""
    vto, kp, lam, w, l = wp[:5]
    beta = kp * (w / l)
    vgs, vds = vg - vs, vd - vs
    if vgs <= vto:
        return 0.0, 0.0, 0.0, vgs, vds
    if 0.0 <= vds <= vgs - vto:
        return beta * vds, beta * (vgs - vto - vds), beta * ((vgs - vto) * vds - vds * vds / 2.0), vgs, vds
    if vds >= vgs - vto and vds >= 0.0:
        ov = vgs - vto
        return (beta * ov * (1.0 + lam * vds), (beta / 2.0) * lam * (ov * ov),
                (beta / 2.0) * (ov * ov) * (1.0 + lam * vds), vgs, vds)
    return 0.0, 0.0, 0.0, vgs, vds


def _dense_dc_sweep(t, n, sweep, start, stop, step, cur):
    """dc.rs:14-124 over a dense matrix: warm start, the "step" key, solver.rs:76-104's
    convergence test (reltol 1e-3, 1e-12 for currents, 1e-6 otherwise).  R, V, NMOS only."""
    npts = int(abs((stop - start) / step)) + 1
    out = np.zeros((npts, n))
    x = None
    for i in range(npts):
        t = t.copy()
        t["value"][sweep] = start + i * step
        guess, gstep = x, i - 1.0
        for it in range(300):
            A = np.zeros((n, n))
            b = np.zeros(n)
            for e in t:
                k, p, m, br = int(e["kind"]), int(e["p"]), int(e["m"]), int(e["b"])
                if k == 1:
                    g = 1.0 / e["value"]
                    for r, c, s in ((p, p, 1), (m, m, 1), (p, m, -1), (m, p, -1)):
                        if r >= 0 and c >= 0:
                            A[r, c] += s * g
                elif k == 4:
                    for r, c, s in ((p, br, 1), (br, p, 1), (m, br, -1), (br, m, -1)):
                        if r >= 0 and c >= 0:
                            A[r, c] += s
                    b[br] += e["value"]
                elif k == 7:
                    gi = int(e["g"])
                    v = (lambda j: 0.0 if (guess is None or j < 0) else guess[j])
                    gm, gds, idd, vgs, vds = _nmos_lin(e["wp"], v(gi), v(m), v(p))
                    for r, c, val in ((p, p, gds), (m, m, gds + gm), (p, m, -(gds + gm)), (m, p, gds + gm),
                                      (m, gi, gm), (p, gi, gm)):
                        if r >= 0 and c >= 0:
                            A[r, c] += val
                    ieq = idd - gds * vds - gm * vgs
                    if m >= 0:
                        b[m] += ieq
                    if p >= 0:
                        b[p] -= ieq
                else:
                    raise AssertionError(k)
            xn = np.linalg.solve(A, b)
            if guess is not None:
                tol = 1e-3 * np.maximum(np.abs(xn), np.abs(guess)) + np.where(cur, 1e-12, 1e-6)
                step_ok = abs(i - gstep) <= 1e-3 * max(abs(i), abs(gstep)) + 1e-6
                if np.all(np.abs(xn - guess) <= tol) and step_ok:
                    break
            guess, gstep = xn, float(i)
        x = xn
        out[i] = x
    return out


def test_oracle_resolved_nmos_matches_dense_restatement(oracle_lib):
    c = _inverter()
    cur = is_current_mask(c)
    t = element_table(c, nmos_resolved=True)
    sweep = next(k for k, el in enumerate(c.elements) if el.identifier == "V1")
    got = oracle_lib.dc(t, c.size, sweep, 0.0, 1.0, 0.01)
    ref = _dense_dc_sweep(t, c.size, sweep, 0.0, 1.0, 0.01, cur)
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-15)
    # the device conducts above threshold: V(S) moves, unlike the reference's no-stamp result
    assert abs(got[-1, c.index_map["V(S)"]]) > 1e-3


def test_default_keeps_the_reference_no_stamp(oracle_lib):
    c = _inverter()
    sweep = next(k for k, el in enumerate(c.elements) if el.identifier == "V1")
    x = oracle_lib.dc(element_table(c), c.size, sweep, 0.0, 1.0, 0.01)
    assert np.all(x[:, c.index_map["V(S)"]] == 0.0)


def test_program_wires_the_nmos_coefficient_slots(oracle_lib):
    """The exported DC program, walked by the CPU emulator with the extended coefficient
    vector (slot e = g_ds + g_m, then g_ds, g_m after the elements' own slots), performs
    the same Newton step as the dense restatement from the same guess."""
    from program_emulator import element_coefs, emulate, export
    c = _inverter()
    n = c.size
    t = element_table(c, nmos_resolved=True)
    t["value"][next(k for k, el in enumerate(c.elements) if el.identifier == "V1")] = 0.8
    guess = oracle_lib.op(t, n) + 0.01   # a point where the device conducts
    ca, cb = element_coefs(t, 0)
    ne = len(t)
    ca = np.concatenate([ca, np.zeros(2, dtype=complex)])
    e = next(k for k, el in enumerate(c.elements) if el.kind == 7)
    gm, gds, idd, vgs, vds = _nmos_lin(t["wp"][e], guess[t["g"][e]], guess[t["m"][e]], guess[t["p"][e]])
    assert gm > 0 and gds > 0
    ca[e], ca[ne], ca[ne + 1] = gds + gm, gds, gm
    cb[e] = idd - gds * vds - gm * vgs
    x = emulate(export(t, n, 0), t, n, ca, cb)
    # dense: one iteration of _dense_dc_sweep's body from `guess`
    A = np.zeros((n, n))
    b = np.zeros(n)
    for k, el in enumerate(t):
        p, m, br = int(el["p"]), int(el["m"]), int(el["b"])
        if el["kind"] == 1:
            for r, cc, sg in ((p, p, 1), (m, m, 1), (p, m, -1), (m, p, -1)):
                if r >= 0 and cc >= 0:
                    A[r, cc] += sg / el["value"]
        elif el["kind"] == 4:
            for r, cc, sg in ((p, br, 1), (br, p, 1), (m, br, -1), (br, m, -1)):
                if r >= 0 and cc >= 0:
                    A[r, cc] += sg
            b[br] += el["value"]
    d, src, g = int(t["p"][e]), int(t["m"][e]), int(t["g"][e])
    for r, cc, val in ((d, d, gds), (src, src, gds + gm), (d, src, -(gds + gm)), (src, d, gds + gm),
                       (src, g, gm), (d, g, gm)):
        if r >= 0 and cc >= 0:
            A[r, cc] += val
    b[src] += cb[e]
    b[d] -= cb[e]
    np.testing.assert_allclose(x.real, np.linalg.solve(A, b), rtol=1e-12, atol=1e-15)


def test_flag_only_on_nmos():
    c = parse_circuit_description(COMMON_SOURCE)
    t = element_table(c, nmos_resolved=True)
    flagged = (t["flags"] & 2) != 0
    assert flagged.tolist() == [el.kind == 7 for el in c.elements]


# ------------------------------------------------------------------------------ GPU
def _rel(x, ref, cur):
    """Norm-wise relative error per quantity class; a class whose values are all below the
    reference's absolute tolerance (1e-12 A, 1e-6 V: config.rs:26-36) is scaled by it (an
    off device carries a branch current of 0 that the oracle rounds to ~1e-19)."""
    worst = 0.0
    for m, atol in ((cur, 1e-12), (~cur, 1e-6)):
        if m.any():
            r = max(np.abs(ref[..., m]).max(), atol)
            d = np.abs(x[..., m] - ref[..., m]).max()
            worst = max(worst, d / r)
    return worst


@pytest.mark.gpu
def test_gpu_resolved_nmos_dc_and_op(oracle_lib):
    from krets_gb300 import _lib
    from krets_gb300.analyses import DcAnalysis
    from krets_gb300.solver import Solver
    c = _inverter()
    cur = is_current_mask(c)
    t = element_table(c, nmos_resolved=True)
    sweep = next(k for k, el in enumerate(c.elements) if el.identifier == "V1")
    res = Solver(c, nmos_resolved=True).solve(DcAnalysis("V1", 0.0, 1.0, 0.01))
    ref = oracle_lib.dc(t, c.size, sweep, 0.0, 1.0, 0.01)
    assert _rel(res.array, ref, cur) < 1e-9
    c2 = parse_circuit_description(COMMON_SOURCE)
    t2 = element_table(c2, nmos_resolved=True)
    t2["value"][[el.identifier for el in c2.elements].index("VIN")] = 1.5   # gate above threshold
    x, _ = _lib.GpuCircuit(t2, c2.size).op()
    assert _rel(x, oracle_lib.op(t2, c2.size), is_current_mask(c2)) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["be", "tr"])
def test_gpu_resolved_nmos_transient(oracle_lib, method):
    from krets_gb300 import _lib
    from krets_gb300.generators import monte_carlo_values
    c = parse_circuit_description(COMMON_SOURCE)
    cur = is_current_mask(c)
    t = element_table(c, nmos_resolved=True)
    g = _lib.GpuCircuit(t, c.size)
    h, n_steps = 1e-10, 300
    ref = oracle_lib.tran(t, c.size, h, n_steps, method=method)
    vd = ref[:, c.index_map["V(d)"]]
    assert vd.max() - vd.min() > 0.5   # the device switches
    assert _rel(g.tran(h, n_steps, method), ref, cur) < 1e-9
    vals = monte_carlo_values(c, 8, seed=11)
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        xb = g.batch_tran(vals, h, n_steps, method, precision=prec)
        for i in range(len(vals)):
            ti = t.copy()
            ti["value"] = vals[i]
            assert _rel(xb[i], oracle_lib.tran(ti, c.size, h, n_steps, method=method), cur) < 1e-9, (prec, i)


@pytest.mark.gpu
def test_gpu_resolved_nmos_ac_is_not_implemented():
    from krets_gb300 import _lib
    from krets_gb300.errors import KretsError
    c = _inverter()
    g = _lib.GpuCircuit(element_table(c, nmos_resolved=True), c.size)
    with pytest.raises(KretsError):
        g.ac(np.array([1.0, 10.0]))
