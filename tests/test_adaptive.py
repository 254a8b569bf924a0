"""Transient with truncation-error step control (an extension: krets steps at a fixed h).
CPU: the oracle's adaptive transient against closed forms (RC step response) and its own
fixed-step form.  GPU: krets_batch_tran_adaptive against the oracle, instance by
instance: the same accepted time grid (exact binary step factors) and 1e-9 on the states."""
import numpy as np
import pytest

from krets_gb300 import parse_circuit_description
from krets_gb300.table import element_table, is_current_mask

RC = "V1 in 0 0 PULSE(0 1 0 1e-12 1e-12 1 2)\nR1 in out 1000\nC1 out 0 1e-9\n"   # tau = 1 us
RECTIFIER = """* half-wave rectifier with RC load
V1 in 0 0 SIN(0 5 1e6 0 0 0)
D1 in out DMOD
C1 out 0 1e-9
R1 out 0 1000
.model DMOD D (is=1e-12)
"""
TOL = 1e-9


@pytest.mark.parametrize("method", ["be", "tr"])
def test_oracle_adaptive_rc_step_response(oracle_lib, method):
    c = parse_circuit_description(RC)
    t = element_table(c)
    io = c.index_map["V(out)"]
    errs, counts = [], []
    for tol in (1e-2, 1e-3, 1e-4):
        ts, xs = oracle_lib.tran_adaptive(t, c.size, 1e-10, 5e-6, method=method, lte_tol=tol, h_min=1e-15)
        assert ts[0] == 0.0 and ts[-1] == 5e-6 and np.all(np.diff(ts) > 0)
        errs.append(np.abs(xs[:, io] - (1.0 - np.exp(-ts / 1e-6))).max())
        counts.append(len(ts))
    # tighter tolerance: more points, smaller error; all far below the 50 000 fixed steps
    assert counts[0] < counts[1] < counts[2] < 2000
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < (2e-3 if method == "be" else 2e-4)


def test_oracle_adaptive_matches_fixed_steps_on_its_grid(oracle_lib):
    """With h_min = h_max = h0 every step is forced to h0: the adaptive form then equals the
    fixed-step transient (sources at t_n, no lag)."""
    c = parse_circuit_description(RC)
    t = element_table(c)
    h = 1e-8
    ts, xs = oracle_lib.tran_adaptive(t, c.size, h, 2e-6, method="tr", lte_tol=1e9, h_min=h, h_max=h)
    ref = oracle_lib.tran(t, c.size, h, 200, method="tr", lag=False)
    assert len(ts) == 201
    np.testing.assert_allclose(ts, np.arange(201) * h, rtol=1e-12, atol=0)
    np.testing.assert_allclose(xs, ref, rtol=1e-12, atol=1e-15)


def test_oracle_adaptive_errors(oracle_lib):
    from oracle.oracle import OracleError
    c = parse_circuit_description(RC)
    t = element_table(c)
    with pytest.raises(OracleError):          # h_min too large for the edge: step below h_min
        oracle_lib.tran_adaptive(t, c.size, 1e-7, 5e-6, lte_tol=1e-9, h_min=1e-8)
    with pytest.raises(OracleError):          # not enough room for the accepted points
        oracle_lib.tran_adaptive(t, c.size, 1e-10, 5e-6, lte_tol=1e-4, h_min=1e-15, max_points=10)


# ------------------------------------------------------------------------------ GPU
def _rel(x, ref, cur):
    worst = 0.0
    for m, atol in ((cur, 1e-12), (~cur, 1e-6)):
        if m.any():
            r = max(np.abs(ref[..., m]).max(), atol)
            worst = max(worst, np.abs(x[..., m] - ref[..., m]).max() / r)
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["be", "tr"])
def test_gpu_adaptive_monte_carlo_matches_oracle(oracle_lib, method):
    from krets_gb300 import _lib
    from krets_gb300.generators import monte_carlo_values, rlc_ladder
    c = rlc_ladder(20)
    t = element_table(c)
    cur = is_current_mask(c)
    vals = monte_carlo_values(c, 6, seed=21)
    g = _lib.GpuCircuit(t, c.size)
    res, st, rc = g.batch_tran_adaptive(vals, 1e-12, 2e-9, method, lte_tol=1e-4, h_min=1e-18)
    assert rc == 0 and not st.any()
    for i in range(len(vals)):
        ti = t.copy()
        ti["value"] = vals[i]
        ts, xs = oracle_lib.tran_adaptive(ti, c.size, 1e-12, 2e-9, method=method, lte_tol=1e-4, h_min=1e-18)
        tg, xg = res[i]
        assert len(tg) == len(ts), (i, len(tg), len(ts))
        assert np.array_equal(tg, ts)          # the same accepted grid, bit for bit
        assert _rel(xg, xs, cur) < TOL, i
    assert 20 < len(res[0][0]) < 20000


@pytest.mark.gpu
def test_gpu_adaptive_nonlinear_rectifier(oracle_lib):
    from krets_gb300 import _lib
    c = parse_circuit_description(RECTIFIER)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    res, st, rc = g.batch_tran_adaptive(None, 1e-10, 3e-6, "tr", lte_tol=1e-3, h_min=1e-18)
    assert rc == 0 and not st.any()
    ts, xs = oracle_lib.tran_adaptive(t, c.size, 1e-10, 3e-6, method="tr", lte_tol=1e-3, h_min=1e-18)
    tg, xg = res[0]
    assert np.array_equal(tg, ts)
    assert _rel(xg, xs, is_current_mask(c)) < TOL
    vout = xg[:, c.index_map["V(out)"]]
    assert vout.max() > 3.5                    # the load charges towards the peak


@pytest.mark.gpu
def test_gpu_adaptive_reports_limits():
    from krets_gb300 import _lib
    c = parse_circuit_description(RC)
    g = _lib.GpuCircuit(element_table(c), c.size)
    res, st, rc = g.batch_tran_adaptive(None, 1e-10, 5e-6, "tr", lte_tol=1e-4, h_min=1e-15, max_points=10)
    assert rc == 11 and st[0] != 0 and len(res[0][0]) == 10
    res, st, rc = g.batch_tran_adaptive(None, 1e-7, 5e-6, "tr", lte_tol=1e-9, h_min=1e-8)
    assert rc == 4 and st[0] != 0
