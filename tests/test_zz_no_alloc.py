"""The allocation-free batched transient (krets_batch_tran_noalloc).

It exists for callers that may not allocate device memory while they run (a host that
owns all GPU memory through its own arena, a real-time loop, work enqueued during a CUDA
graph capture that forbids cudaMalloc).  These tests check, through the C ABI, that for
every precision it returns what the ordinary entry point krets_batch_tran returns for the
same inputs — bit for bit, since both run the same kernels with the same parameters — on
two calls in a row (the fixed scratch keeps the previous call's contents), and that it
refuses what it cannot do without allocating.  This file is collected last on purpose.
"""
import numpy as np
import pytest

from krets_gb300 import _lib, parse_circuit_description
from krets_gb300.errors import KretsError
from krets_gb300.generators import monte_carlo_values, rc_ladder_step, rlc_ladder
from krets_gb300.table import element_table, is_current_mask

pytestmark = pytest.mark.gpu

TOL = 1e-9        # the tolerance of the other GPU parity tests


def _rel_err(x, ref, mask):
    if not (np.all(np.isfinite(x)) and np.all(np.isfinite(ref))):
        return np.inf
    worst = 0.0
    for m in (mask, ~mask):
        r = np.abs(ref[..., m]).max()
        worst = max(worst, np.abs(x[..., m] - ref[..., m]).max() / r)
    return worst


def _check_two_calls(g, c, vals, h, steps, method, lag, precision):
    n_inst = len(vals)
    # the ordinary entry point: the result to compare with (it also compiles the programs
    # and, for the double-float engine, caches the autotuned group size)
    ref = g.batch_tran(vals, h, steps, method, lag=lag, precision=precision)
    d_vals = _lib.DeviceArray(vals.shape).upload(vals)
    d_out = _lib.DeviceArray((n_inst, steps + 1, c.size))
    d_st = _lib.DeviceArray((n_inst,), np.int32)
    mask = is_current_mask(c)
    for call in range(2):
        d_out.upload(np.full((n_inst, steps + 1, c.size), np.nan))   # every value must be rewritten
        d_st.upload(np.full(n_inst, -1, dtype=np.int32))
        g.batch_tran_noalloc(d_vals, h, steps, d_out, d_st, n_inst, method=method, lag=lag, precision=precision)
        out = d_out.download()
        assert np.all(d_st.download() == 0), call
        assert _rel_err(out, ref, mask) < TOL, call
        np.testing.assert_array_equal(out, ref, err_msg=f"call {call}")


@pytest.mark.parametrize("precision", [_lib.PREC_MIXED, _lib.PREC_FP64, _lib.PREC_DF])
def test_noalloc_matches_batch_tran_on_two_calls(precision):
    c = rlc_ladder(60)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    vals = monte_carlo_values(c, 40, seed=21)
    _check_two_calls(g, c, vals, 1e-12, 300, "tr", False, precision)


@pytest.mark.parametrize("precision", [_lib.PREC_MIXED, _lib.PREC_DF])
def test_noalloc_nonlinear_matches_batch_tran(precision):
    # a diode rectifier: both precisions run the FP32-factor Newton engine with FP64
    # fallback factors taken from the fixed scratch
    c = parse_circuit_description(
        "V1 in 0 SIN(0 5 60 0 0 0)\nR1 in a 10\nD1 a out DMOD\nC1 out 0 10u\nR2 out 0 1k\n"
        ".model DMOD D (is=1e-12)\n")
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    vals = monte_carlo_values(c, 8, seed=5)
    _check_two_calls(g, c, vals, 50e-6, 200, "be", True, precision)


def test_noalloc_refuses_what_needs_allocation():
    c = rlc_ladder(10)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    d_out = _lib.DeviceArray((2, 11, c.size))
    d_st = _lib.DeviceArray((2,), np.int32)
    # no compiled program for this step yet: compiling would allocate
    with pytest.raises(KretsError):
        g.batch_tran_noalloc(None, 1e-12, 10, d_out, d_st, 2)
    g.batch_tran(None, 1e-12, 10, "tr", lag=False, n_inst=2)
    g.batch_tran_noalloc(None, 1e-12, 10, d_out, d_st, 2)
    # host buffers would need staging copies on the device
    with pytest.raises(KretsError):
        g.batch_tran_noalloc(None, 1e-12, 10, np.zeros((2, 11, c.size)), d_st, 2)
    # an unknown precision
    with pytest.raises(KretsError):
        g.batch_tran_noalloc(None, 1e-12, 10, d_out, d_st, 2, precision=7)


def test_noalloc_refuses_a_circuit_that_needs_global_workspaces():
    # 3000 RC sections: krets_batch_tran runs it with global-memory workspaces, which the
    # allocation-free entry cannot have
    c = rc_ladder_step(3000)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    steps = 4
    ref = g.batch_tran(None, 1e-9, steps, "tr", lag=False, precision=_lib.PREC_DF, n_inst=2)
    assert np.all(np.isfinite(ref))
    d_out = _lib.DeviceArray((2, steps + 1, c.size))
    d_st = _lib.DeviceArray((2,), np.int32)
    for prec in (_lib.PREC_DF, _lib.PREC_MIXED, _lib.PREC_FP64):
        with pytest.raises(KretsError, match="too large"):
            g.batch_tran_noalloc(None, 1e-9, steps, d_out, d_st, 2, method="tr", lag=False, precision=prec)
