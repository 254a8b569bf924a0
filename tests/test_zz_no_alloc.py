"""The allocation-free batched transient (krets_batch_tran_noalloc).

It exists for callers that may not allocate device memory while they run (a host that
owns all GPU memory through its own arena, a real-time loop, work enqueued during a CUDA
graph capture that forbids cudaMalloc).  These tests check, through the C ABI, that it
returns what the ordinary entry point krets_batch_tran returns for the same inputs, on two
calls in a row (the fixed scratch keeps the previous call's contents), and that it refuses
what it cannot do without allocating.  This file is collected last on purpose.
"""
import numpy as np
import pytest

from krets_gb300 import _lib
from krets_gb300.errors import KretsError
from krets_gb300.generators import monte_carlo_values, rlc_ladder
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


@pytest.mark.parametrize("precision", [_lib.PREC_MIXED, _lib.PREC_FP64])
def test_noalloc_matches_batch_tran_on_two_calls(precision):
    c = rlc_ladder(60)
    t = element_table(c)
    n_inst, steps, h = 40, 300, 1e-12
    vals = monte_carlo_values(c, n_inst, seed=21)
    g = _lib.GpuCircuit(t, c.size)
    # the ordinary entry point: result to compare with, and it compiles the programs
    ref = g.batch_tran(vals, h, steps, "tr", lag=False, precision=precision)
    d_vals = _lib.DeviceArray(vals.shape).upload(vals)
    d_out = _lib.DeviceArray((n_inst, steps + 1, c.size))
    d_st = _lib.DeviceArray((n_inst,), np.int32)
    mask = is_current_mask(c)
    for call in range(2):
        d_out.upload(np.full((n_inst, steps + 1, c.size), np.nan))   # every value must be rewritten
        d_st.upload(np.full(n_inst, -1, dtype=np.int32))
        g.batch_tran_noalloc(d_vals, h, steps, d_out, d_st, n_inst, method="tr", lag=False, precision=precision)
        out = d_out.download()
        assert np.all(d_st.download() == 0), call
        assert _rel_err(out, ref, mask) < TOL, call


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
