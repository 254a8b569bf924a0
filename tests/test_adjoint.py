"""Adjoint sensitivities of a batched linear transient (no counterpart in the reference).

The loss of an instance is sum_{n=1..N} x_out(t_n)^2.  The GPU gradient (discrete adjoint
with checkpointed reverse sweep) is checked against central finite differences of the same
loss computed by the CPU oracle's transient (FP64), and the GPU loss against the oracle's.
"""
import numpy as np
import pytest

from krets_gb300 import _lib
from krets_gb300.errors import KretsError
from krets_gb300.generators import monte_carlo_values, rc_ladder_step, rlc_ladder
from krets_gb300.netlist import parse_circuit_description
from krets_gb300.table import element_table

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-6     # norm-wise, against central differences
LOSS_TOL = 1e-12


def _oracle_loss(oracle_lib, table, n, vals, h, steps, method, out):
    t = table.copy()
    t["value"] = vals
    x = oracle_lib.tran(t, n, h, steps, method=method, lag=False)
    return float(np.sum(x[1:, out] ** 2))


def _fd_grad(oracle_lib, table, n, vals, h, steps, method, out, rel=1e-5):
    g = np.zeros(len(vals))
    for e in range(len(vals)):
        if int(table["kind"][e]) not in (1, 2, 3):
            continue
        d = rel * vals[e]
        vp, vm = vals.copy(), vals.copy()
        vp[e] += d
        vm[e] -= d
        g[e] = (_oracle_loss(oracle_lib, table, n, vp, h, steps, method, out)
                - _oracle_loss(oracle_lib, table, n, vm, h, steps, method, out)) / (2 * d)
    return g


def _scaled_source(table, e, alpha):
    """The table with source e's transient value scaled by alpha (PULSE V1/V2, SIN VO/VA,
    and the DC value)."""
    t = table.copy()
    t["value"][e] *= alpha
    if t["wave"][e] in (1, 2):
        t["wp"][e][0] *= alpha
        t["wp"][e][1] *= alpha
    return t


def _fd_source(oracle_lib, table, n, vals, h, steps, method, out, e, rel=1e-5):
    t = table.copy()
    t["value"] = vals
    lp = _oracle_loss(oracle_lib, _scaled_source(t, e, 1 + rel), n, vals * np.where(np.arange(len(vals)) == e,
                                                                                      1 + rel, 1), h, steps, method,
                      out)
    lm = _oracle_loss(oracle_lib, _scaled_source(t, e, 1 - rel), n, vals * np.where(np.arange(len(vals)) == e,
                                                                                      1 - rel, 1), h, steps, method,
                      out)
    return (lp - lm) / (2 * rel)


def _check(oracle_lib, c, vals, h, steps, method, out_name, K):
    t = element_table(c)
    out = c.index_map[out_name]
    g = _lib.GpuCircuit(t, c.size)
    loss, grad = g.adjoint_tran(vals, h, steps, out, method=method, checkpoint_every=K)
    loss0 = g.adjoint_tran(vals, h, steps, out, method=method, checkpoint_every=K, gradient=False)
    assert np.array_equal(loss, loss0)
    for i in range(len(vals)):
        ref = _oracle_loss(oracle_lib, t, c.size, vals[i], h, steps, method, out)
        assert abs(loss[i] - ref) <= LOSS_TOL * abs(ref), (i, loss[i], ref)
        fd = _fd_grad(oracle_lib, t, c.size, vals[i], h, steps, method, out)
        for e in np.nonzero(np.isin(t["kind"], (4, 5)))[0]:    # sources: waveform scale
            fd[e] = _fd_source(oracle_lib, t, c.size, vals[i], h, steps, method, out, e)
        err = np.max(np.abs(grad[i] - fd)) / np.max(np.abs(fd))
        assert err < GRAD_TOL, (i, err)
        src = np.isin(t["kind"], (4, 5))
        if src.any() and np.max(np.abs(fd[src])) > 0:
            serr = np.max(np.abs(grad[i][src] - fd[src])) / np.max(np.abs(fd[src]))
            assert serr < GRAD_TOL, (i, serr)
        # elements that carry no gradient read exactly zero
        assert np.all(grad[i][~np.isin(t["kind"], (1, 2, 3, 4, 5))] == 0.0)
    return loss, grad


@pytest.mark.parametrize("method", ["tr", "be"])
def test_adjoint_rc_ladder_matches_finite_differences(oracle_lib, method):
    c = rc_ladder_step(12, seed=7)
    vals = monte_carlo_values(c, 3, seed=5, kinds=(1, 2))
    # 150 steps in segments of 32: the last segment is partial
    _check(oracle_lib, c, vals, 1e-9, 150, method, "V(n12)", 32)


def test_adjoint_rlc_ladder_inductor_gradients(oracle_lib):
    c = rlc_ladder(8, rise="50p", width="1n")
    vals = monte_carlo_values(c, 2, seed=9)
    _check(oracle_lib, c, vals, 2e-11, 120, "tr", "V(n8)", 25)


def test_adjoint_checkpoint_interval_does_not_change_result():
    c = rc_ladder_step(40, seed=3)
    t = element_table(c)
    vals = monte_carlo_values(c, 4, seed=2, kinds=(1, 2))
    g = _lib.GpuCircuit(t, c.size)
    out = c.index_map["V(n40)"]
    l1, g1 = g.adjoint_tran(vals, 1e-9, 200, out, checkpoint_every=200)
    l2, g2 = g.adjoint_tran(vals, 1e-9, 200, out, checkpoint_every=7)
    l3, g3 = g.adjoint_tran(vals, 1e-9, 200, out, checkpoint_every=7)
    # the loss comes from the forward pass alone; recomputed segments and the segment-wise
    # gradient sums differ from a single segment only in rounding
    assert np.array_equal(l1, l2)
    assert np.max(np.abs(g1 - g2)) <= 1e-12 * np.max(np.abs(g1))
    assert np.array_equal(l2, l3) and np.array_equal(g2, g3)      # run to run


def test_adjoint_rejects_nonzero_operating_point_and_nonlinear():
    c = parse_circuit_description("V1 in 0 dc 1\nR1 in out 1k\nC1 out 0 1n\n")
    g = _lib.GpuCircuit(element_table(c), c.size)
    with pytest.raises(KretsError):
        g.adjoint_tran(None, 1e-9, 10, c.index_map["V(out)"], n_inst=1)
    c = parse_circuit_description("V1 in 0 dc 0 SIN(0 1 1e6 0 0 0)\nR1 in a 1k\nD1 a 0 DM\n"
                                  ".model DM D (is=1e-14)\n")
    g = _lib.GpuCircuit(element_table(c), c.size)
    with pytest.raises(KretsError):
        g.adjoint_tran(None, 1e-9, 10, c.index_map["V(a)"], n_inst=1)


def test_adjoint_full_size_config5(oracle_lib):
    """Config 5 at its full size: 1024 instances of the 1000-section RC ladder, 2000 TR
    steps, checkpoints every 100.  Instances with identical values give bit-identical
    losses and gradients whatever CTA ran them; instance 0 matches the FP64 oracle adjoint
    (loss 1e-12, gradient 1e-9 norm-wise)."""
    c = rc_ladder_step(1000)
    t = element_table(c)
    out = c.index_map["V(n20)"]
    vals = np.tile(t["value"], (1024, 1))
    g = _lib.GpuCircuit(t, c.size)
    loss, grad = g.adjoint_tran(vals, 1e-9, 2000, out, method="tr", checkpoint_every=100)
    assert np.all(loss == loss[0]) and np.all(grad == grad[0])
    L, gref = oracle_lib.adjoint_tran(t, c.size, 1e-9, 2000, out)
    assert abs(loss[0] - L) <= 1e-12 * abs(L)
    assert np.max(np.abs(grad[0] - gref)) <= 1e-9 * np.max(np.abs(gref))


def test_adjoint_single_kernel_form_agrees(monkeypatch):
    """The forward pass on the double-float engine plus the reverse-only kernel, and the
    single-kernel form (both passes in the adjoint kernel, used when the circuit does not
    fit the double-float engine), give the same loss and gradient to double-float rounding."""
    c = rc_ladder_step(60, seed=11)
    t = element_table(c)
    vals = monte_carlo_values(c, 9, seed=4, kinds=(1, 2))
    g = _lib.GpuCircuit(t, c.size)
    out = c.index_map["V(n30)"]
    l_split, g_split = g.adjoint_tran(vals, 1e-9, 400, out, method="tr", checkpoint_every=64)
    monkeypatch.setenv("KRETS_ADJ_SINGLE", "1")
    l_one, g_one = g.adjoint_tran(vals, 1e-9, 400, out, method="tr", checkpoint_every=64)
    assert np.max(np.abs(l_split - l_one) / np.abs(l_one)) < 1e-12
    assert np.max(np.abs(g_split - g_one)) <= 1e-12 * np.max(np.abs(g_one))


def test_adjoint_150_section_ladder_against_central_differences_1e4(oracle_lib):
    """A 150-section RC ladder (seeded per-instance values, TR 1 ns, 400 steps, loss at
    V(n20)): the device gradient of every R and C against central differences of the FP64
    oracle loss at a relative step of 1e-4, where the differences are accurate to ~1e-9
    (at 1e-6 they are limited by the FP64 loss's own rounding), to 1e-6 relative."""
    from krets_gb300.generators import rc_ladder_step_values
    c = rc_ladder_step(150)
    t = element_table(c)
    out = c.index_map["V(n20)"]
    vals = rc_ladder_step_values(c, 3, seed=11)
    g = _lib.GpuCircuit(t, c.size)
    loss, grad = g.adjoint_tran(vals, 1e-9, 400, out, checkpoint_every=50)
    for i in (0, 2):
        fd = _fd_grad(oracle_lib, t, c.size, vals[i], 1e-9, 400, "tr", out, rel=1e-4)
        rc = np.isin(t["kind"], (1, 2))
        err = np.max(np.abs(grad[i][rc] - fd[rc])) / np.max(np.abs(fd[rc]))
        assert err < GRAD_TOL, (i, err)
        assert abs(loss[i] - _oracle_loss(oracle_lib, t, c.size, vals[i], 1e-9, 400, "tr", out)) <= LOSS_TOL * loss[i]
