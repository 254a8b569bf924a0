"""GPU parity: every analysis through the C ABI against the CPU oracle on the same
inputs.  Tolerance 1e-9, asserted in two forms (oracle/compare.py): norm-wise relative
error per quantity class (node voltages, branch currents), and element-wise in the form of
the reference's convergence test, |x - x_ref| <= 1e-9 |x_ref| + 1e-12 V (1e-18 A) for
every unknown at every step.  Also the reference's own known answers."""
import numpy as np
import pytest

from conftest import analysis_from_case, circuit_from_case
from krets_gb300 import AnalysisSpec, Solver, generate_frequencies, parse_circuit_description
from krets_gb300 import _lib
from krets_gb300.generators import (config1_circuit, monte_carlo_values, rc_ladder_ac, rc_ladder_step,
                                    rlc_ladder)
from krets_gb300.table import element_table, is_current_mask
from oracle.compare import elementwise_err, normwise_err

pytestmark = pytest.mark.gpu

TOL = 1e-9


def rel_err(x, ref, cur_mask):
    """The larger of the norm-wise and the element-wise error (both must be below 1e-9)."""
    return max(normwise_err(x, ref, cur_mask), elementwise_err(x, ref, cur_mask))


def _oracle(O, case):
    from test_oracle_golden import _run_oracle
    return _run_oracle(O, case)


@pytest.mark.parametrize("group", ["op", "ac", "dc", "tran"])
def test_reference_cases_through_solver(oracle_lib, golden, group):
    from test_oracle_golden import _check
    for case in golden[group]:
        c = circuit_from_case(case)
        res = Solver(c).solve(analysis_from_case(case))
        maps = res.data if isinstance(res.data, list) else [res.data]
        _check(maps, case["expect"])
        _, ref = _oracle(oracle_lib, case)
        assert len(ref) == len(maps)
        names = list(c.index_map)
        got = np.array([[m[k] for k in names] for m in maps])
        exp = np.array([[m[k] for k in names] for m in ref])
        mask = np.array([k.startswith("I") for k in names])
        assert rel_err(got, exp, mask) < TOL, case["name"]


def test_low_pass_ac_parquet(golden):
    fx = golden["parquet"]["low_pass_ac"]
    spec = AnalysisSpec.from_str(fx["toml"])
    c = parse_circuit_description(fx["netlist"])
    res = Solver(c).solve(spec.analysis)
    cols = fx["columns"]
    for key, idx in c.index_map.items():
        z = res.array[:, idx]
        np.testing.assert_allclose(np.abs(z), cols[key + "_mag"], rtol=1e-12)
        np.testing.assert_allclose(np.degrees(np.arctan2(z.imag, z.real)), cols[key + "_phase_deg"], rtol=1e-10,
                                   atol=1e-10)


def test_inverter_dc_parquet(golden):
    fx = golden["parquet"]["inverter_dc"]
    spec = AnalysisSpec.from_str(fx["toml"])
    c = parse_circuit_description(fx["netlist"])
    res = Solver(c).solve(spec.analysis)
    for key, v in c.index_map.items():
        np.testing.assert_allclose(res.array[:, v], fx["columns"][key], rtol=1e-12, atol=1e-15)


def test_config1_plain_op(oracle_lib):
    c = config1_circuit()
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    x, it = g.op()
    ref = oracle_lib.op(t, c.size)
    assert it == 1
    assert rel_err(x, ref, is_current_mask(c)) < TOL


def test_plain_transient_refactor_matches_reuse(oracle_lib):
    c = rlc_ladder(40)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    a = g.tran(1e-12, 400, "tr", lag=False, refactor_each_step=True)
    b = g.tran(1e-12, 400, "tr", lag=False, refactor_each_step=False)
    np.testing.assert_array_equal(a, b)      # identical factors -> identical results
    ref = oracle_lib.tran(t, c.size, 1e-12, 400, method="tr", lag=False)
    assert rel_err(a, ref, is_current_mask(c)) < TOL


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED, _lib.PREC_DF])
def test_batched_mc_transient_matches_oracle(oracle_lib, precision):
    c = rlc_ladder(200)
    t = element_table(c)
    vals = monte_carlo_values(c, 6, seed=11)
    g = _lib.GpuCircuit(t, c.size)
    steps = 1500
    x = g.batch_tran(vals, 1e-12, steps, "tr", lag=False, precision=precision)
    mask = is_current_mask(c)
    for i in range(len(vals)):
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.tran(ti, c.size, 1e-12, steps, method="tr", lag=False)
        assert rel_err(x[i], ref, mask) < TOL, i
    if precision == _lib.PREC_MIXED:
        hist, fb = g.refine_stats()
        assert hist.sum() == len(vals) * steps and fb == 0


def test_batched_be_with_source_lag(oracle_lib):
    net = "V1 in 0 dc 0 PULSE (0 1 1u 1u 1u 1 1)\nR1 in out 1000\nC1 out 0 1u\n"
    c = parse_circuit_description(net)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    x = g.batch_tran(None, 50e-6, 400, "be", lag=True, precision=_lib.PREC_MIXED, n_inst=1)
    assert abs(x[0, 42, c.index_map["V(out)"]] - 0.8647) < 1e-3
    ref = oracle_lib.tran(t, c.size, 50e-6, 400, method="be", lag=True)
    assert rel_err(x[0], ref, is_current_mask(c)) < TOL


HALF_WAVE = ("V1 in 0 SIN(0 5 60 0 0 0)\nR1 in a 10\nD1 a out DMOD\nC1 out 0 10u\nR2 out 0 1k\n"
             ".model DMOD D (is=1e-12)\n")


def test_nonlinear_transient_newton(oracle_lib):
    """Diode half-wave rectifier: a Newton loop per step (transient.rs:51-109), BE with the
    reference's source timing, plain and batched forms against the oracle."""
    c = parse_circuit_description(HALF_WAVE)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    ref, iters = oracle_lib.tran(t, c.size, 50e-6, 400, method="be", lag=True, return_iters=True)
    assert iters.max() > 2                      # a genuinely nonlinear solve
    mask = is_current_mask(c)
    assert rel_err(g.tran(50e-6, 400, "be", lag=True), ref, mask) < TOL
    vals = np.tile(t["value"], (3, 1))
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED):
        x = g.batch_tran(vals, 50e-6, 400, "be", lag=True, precision=prec)
        for i in range(3):
            assert rel_err(x[i], ref, mask) < TOL, prec


@pytest.mark.parametrize("sections", [60, 1000, 1500, 4000])
def test_plain_op_program_placements(oracle_lib, sections):
    """The plain OP with its factorisation and solve arrays copied into shared memory (60,
    1000 sections), read from global memory beside a shared-memory workspace (1500), and
    with the workspace itself in global memory (4000), each against the oracle."""
    from krets_gb300.generators import resistor_ladder_netlist
    c = parse_circuit_description(resistor_ladder_netlist(sections, shunts=True))
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    x, it = g.op()
    assert it == 1
    assert rel_err(x, oracle_lib.op(t, c.size), is_current_mask(c)) < TOL


def test_reference_rectifier_runs():
    """The reference's rectifier test is smoke only (test_transient.rs:163-178): its
    ground-anode diodes always see the 0.5 V default guess (diode.rs:26-30), and the
    solution grows without bound, in the reference as here.  Check it runs to the end."""
    import json
    from conftest import GOLDEN
    case = next(cc for cc in json.loads(GOLDEN.read_text())["tran"] if cc["name"] == "rectifier_tran")
    c = circuit_from_case(case)
    g = _lib.GpuCircuit(element_table(c), c.size)
    x = g.tran(50e-6, 50, "be", lag=True)
    assert x.shape == (51, c.size)


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_batched_ac_sweep_matches_oracle(oracle_lib, precision):
    from krets_gb300.analyses import AcAnalysis, Decade
    c = rc_ladder_ac()
    t = element_table(c)
    f = np.array(generate_frequencies(AcAnalysis(Decade(455), 1.0, 1e9)))   # all 4096 points
    g = _lib.GpuCircuit(t, c.size)
    z = g.batch_ac(None, f, precision=precision)[0]
    ref = oracle_lib.ac(t, c.size, f)
    mask = is_current_mask(c)
    for i in range(len(f)):   # per frequency point (each is its own system)
        assert rel_err(z[i], ref[i], mask) < TOL, (i, f[i])


AC_DIODE = """* diode clamp biased at its operating point, AC source
V1 in 0 dc 0.7 AC 1
R1 in a 100
D1 a 0 DMOD
C1 a 0 10n
R2 a b 1000
C2 b 0 1n
.model DMOD D (is=1e-12)
"""


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED])
@pytest.mark.parametrize("case", ["ladder", "diode"])
def test_batched_ac_monte_carlo_instances(oracle_lib, precision, case):
    """Several parameter sets in one batched sweep: the work items of the instances
    interleave on the CTAs, which keep each instance's frequency-independent coefficients
    (conductances, C and L values, the diode's small-signal conductance at that
    instance's operating point) between points.  Every (instance, point) against the
    oracle's sweep with that instance's values."""
    from krets_gb300.analyses import AcAnalysis, Decade
    c = rc_ladder_ac(60, seed=5) if case == "ladder" else parse_circuit_description(AC_DIODE)
    t = element_table(c)
    f = np.array(generate_frequencies(AcAnalysis(Decade(7), 10.0, 1e8)))
    vals = monte_carlo_values(c, 12, seed=8)
    g = _lib.GpuCircuit(t, c.size)
    z = g.batch_ac(vals, f, precision=precision)
    mask = is_current_mask(c)
    for i in range(len(vals)):
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.ac(ti, c.size, f)
        for k in range(len(f)):
            assert rel_err(z[i, k], ref[k], mask) < TOL, (i, k, f[k])


def test_batch_op_monte_carlo(oracle_lib):
    c = config1_circuit()
    t = element_table(c)
    vals = monte_carlo_values(c, 8, seed=4)
    g = _lib.GpuCircuit(t, c.size)
    x = g.batch_op(vals)
    for i in range(len(vals)):
        ti = t.copy()
        ti["value"] = vals[i]
        assert rel_err(x[i], oracle_lib.op(ti, c.size), is_current_mask(c)) < TOL


DIODE_LADDER = """* diode ladder, DC sweep of V1
V1 in 0 1
R1 in a 1000
D1 a 0 DMOD
R2 a b 2200
D2 b 0 DMOD
R3 b c 470
D3 c 0 DMOD
R4 c 0 10000
.model DMOD D (is=1e-12)
"""


def test_batch_dc_monte_carlo(oracle_lib):
    """Warm-started nonlinear sweeps of 16 parameter sets: each instance against the oracle's
    dc::solve restatement with that instance's values."""
    c = parse_circuit_description(DIODE_LADDER)
    t = element_table(c)
    vals = monte_carlo_values(c, 16, seed=7)
    g = _lib.GpuCircuit(t, c.size)
    sweep = int(np.nonzero(t["kind"] == 4)[0][0])
    x, st = g.batch_dc(vals, sweep, -0.5, 3.0, 0.05)
    assert x.shape == (16, 71, c.size) and not st.any()
    mask = is_current_mask(c)
    for i in range(len(vals)):
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.dc(ti, c.size, sweep, -0.5, 3.0, 0.05)
        assert rel_err(x[i], ref, mask) < TOL, i
    # one instance with the nominal values equals the single-instance sweep
    x1, _ = g.batch_dc(t["value"][None, :], sweep, -0.5, 3.0, 0.05)
    np.testing.assert_array_equal(x1[0], g.dc(sweep, -0.5, 3.0, 0.05))


def test_batched_transient_is_deterministic():
    c = rlc_ladder(100)
    t = element_table(c)
    vals = monte_carlo_values(c, 32, seed=1)
    g = _lib.GpuCircuit(t, c.size)
    a = g.batch_tran(vals, 1e-12, 300, "tr", precision=_lib.PREC_MIXED)
    b = g.batch_tran(vals, 1e-12, 300, "tr", precision=_lib.PREC_MIXED)
    np.testing.assert_array_equal(a, b)


def test_errors_are_reported():
    from krets_gb300.errors import DecompositionFailed, ElementNotFound, MatrixDecomposition
    from krets_gb300.analyses import DcAnalysis, Op
    c = parse_circuit_description("V1 a 0 1\nV2 a 0 2\nR1 a 0 1\n")   # V-source loop: singular
    with pytest.raises((DecompositionFailed, MatrixDecomposition)):
        Solver(c).solve(Op())
    c = parse_circuit_description("V1 a 0 1\nR1 a 0 1\n")
    with pytest.raises(ElementNotFound):
        Solver(c).solve(DcAnalysis("V9", 0, 1, 0.5))


@pytest.mark.parametrize("precision", [_lib.PREC_FP64, _lib.PREC_MIXED, _lib.PREC_DF])
def test_batched_failure_stays_with_its_instance(oracle_lib, precision):
    """A parameter set that makes the matrix non-finite (a 0-ohm resistor) fails alone: its
    status is set, the call reports the failure, and every other instance still matches
    the oracle."""
    import ctypes
    c = rlc_ladder(30)
    t = element_table(c)
    vals = monte_carlo_values(c, 6, seed=9)
    bad = 3
    vals[bad, int(np.nonzero(t["kind"] == 1)[0][4])] = 0.0
    g = _lib.GpuCircuit(t, c.size)
    n_steps = 200
    out = _lib.host_buffer((6, n_steps + 1, c.size))
    st = np.zeros(6, dtype=np.int32)
    rc = _lib.lib().krets_batch_tran(g.h, 6, _lib.ptr(vals), 1e-12, n_steps, 1, 0, precision, _lib.ptr(out),
                                     _lib.ptr(st))
    assert rc != 0 and st[bad] != 0
    assert not np.delete(st, bad).any()
    mask = is_current_mask(c)
    for i in range(6):
        if i == bad:
            continue
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.tran(ti, c.size, 1e-12, n_steps, method="tr", lag=False)
        assert rel_err(out[i], ref, mask) < TOL, i


def test_double_float_group_size_autotuner(oracle_lib, monkeypatch):
    """The first double-float run of a sparsity signature times the group sizes and caches
    the fastest; later runs reuse it; KRETS_GROUP overrides.  Every choice meets 1e-9."""
    c = rlc_ladder(37)          # a signature no other test uses
    t = element_table(c)
    vals = monte_carlo_values(c, 40, seed=13)
    g = _lib.GpuCircuit(t, c.size)
    mask = is_current_mask(c)
    x = g.batch_tran(vals, 1e-12, 150, "tr", lag=False, precision=_lib.PREC_DF)
    first = g.last_launch()
    assert first["group_size_from"] == "autotuner" and first["threads_per_instance"] in (32, 64, 128)
    g.batch_tran(vals, 1e-12, 150, "tr", lag=False, precision=_lib.PREC_DF)
    again = g.last_launch()
    assert again["group_size_from"] == "autotuner cache"
    assert again["threads_per_instance"] == first["threads_per_instance"]
    monkeypatch.setenv("KRETS_GROUP", "64")
    y = g.batch_tran(vals, 1e-12, 150, "tr", lag=False, precision=_lib.PREC_DF)
    assert g.last_launch()["threads_per_instance"] == 64 and g.last_launch()["group_size_from"] == "default"
    for i in (0, 39):
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.tran(ti, c.size, 1e-12, 150, method="tr", lag=False)
        assert rel_err(x[i], ref, mask) < TOL and rel_err(y[i], ref, mask) < TOL


@pytest.mark.parametrize("place", ["auto", "global"])
def test_probe_only_transient_equals_full_waveform_columns(monkeypatch, place):
    """The probe-only run writes exactly the probed columns of the full double-float run
    (same arithmetic, bit for bit), row 0 included; out-of-range probes are rejected.  With
    the factors in global memory (64-thread groups) both runs take the direct
    right-hand-side step."""
    if place == "global":
        monkeypatch.setenv("KRETS_GROUP", "64")
        monkeypatch.setenv("KRETS_DFD_LU", "global")
    c = rlc_ladder(40)
    t = element_table(c)
    vals = monte_carlo_values(c, 37, seed=17)
    g = _lib.GpuCircuit(t, c.size)
    full = g.batch_tran(vals, 1e-12, 400, "tr", lag=False, precision=_lib.PREC_DF)
    probe = [c.index_map["V(n40)"], c.index_map["V(n1)"], c.index_map["I(V1)"]]
    got = g.batch_tran_probe(vals, 1e-12, 400, probe, "tr", lag=False)
    assert got.shape == (37, 401, 3)
    assert np.array_equal(got, full[:, :, probe])
    from krets_gb300.errors import KretsError
    with pytest.raises(KretsError):
        g.batch_tran_probe(vals, 1e-12, 10, [c.size], "tr")


def test_zero_step_transient_is_the_operating_point(oracle_lib):
    """stop_time < time_step / 2 gives num_steps = 0: the result is the t = 0 operating
    point alone (transient.rs:14-114)."""
    c = rlc_ladder(10)
    t = element_table(c)
    g = _lib.GpuCircuit(t, c.size)
    x = g.tran(1e-12, 0, "be")
    assert x.shape == (1, c.size)
    np.testing.assert_allclose(x[0], oracle_lib.op(t, c.size), rtol=1e-12, atol=1e-15)
    xb = g.batch_tran(monte_carlo_values(c, 3, seed=1), 1e-12, 0, "tr", precision=_lib.PREC_DF)
    assert xb.shape == (3, 1, c.size)


def test_batched_transient_host_and_device_outputs_identical():
    """Host output buffers (used in place when the GPU shares the host page tables, else
    through a device copy) give the same bits as a device buffer."""
    c = rlc_ladder(20)
    t = element_table(c)
    vals = monte_carlo_values(c, 5, seed=2)
    g = _lib.GpuCircuit(t, c.size)
    host = g.batch_tran(vals, 1e-12, 300, "tr", lag=False, precision=_lib.PREC_DF)
    dev = _lib.DeviceArray((5, 301, c.size))
    g.batch_tran(vals, 1e-12, 300, "tr", lag=False, precision=_lib.PREC_DF, out=dev)
    assert np.array_equal(host, dev.download())
    assert _lib.lib().krets_direct_host_access() in (0, 1)


def test_config3_full_size_sampled_parity_and_exact_linearity(oracle_lib):
    """The headline workload at its full size (2048 instances x 10 000 TR steps x 602
    unknowns, double-float engine): three instances against the FP64 oracle over all
    steps, and a size-independent property of the linear system — doubling the source
    amplitude doubles every waveform.  Scaling by 2 is exact in floating point except
    where values underflow (the far sections of the ladder before the front arrives
    reach ~1e-300, beyond the double-float pairs' FP32 range), so the check is 1e-12
    relative to each instance's largest value."""
    n_inst, n_steps, h = 2048, 10000, 1e-12
    c = rlc_ladder(200)
    t = element_table(c)
    vals = monte_carlo_values(c, n_inst, sigma=0.1, seed=3)
    mask = is_current_mask(c)
    n = c.size
    row_bytes = (n_steps + 1) * n * 8
    sample = (0, 1023, 2047)

    def run(table):
        g = _lib.GpuCircuit(table, n)
        out = _lib.DeviceArray((n_inst, n_steps + 1, n))
        g.batch_tran(vals, h, n_steps, "tr", lag=False, precision=_lib.PREC_DF, out=out)
        rows = {}
        for i in sample:
            x = np.empty((n_steps + 1, n))
            _lib.check(_lib.lib().krets_memcpy_d2h(x.ctypes.data_as(_lib.ctypes.c_void_p),
                                                   _lib.ctypes.c_void_p(out.ptr + i * row_bytes), x.nbytes))
            rows[i] = x
        del out
        return rows

    base = run(t)
    for i in sample:
        ti = t.copy()
        ti["value"] = vals[i]
        ref = oracle_lib.tran(ti, n, h, n_steps, method="tr", lag=False)
        assert rel_err(base[i], ref, mask) < TOL, i
    t2 = t.copy()
    src = int(np.nonzero(t["kind"] == 4)[0][0])
    t2["wp"][src][1] *= 2.0          # PULSE V2: 1 V -> 2 V (V1 = 0)
    doubled = run(t2)
    for i in sample:
        scale = np.abs(2.0 * base[i]).max()
        assert np.abs(doubled[i] - 2.0 * base[i]).max() <= 1e-12 * scale, i


@pytest.mark.parametrize("G", ["32", "64", "128"])
def test_factor_placements_give_identical_bits(oracle_lib, monkeypatch, G):
    """The double-float engine with its factors in shared memory (row-descriptor solves)
    and in global memory (interleaved solves, zero-padded levels) runs the same arithmetic:
    identical bits, on the RLC ladder (TR) and on a random uneven netlist (BE with the
    reference's source lag); both against the oracle."""
    from krets_gb300.generators import uneven_table
    cases = []
    c = rlc_ladder(100)
    cases.append((element_table(c), c.size, is_current_mask(c), "tr", False, 1e-12, monte_carlo_values(c, 20, seed=6)))
    t6, n6 = uneven_table(0)   # n = 630: both placements fit
    m6 = np.zeros(n6, bool)
    m6[t6["b"][t6["b"] >= 0]] = True
    cases.append((t6, n6, m6, "be", True, 1e-9, np.tile(t6["value"], (3, 1))))
    monkeypatch.setenv("KRETS_GROUP", G)
    for t, n, mask, method, lag, h, vals in cases:
        outs = {}
        for place in ("smem", "global"):
            monkeypatch.setenv("KRETS_DFD_LU", place)
            g = _lib.GpuCircuit(t, n)
            outs[place] = g.batch_tran(vals, h, 300, method, lag=lag, precision=_lib.PREC_DF)
            assert g.last_launch()["factors"] == ("global memory" if place == "global" else "shared memory")
        np.testing.assert_array_equal(outs["smem"], outs["global"])
        ti = t.copy()
        ti["value"] = vals[0]
        ref = oracle_lib.tran(ti, n, h, 300, method=method, lag=lag)
        assert normwise_err(outs["global"][0], ref, mask) < TOL


MIXED_DIRECT = ("V1 in 0 SIN(0 1 1e9 0 0 0)\nR1 in a 50\nL1 a b 1n\nC1 b 0 1p\nR2 b c 100\n"
                "C3 c d 1p\nR3 d 0 1k\nI1 e 0 1m\nR4 e 0 1k\n")


@pytest.mark.parametrize("G", ["32", "64", "128"])
def test_direct_rhs_step_gives_identical_bits(oracle_lib, monkeypatch, G):
    """The interleaved double-float step with a direct right-hand side (each element writes
    the rows it feeds, no gather pass; output converted on the FP64 pipe or by integer
    widening) and the one with the gather pass (KRETS_DFD_OPTS bit 3) give identical bits: TR with companion currents and BE on the RLC ladder, and TR on
    a netlist with a floating capacitor, a current source and a tabulated SIN source; also
    when the transient runs as spans resuming from saved state (staged host output).
    Against the oracle in both error measures."""
    c = rlc_ladder(100)
    m = parse_circuit_description(MIXED_DIRECT)
    cases = [(c, "tr", False, 1e-12, monte_carlo_values(c, 20, seed=6)),
             (c, "be", False, 1e-12, monte_carlo_values(c, 7, seed=8)),
             (c, "be", True, 1e-12, monte_carlo_values(c, 5, seed=9)),   # the reference's source lag
             (m, "tr", False, 2e-11, monte_carlo_values(m, 9, seed=3))]
    monkeypatch.setenv("KRETS_GROUP", G)
    monkeypatch.setenv("KRETS_DFD_LU", "global")
    for ckt, method, lag, h, vals in cases:
        t = element_table(ckt)
        outs = {}
        # 20: the default (direct rhs, output converted on the FP64 pipe), 4: direct rhs with
        # integer widening of the output, 12: the gather pass
        for opts in ("20", "4", "12"):
            monkeypatch.setenv("KRETS_DFD_OPTS", opts)
            g = _lib.GpuCircuit(t, ckt.size)
            outs[opts] = g.batch_tran(vals, h, 300, method, lag=lag, precision=_lib.PREC_DF)
        np.testing.assert_array_equal(outs["20"], outs["12"])
        np.testing.assert_array_equal(outs["4"], outs["12"])
        monkeypatch.delenv("KRETS_DFD_OPTS")
        monkeypatch.setenv("KRETS_HOST_OUT", "staged")
        spans = _lib.GpuCircuit(t, ckt.size).batch_tran(vals, h, 300, method, lag=lag, precision=_lib.PREC_DF)
        monkeypatch.delenv("KRETS_HOST_OUT")
        np.testing.assert_array_equal(spans, outs["20"])
        ti = t.copy()
        ti["value"] = vals[-1]
        ref = oracle_lib.tran(ti, ckt.size, h, 300, method=method, lag=lag)
        assert rel_err(outs["20"][-1], ref, is_current_mask(ckt)) < TOL
