"""Pins the CPU oracle to the reference's own answers: the known-answer asserts of
crates/krets-solver/tests/*.rs, the full-precision parquet outputs the reference wrote,
and the waveform known answers of voltage_source.rs.  CPU only."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import analysis_from_case, circuit_from_case
from krets_gb300 import AnalysisSpec, generate_frequencies, parse_circuit_description
from krets_gb300.analyses import TransientAnalysis
from krets_gb300.table import element_table


def _run_oracle(O, case):
    c = circuit_from_case(case)
    t = element_table(c)
    an = analysis_from_case(case)
    kind = next(iter(case["analysis"]))
    if kind == "op":
        x = O.op(t, c.size)
        return c, [{k: x[v] for k, v in c.index_map.items()}]
    if kind == "ac":
        f = [v for v in generate_frequencies(an) if v > 0]
        z = O.ac(t, c.size, f)
        return c, [{**{k: z[i, v] for k, v in c.index_map.items()}, "frequency": complex(f[i], 0)}
                   for i in range(len(f))]
    if kind == "dc":
        idx = next(k for k, el in enumerate(c.elements) if el.identifier == an.element)
        x = O.dc(t, c.size, idx, an.start, an.stop, an.step_size)
        return c, [{**{k: x[i, v] for k, v in c.index_map.items()}, "step": float(i)} for i in range(len(x))]
    if kind == "transient":
        n_steps = int(np.floor(an.stop_time / an.time_step + 0.5))
        x = O.tran(t, c.size, an.time_step, n_steps)
        return c, [{**{k: x[i, v] for k, v in c.index_map.items()}, "time": i * an.time_step}
                   for i in range(n_steps + 1)]
    raise AssertionError(kind)


def _check(maps, expect):
    for key, (val, tol) in expect.items():
        if key == "len":
            assert len(maps) == val
            continue
        if ":" in key:
            i, name = key.split(":", 1)
            row = maps[int(i)]
        else:
            row, name = maps[0], key
        if name.endswith(".re") or name.endswith(".im"):
            v = row[name[:-3]]
            got = v.real if name.endswith(".re") else v.imag
        else:
            got = row[name]
        assert abs(got - val) < tol, (key, got, val)


@pytest.mark.parametrize("group", ["op", "ac", "dc", "tran"])
def test_reference_known_answers(oracle_lib, golden, group):
    for case in golden[group]:
        _, maps = _run_oracle(oracle_lib, case)
        _check(maps, case["expect"])


def test_low_pass_ac_parquet_full_precision(oracle_lib, golden):
    fx = golden["parquet"]["low_pass_ac"]
    spec = AnalysisSpec.from_str(fx["toml"])
    c = parse_circuit_description(fx["netlist"])
    f = generate_frequencies(spec.analysis)
    cols = fx["columns"]
    assert f == cols["frequency"]          # bit-identical frequency list
    z = oracle_lib.ac(element_table(c), c.size, f)
    for key, idx in c.index_map.items():
        mag = np.sqrt(z[:, idx].real ** 2 + z[:, idx].imag ** 2)
        ph = np.arctan2(z[:, idx].imag, z[:, idx].real) * 180.0 / np.pi
        np.testing.assert_allclose(mag, cols[key + "_mag"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(ph, cols[key + "_phase_deg"], rtol=1e-12, atol=1e-12)


def test_inverter_dc_parquet(oracle_lib, golden):
    fx = golden["parquet"]["inverter_dc"]
    spec = AnalysisSpec.from_str(fx["toml"])
    c = parse_circuit_description(fx["netlist"])
    an = spec.analysis
    idx = next(k for k, el in enumerate(c.elements) if el.identifier == an.element)
    x = oracle_lib.dc(element_table(c), c.size, idx, an.start, an.stop, an.step_size)
    cols = fx["columns"]
    assert len(cols["step"]) == len(x)
    for key, v in c.index_map.items():
        np.testing.assert_allclose(x[:, v], cols[key], rtol=1e-12, atol=1e-15)
    np.testing.assert_array_equal(np.arange(len(x), dtype=float), cols["step"])


def test_simple_results_parquet(oracle_lib, golden):
    # an OP of basic_001 (V(1)=3, V(2)=0.5) written by the reference's result crate
    cols = golden["parquet"]["simple_results"]["columns"]
    case = next(c for c in golden["op"] if c["name"] == "basic_001_op")
    c = circuit_from_case(case)
    x = oracle_lib.op(element_table(c), c.size)
    got = {"V1": x[c.index_map["V(1)"]], "V2": x[c.index_map["V(2)"]]}
    for name, val in zip(cols["name"], cols["value"]):
        assert abs(got[name] - val) < 1e-12


def test_waveform_known_answers(oracle_lib, golden):
    w = golden["waveforms"]
    for t, v in w["pulse"]["points"]:
        assert abs(oracle_lib.pulse(w["pulse"]["params"], t) - v) < w["pulse"]["tol"]
    for t, v in w["sin"]["points"]:
        assert abs(oracle_lib.sin(w["sin"]["params"], t) - v) < w["sin"]["tol"]
    for t, v in w["sin"]["points_phase90"]:
        assert abs(oracle_lib.sin(w["sin"]["params_phase90"], t) - v) < w["sin"]["tol"]


def test_source_lag_pinned(oracle_lib, golden):
    """test_transient.rs:203-206 pins the one-step source lag: BE with h/tau = 0.05
    gives 1-1.05^-41 at index 42 (the unlagged value 1-1.05^-42 fails the assert)."""
    case = next(c for c in golden["tran"] if c["name"] == "low_pass_tran")
    _, maps = _run_oracle(oracle_lib, case)
    v = maps[42]["V(out)"]
    assert abs(v - (1 - 1.05 ** -41)) < 1e-12
    assert abs(v - (1 - 1.05 ** -42)) > 1e-3


def test_oracle_lu_matches_scipy(oracle_lib):
    rng = np.random.default_rng(7)
    for n in (5, 40, 300):
        A = sp.random(n, n, density=min(1.0, 4.0 / n), random_state=rng, format="csc") + sp.eye(n) * 0.5
        A = A.tocsc()
        b = rng.standard_normal(n)
        x = oracle_lib.lu_solve_csc(n, A.indptr, A.indices, A.data, b)
        xs = spla.splu(A).solve(b)
        np.testing.assert_allclose(x, xs, rtol=1e-10, atol=1e-12)


def test_oracle_assembled_matrix_solves_like_dense(oracle_lib):
    from krets_gb300.generators import rlc_ladder
    c = rlc_ladder(30)
    t = element_table(c)
    prev = np.linspace(-1, 1, c.size)
    A, b = oracle_lib.assemble(t, c.size, "tran", h=1e-12, method="tr", sol=prev)
    x = np.linalg.solve(A, b)
    assert np.all(np.isfinite(x))


def test_trapezoidal_second_order(oracle_lib):
    """TR extension: halving h cuts the error ~4x on an RC ramp response (BE: ~2x).
    The reference is the same method at h/32 (Richardson-style check)."""
    net = "V1 in 0 dc 0 PULSE(0 1 0 1e-3 1e-3 1 2)\nR1 in out 1000\nC1 out 0 1e-6\n"
    c = parse_circuit_description(net)
    t = element_table(c)
    T = 2e-3
    out = c.index_map["V(out)"]
    ratios = {}
    for method in ("be", "tr"):
        fine = oracle_lib.tran(t, c.size, 2e-5 / 32, int(round(T / (2e-5 / 32))), method=method, lag=False)
        vref = fine[-1, out]
        e = []
        for h in (2e-5, 1e-5):
            x = oracle_lib.tran(t, c.size, h, int(round(T / h)), method=method, lag=False)
            e.append(abs(x[-1, out] - vref))
        ratios[method] = e[0] / e[1]
    assert 1.7 < ratios["be"] < 2.3, ratios
    assert 3.5 < ratios["tr"] < 4.5, ratios
