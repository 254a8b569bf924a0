"""Netlist front-end, krets.toml loading and frequency generation (CPU only)."""
import numpy as np
import pytest

from krets_gb300 import AnalysisSpec, generate_frequencies, parse_circuit_description
from krets_gb300.analyses import AcAnalysis, Decade, Linear, Octave, TransientAnalysis
from krets_gb300.errors import ParseError
from krets_gb300.generators import config1_circuit, rc_ladder_ac, resistor_ladder_netlist, rlc_ladder
from krets_gb300.netlist import parse_value
from krets_gb300.table import element_table


def test_index_layout_group2_first(golden):
    # parser.rs:105-125: I(<id>) before the element's new nodes, file order, ground skipped
    c = parse_circuit_description("V1 2 1 32\nR1 1 0 2\nR2 2 3 4\nR3 2 0 8\nV2 3 0 20\n")
    assert c.index_map == {"I(V1)": 0, "V(2)": 1, "V(1)": 2, "V(3)": 3, "I(V2)": 4}


def test_najm_netlist_counts(golden):
    case = next(c for c in golden["op"] if c["name"] == "najm")
    c = parse_circuit_description(case["netlist"])
    assert len(c.elements) == 13          # test_parse_netlist.rs:30-31
    assert len(c.nodes) == 9


def test_empty_netlist_is_error():
    with pytest.raises(ParseError):
        parse_circuit_description("")


def test_subcircuit_flattening(golden):
    c = parse_circuit_description(golden["subckt_netlist"])
    ids = [e.identifier for e in c.elements]
    assert ids == ["Rdiv1_1", "Rdiv1_2", "V1"]
    assert c.elements[0].nodes == ["10", "7"] and c.elements[1].nodes == ["7", "0"]
    nested = """
xdiv1 10 7 0 vdivide
.subckt vdivide 1 2 3
xr1 1 2 myresistor
xr2 2 3 myresistor
.ends
.subckt myresistor plus minus
r0 plus minus 1k
.ends
"""
    c2 = parse_circuit_description(nested)
    assert len(c2.elements) == 2       # test_parse_netlist.rs:76-101


def test_models_and_diode_binding():
    c = parse_circuit_description("V1 in 0 1\nR1 in out 1000\nD1 out 0 DMOD\n.model DMOD D (is=1e-9 n=1.5)\n")
    d = c.elements[2]
    assert d.model["is"] == 1e-9 and d.model["n"] == 1.5
    t = element_table(c)
    assert t[2]["value"] == 1e-9 and t[2]["wp"][0] == 1.5


def test_value_suffixes():
    assert parse_value("1.5k") == 1500.0
    assert abs(parse_value("10u") - 10e-6) < 1e-20
    assert parse_value("3MEG") == 3e6
    assert abs(parse_value("1.2p") - 1.2e-12) < 1e-25
    with pytest.raises(ParseError):
        parse_value("1.5x")


def test_voltage_source_params():
    c = parse_circuit_description("V1 in 0 dc 0 PULSE (0 5 1u 100u 100u 5u 10u)\nR1 in 0 1\n")
    v = c.elements[0]
    assert v.value == 0.0 and v.wave == 1
    np.testing.assert_allclose(v.wave_params, [0, 5, 1e-6, 100e-6, 100e-6, 5e-6, 10e-6])
    c = parse_circuit_description("V2 3 4 0 AC 1.5\nR1 3 4 1\n")
    assert c.elements[0].ac == 1.5


def test_frequency_generation():
    f = generate_frequencies(AcAnalysis(Decade(455), 1.0, 1e9))
    assert len(f) == 4096 and f[0] == 1.0 and f[-1] == 1e9
    f = generate_frequencies(AcAnalysis(Linear(1), 1000.0, 1000.0))
    assert f == [1000.0]
    f = generate_frequencies(AcAnalysis(Octave(3), 1.0, 8.0))
    assert len(f) == 10 and f[-1] == 8.0
    assert generate_frequencies(AcAnalysis(Linear(5), 10.0, 1.0)) == []


def test_krets_toml():
    spec = AnalysisSpec.from_str('circuit_path = "a.cir"\n[analysis.transient]\ntime_step = 1e-6\nstop_time = 1e-3\n')
    assert isinstance(spec.analysis, TransientAnalysis) and spec.analysis.method == "be"
    spec = AnalysisSpec.from_str('circuit_path = "a.cir"\n[analysis.transient]\ntime_step = 1e-6\nstop_time = 1e-3\n'
                                 '[gb300]\nmethod = "tr"\n')
    assert spec.analysis.method == "tr"
    spec = AnalysisSpec.from_str('circuit_path = "x"\n[analysis.ac]\nsweep = { variation = "Decade", '
                                 'points_per_decade = 5 }\nfstart = 10.0\nfstop = 1000.0\n')
    assert isinstance(spec.analysis.sweep, Decade) and spec.analysis.sweep.points_per_decade == 5


def test_workload_sizes():
    assert config1_circuit().size == 1001
    assert rc_ladder_ac().size == 502
    assert rlc_ladder().size == 602
    assert "R5000 5000 0 1000" in resistor_ladder_netlist(5000)


def _write_case(tmp_path, case):
    (tmp_path / "krets.toml").write_text(case["toml"])
    import tomllib
    circ = tomllib.loads(case["toml"])["circuit_path"]
    (tmp_path / circ).write_text(case["netlist"])
    return tmp_path / "krets.toml"


def test_cli_ac_parquet_matches_reference_file(tmp_path, golden, oracle_lib):
    """The CLI path (krets.toml -> netlist -> solve -> result.parquet, main.rs:27-138) with
    the parquet layout of krets-result (lib.rs:127-208) reproduces the reference's own
    circuits/low_pass_filter/ac/result.parquet: column names, order and values."""
    pq = pytest.importorskip("pyarrow.parquet")
    from oracle_solver import OracleSolver
    from krets_gb300.__main__ import run
    case = golden["parquet"]["low_pass_ac"]
    out = run(_write_case(tmp_path, case), solver_factory=OracleSolver)
    t = pq.read_table(out)
    ref = case["columns"]
    assert t.column_names == list(ref)
    for k, v in ref.items():
        np.testing.assert_allclose(t.column(k).to_numpy(), v, rtol=1e-12, atol=1e-15)


def test_transient_and_dc_writers_put_keys_in_order(tmp_path):
    pq = pytest.importorskip("pyarrow.parquet")
    from krets_gb300.results import write_dc_results_to_parquet, write_tran_results_to_parquet
    rows = [{"V(b)": 1.0, "time": 0.0, "I(V1)": 2.0}, {"V(b)": 3.0, "time": 1e-3}]
    name = write_tran_results_to_parquet(rows, tmp_path / "tran")
    t = pq.read_table(name)
    assert name.endswith(".parquet") and t.column_names == ["time", "I(V1)", "V(b)"]
    assert t.column("I(V1)").to_pylist() == [2.0, None]
    t = pq.read_table(write_dc_results_to_parquet([{"step": 0.0, "V(a)": 1.5}], tmp_path / "dc.parquet"))
    assert t.column_names == ["V(a)", "step"]
