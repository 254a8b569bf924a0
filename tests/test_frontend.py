"""Netlist front-end, krets.toml loading and frequency generation (CPU only)."""
import numpy as np
import pytest

from conftest import ROOT
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
    circuits/low_pass_filter/ac/result.parquet: column names, order and values (solved
    here by the oracle; the GPU form of this test is below)."""
    from oracle_solver import OracleSolver
    from krets_gb300.__main__ import run
    from krets_gb300.parquet import read_parquet
    case = golden["parquet"]["low_pass_ac"]
    out = run(_write_case(tmp_path, case), solver_factory=OracleSolver)
    got = read_parquet(out)
    ref = case["columns"]
    assert list(got) == list(ref)
    for k, v in ref.items():
        np.testing.assert_allclose(got[k], v, rtol=1e-12, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["low_pass_ac", "inverter_dc"])
def test_cli_on_the_gpu_matches_reference_files(tmp_path, golden, name):
    """The command line end to end on the GPU: krets.toml and the netlist in a folder,
    `python -m krets_gb300 krets.toml` (a child process, the reference CLI's behaviour:
    main.rs:27-138) solves with the default GPU Solver and writes result.parquet, whose
    columns equal the reference's own result.parquet (AC: magnitude and phase of every
    unknown at 10 frequencies; DC: the inverter's 101-point sweep)."""
    import subprocess
    import sys
    from krets_gb300.parquet import read_parquet
    case = golden["parquet"][name]
    toml = _write_case(tmp_path, case)
    r = subprocess.run([sys.executable, "-m", "krets_gb300", str(toml)], cwd=str(ROOT), capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = read_parquet(tmp_path / "result.parquet")
    ref = case["columns"]
    assert sorted(got) == sorted(ref)
    for k, v in ref.items():
        np.testing.assert_allclose(got[k], v, rtol=1e-12, atol=1e-15, err_msg=k)


@pytest.mark.gpu
def test_run_with_the_gpu_solver_writes_reference_columns(tmp_path, golden):
    """run() in-process with the default (GPU) solver on the low-pass AC fixture."""
    from krets_gb300.__main__ import run
    from krets_gb300.parquet import read_parquet
    case = golden["parquet"]["low_pass_ac"]
    got = read_parquet(run(_write_case(tmp_path, case)))
    ref = case["columns"]
    assert list(got) == list(ref)
    for k, v in ref.items():
        np.testing.assert_allclose(got[k], v, rtol=1e-12, atol=1e-15, err_msg=k)


def test_parquet_writer_reader_round_trip_and_arrow(tmp_path):
    """The package's own parquet writer: nullable double columns read back by its reader,
    and by pyarrow (an independent implementation) where it is installed; files pyarrow
    writes uncompressed with PLAIN pages read back by the package's reader."""
    from krets_gb300.parquet import read_parquet, write_parquet
    cols = {"time": [0.0, 1e-3, None] + [float(i) for i in range(30)],
            "V(a)": [None, 1.5, -2.0] + [None] * 10 + [3.25] * 20,
            "I(V1)": [np.pi] * 33}
    f = tmp_path / "a.parquet"
    write_parquet(cols, f)
    assert read_parquet(f) == cols
    write_parquet({"only": [2.5]}, f)
    assert read_parquet(f) == {"only": [2.5]}
    pa = pytest.importorskip("pyarrow")
    pq = pytest.importorskip("pyarrow.parquet")
    write_parquet(cols, f)
    t = pq.read_table(f)
    assert t.column_names == list(cols)
    for k, v in cols.items():
        assert t.column(k).to_pylist() == v
    g = tmp_path / "b.parquet"
    pq.write_table(pa.table({k: pa.array(v, type=pa.float64()) for k, v in cols.items()}), g,
                   compression="none", use_dictionary=False, data_page_version="1.0")
    assert read_parquet(g) == cols


def test_transient_and_dc_writers_put_keys_in_order(tmp_path):
    from krets_gb300.parquet import read_parquet
    from krets_gb300.results import write_dc_results_to_parquet, write_tran_results_to_parquet
    rows = [{"V(b)": 1.0, "time": 0.0, "I(V1)": 2.0}, {"V(b)": 3.0, "time": 1e-3}]
    name = write_tran_results_to_parquet(rows, tmp_path / "tran")
    t = read_parquet(name)
    assert name.endswith(".parquet") and list(t) == ["time", "I(V1)", "V(b)"]
    assert t["I(V1)"] == [2.0, None]
    t = read_parquet(write_dc_results_to_parquet([{"step": 0.0, "V(a)": 1.5}], tmp_path / "dc.parquet"))
    assert list(t) == ["V(a)", "step"]
