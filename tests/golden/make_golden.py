"""Generate tests/golden/reference_cases.json from the reference checkout.

Run once where the reference is mounted (it is not on the GPU machine):

    python tests/golden/make_golden.py /path/to/krets

The JSON holds, per case, the input netlist text (the small fixture netlists of
the reference's `circuits/` folder), the analysis, and the reference's expected
answers:

* the known-answer asserts of crates/krets-solver/tests/{test_op,test_ac,
  test_dc,test_transient}.rs (value, tolerance, file:line), transcribed below
  and checked against the test sources by a text search;
* the full-precision outputs the reference itself wrote to
  circuits/low_pass_filter/ac/result.parquet and
  circuits/inverter/dc/result.parquet, and the two values of
  crates/krets-result/simple_results.parquet;
* the waveform known answers of
  crates/krets-parser/src/elements/voltage_source.rs:370-496.

The resistor ladders (500/1000/5000 sections) are not copied: the test suite
regenerates them, and this script checks that the generator reproduces the
element lines of the reference files exactly.
"""
import json
import re
import sys
from pathlib import Path

import pyarrow.parquet as pq

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from krets_gb300.generators import resistor_ladder_netlist  # noqa: E402

# (case, netlist file or inline text, analysis, {key: (expected, tol)}, citation)
OP_CASES = [
    ("najm", "circuit_simulation_farid_n_najm/circuit_simulation_farid_n_najm.cir", {"op": {}},
     {"V(4)": (1.9888, 1e-3), "V(8)": (1.0, 1e-3), "V(3)": (2.00879, 1e-3), "V(2)": (1.80879, 1e-3),
      "V(6)": (1.98814, 1e-3), "V(5)": (2.0, 1e-3), "V(1)": (1.88527, 1e-3), "V(7)": (3.98814, 1e-3),
      "I(V3)": (0.0, 1e-3), "I(V2)": (-199.88e-3, 1e-3), "I(V1)": (-198.88e-3, 1e-3)},
     "crates/krets-solver/tests/test_op.rs:25-46"),
    ("test_case_1", "V1 2 1 32\nR1 1 0 2\nR2 2 3 4\nR3 2 0 8\nV2 3 0 20\n", {"op": {}},
     {"V(1)": (-8.0, 1e-3), "V(2)": (24.0, 1e-3), "V(3)": (20.0, 1e-3), "I(V1)": (-4.0, 1e-3),
      "I(V2)": (1.0, 1e-3)}, "crates/krets-solver/tests/test_op.rs:48-68"),
    ("voltage_divider_op", "voltage_divider/voltage_divider.cir", {"op": {}},
     {"V(in)": (1.0, 1e-3), "V(out)": (2.0 / 3.0, 1e-3), "I(V1)": (1.0 / 3000.0, 1e-3)},
     "crates/krets-solver/tests/test_op.rs:70-81"),
    ("low_pass_op", "low_pass_filter/low_pass_filter.cir", {"op": {}},
     {"V(in)": (1.0, 1e-3), "V(out)": (1.0, 1e-3)}, "crates/krets-solver/tests/test_op.rs:83-93"),
    ("high_pass_op", "high_pass_filter/high_pass_filter.cir", {"op": {}},
     {"V(in)": (1.0, 1e-3), "V(out)": (1.0, 1e-3)}, "crates/krets-solver/tests/test_op.rs:95-105"),
    ("basic_001_op", "basic_001/basic_001.cir", {"op": {}},
     {"V(1)": (3.0, 1e-3), "V(2)": (0.5, 1e-3), "I(V4)": (-0.5, 1e-3)},
     "crates/krets-solver/tests/test_op.rs:107-118"),
    ("resistor_ladder_500_op", "@ladder500", {"op": {}},
     {"V(1)": (1.0, 1e-3), "V(2)": (1.0 - 1.0 / 500.0, 1e-3)},
     "crates/krets-solver/tests/test_op.rs:120-129"),
    ("diode_iv_curve_op", "diode_iv_curve/diode_iv_curve.cir", {"op": {}},
     {"V(out)": (0.517, 1e-3), "I(V1)": (4.82e-04, 1e-3)},
     "crates/krets-solver/tests/test_op.rs:131-140"),
]

AC_CASES = [
    ("low_pass_ac_1k", "low_pass_filter/low_pass_filter.cir",
     {"ac": {"sweep": {"variation": "Linear", "total_points": 1}, "fstart": 1000.0, "fstop": 1000.0}},
     {"V(out).re": (2.470452e-02, 1e-3), "V(out).im": (-1.55223e-01, 1e-3)},
     "crates/krets-solver/tests/test_ac.rs:25-46"),
    ("high_pass_ac_1k", "high_pass_filter/high_pass_filter.cir",
     {"ac": {"sweep": {"variation": "Linear", "total_points": 1}, "fstart": 1000.0, "fstop": 1000.0}},
     {"frequency.re": (1000.0, 1e-3), "frequency.im": (0.0, 1e-3), "V(out).re": (7.169568e-01, 1e-3),
      "V(out).im": (-4.50477e-01, 1e-3), "I(V1).re": (-7.16957e-03, 1e-4), "I(V1).im": (4.504772e-03, 1e-4)},
     "crates/krets-solver/tests/test_ac.rs:48-74"),
]

DC_CASES = [
    ("voltage_divider_dc", "voltage_divider/voltage_divider.cir",
     {"dc": {"element": "V1", "start": 0.0, "stop": 1.0, "step_size": 1.0}},
     {"0:V(in)": (0.0, 1e-3), "0:V(out)": (0.0, 1e-3), "0:I(V1)": (0.0, 1e-3), "1:V(in)": (1.0, 1e-3),
      "1:V(out)": (2.0 / 3.0, 1e-3), "1:I(V1)": (-1.0 / 3000.0, 1e-4), "len": (2, 0)},
     "crates/krets-solver/tests/test_dc.rs:25-54"),
]

TRAN_CASES = [
    ("dual_rc_ladder_tran", "dual_rc_ladder/dual_rc_ladder.cir",
     {"transient": {"time_step": 50e-6, "stop_time": 50e-3}},
     {"0:V(in)": (0.0, 1e-3), "0:V(out)": (0.0, 1e-3), "-1:V(out)": (0.989, 1e-3)},
     "crates/krets-solver/tests/test_transient.rs:139-161"),
    ("rectifier_tran", "rectifier/rectifier.cir",
     {"transient": {"time_step": 50e-6, "stop_time": 50e-3}}, {},
     "crates/krets-solver/tests/test_transient.rs:163-178 (smoke, no asserts)"),
    ("low_pass_tran", "low_pass_filter/transient.cir",
     {"transient": {"time_step": 50e-6, "stop_time": 20e-3}},
     {"0:V(in)": (0.0, 1e-3), "0:V(out)": (0.0, 1e-3), "42:V(out)": (0.8647, 1e-3),
      "42:time": (2.1e-3, 1e-6), "-1:V(out)": (1.0, 1e-3)},
     "crates/krets-solver/tests/test_transient.rs:180-212"),
    ("high_pass_tran", "high_pass_filter/transient.cir",
     {"transient": {"time_step": 10e-6, "stop_time": 2e-3}},
     {"0:V(in)": (0.0, 1e-3), "0:V(out)": (0.0, 1e-3), "-1:V(out)": (1.0, 1e-3)},
     "crates/krets-solver/tests/test_transient.rs:214-238"),
]

PULSE_KAT = {
    "params": [0.0, 5.0, 1e-6, 10e-9, 10e-9, 5e-6, 10e-6],
    "points": [[0.5e-6, 0.0], [1.005e-6, 2.5], [3.01e-6, 5.0], [6.015e-6, 2.5], [8.0e-6, 0.0],
               [11.005e-6, 2.5]],
    "tol": 1e-9, "cite": "crates/krets-parser/src/elements/voltage_source.rs:370-423",
}
SIN_KAT = {
    "params": [1.0, 5.0, 1000.0, 1e-3, 0.0, 0.0],
    "points": [[0.5e-3, 1.0], [1.25e-3, 6.0], [1.5e-3, 1.0], [1.75e-3, -4.0]],
    "params_phase90": [1.0, 5.0, 1000.0, 1e-3, 0.0, 90.0],
    "points_phase90": [[1e-3, 6.0]],
    "tol": 1e-9, "cite": "crates/krets-parser/src/elements/voltage_source.rs:444-496",
}


def _literal_in(text: str, value: float) -> bool:
    # accept any decimal spelling that parses to the same float
    for tok in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", text):
        try:
            if float(tok) == value or float(tok) == -value:
                return True
        except ValueError:
            pass
    return False


def main(ref: Path):
    circuits = ref / "circuits"
    out = {"op": [], "ac": [], "dc": [], "tran": []}
    for group, cases in (("op", OP_CASES), ("ac", AC_CASES), ("dc", DC_CASES), ("tran", TRAN_CASES)):
        for name, src, analysis, expect, cite in cases:
            if src.startswith("@ladder"):
                text = None
                ladder = int(src[len("@ladder"):])
            elif "\n" in src:
                text, ladder = src, None
            else:
                text, ladder = (circuits / src).read_text(), None
            test_file = ref / cite.split(":")[0]
            body = test_file.read_text()
            for key, (val, _tol) in expect.items():
                if key == "len":
                    continue
                if not _literal_in(body, val) and not abs(val - 2.0 / 3.0) < 1e-15 \
                        and not abs(abs(val) - 1.0 / 3000.0) < 1e-15 and not abs(val - (1 - 1 / 500)) < 1e-15:
                    raise SystemExit(f"{name}: expected value {val} for {key} not found in {test_file}")
            out[group].append({"name": name, "netlist": text, "ladder": ladder, "analysis": analysis,
                               "expect": {k: list(v) for k, v in expect.items()}, "cite": cite})
    # the generated ladders must match the reference's element lines
    for n in (500, 1000, 5000):
        ref_lines = [ln for ln in (circuits / f"resistor_ladder_{n}/resistor_ladder_{n}.cir").read_text().splitlines()
                     if ln[:1] in ("V", "R")]
        gen_lines = [ln for ln in resistor_ladder_netlist(n).splitlines() if ln[:1] in ("V", "R")]
        if ref_lines != gen_lines:
            raise SystemExit(f"ladder generator differs from resistor_ladder_{n}.cir")

    lp = pq.read_table(circuits / "low_pass_filter/ac/result.parquet").to_pydict()
    inv = pq.read_table(circuits / "inverter/dc/result.parquet").to_pydict()
    simple = pq.read_table(ref / "crates/krets-result/simple_results.parquet").to_pydict()
    out["parquet"] = {
        "low_pass_ac": {"netlist": (circuits / "low_pass_filter/ac/ac.cir").read_text(),
                        "toml": (circuits / "low_pass_filter/ac/krets.toml").read_text(),
                        "columns": lp, "cite": "circuits/low_pass_filter/ac/result.parquet"},
        "inverter_dc": {"netlist": (circuits / "inverter/dc/inverter.cir").read_text(),
                        "toml": (circuits / "inverter/dc/krets.toml").read_text(),
                        "columns": inv, "cite": "circuits/inverter/dc/result.parquet"},
        "simple_results": {"columns": simple, "cite": "crates/krets-result/simple_results.parquet"},
    }
    out["waveforms"] = {"pulse": PULSE_KAT, "sin": SIN_KAT}
    out["subckt_netlist"] = (circuits / "voltage_divider/subckt/voltage_divider.cir").read_text()
    (HERE / "reference_cases.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "reference_cases.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the krets checkout>")
    main(Path(sys.argv[1]))
