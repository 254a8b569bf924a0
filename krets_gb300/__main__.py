"""Command line: python -m krets_gb300 <krets file> [-l LEVEL]

As the reference CLI (crates/krets-cli/src/main.rs:27-138): read the krets.toml analysis
spec, resolve the circuit path relative to the krets file (else as given, if absolute),
parse the netlist, solve with the default SolverConfig on the GPU, and write
result.parquet next to the krets file.  The reference's GUI (krets-gui) has no
counterpart in this package; --gui is accepted and reported as unavailable.
"""
from __future__ import annotations

import argparse
import logging
import sys
from pathlib import Path

log = logging.getLogger("krets")


def run(krets_file, solver_factory=None) -> Path:
    from .analyses import AnalysisSpec
    from .config import SolverConfig
    from .netlist import parse_circuit_description_file
    from .results import write_results
    from .solver import Solver
    krets_path = Path(krets_file)
    spec = AnalysisSpec.from_file(krets_path)
    parent = krets_path.parent
    out = parent / "result.parquet"
    rel = parent / spec.circuit_path
    if rel.exists():
        circuit_path = rel
    elif spec.circuit_path.is_absolute() and spec.circuit_path.exists():
        circuit_path = spec.circuit_path
    else:
        raise FileNotFoundError(f"Circuit file not found.\nTried:\n  - relative to krets file: {rel}\n"
                                f"  - as given (absolute or relative to cwd): {spec.circuit_path}")
    circuit = parse_circuit_description_file(circuit_path)
    solver = (solver_factory or Solver)(circuit, SolverConfig())
    log.info("Running %s analysis on '%s'...", type(spec.analysis).__name__, spec.circuit_path)
    result = solver.solve(spec.analysis)
    write_results(result, out)
    log.info("Saved results to %s", out)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="krets", description="SPICE-like circuit simulator (GB300 solve path)")
    ap.add_argument("krets_file")
    ap.add_argument("-g", "--gui", action="store_true", help="not available (no GUI in this package)")
    ap.add_argument("-l", "--log-level", default="info")
    a = ap.parse_args(argv)
    logging.basicConfig(level=getattr(logging, a.log_level.upper(), logging.INFO), format="%(message)s")
    try:
        run(a.krets_file)
    except Exception as e:  # the reference logs and exits with status 1
        log.info("Error: %s", e)
        return 1
    if a.gui:
        log.info("The GUI is not part of this package.")
    return 0


if __name__ == "__main__":
    sys.exit(main())
