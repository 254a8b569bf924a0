"""Parquet result files with the reference's column layout
(crates/krets-result/src/lib.rs:20-208), written by krets_gb300.parquet (no third-party
library needed).

* OP: one row, a column per key.  (The reference takes the order of its HashMap; here
  the keys are sorted so files are reproducible.)
* DC: a column per key, sorted, one row per sweep point, missing values null.
* Transient: as DC with "time" moved first.
* AC: "frequency" (real part) first, then for every other key K, sorted, the columns
  K_mag = |z| and K_phase_deg = atan2(im, re) * 180 / pi.
The file name gets a ".parquet" suffix when it lacks one (lib.rs:10-17).
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Dict, List


def _parquet_name(filename) -> str:
    p = Path(filename)
    return str(p) if p.suffix == ".parquet" else f"{p}.parquet"


def _write(columns: Dict[str, list], filename) -> str:
    from .parquet import write_parquet
    name = _parquet_name(filename)
    write_parquet(columns, name)
    return name


def _headers(rows: List[dict]) -> List[str]:
    return sorted({k for r in rows for k in r})


def write_op_results_to_parquet(data: Dict[str, float], filename) -> str:
    return _write({k: [float(data[k])] for k in sorted(data)}, filename)


def write_dc_results_to_parquet(data: List[Dict[str, float]], filename):
    if not data:
        return None
    return _write({h: [r.get(h) for r in data] for h in _headers(data)}, filename)


def write_tran_results_to_parquet(data: List[Dict[str, float]], filename):
    if not data:
        return None
    hs = _headers(data)
    if "time" in hs:
        hs.remove("time")
        hs.insert(0, "time")
    return _write({h: [r.get(h) for r in data] for h in hs}, filename)


def write_ac_results_to_parquet(data: List[Dict[str, complex]], filename):
    if not data:
        return None
    cols = {"frequency": [None if r.get("frequency") is None else complex(r["frequency"]).real for r in data]}
    for h in (k for k in _headers(data) if k != "frequency"):
        mag, ph = [], []
        for r in data:
            v = r.get(h)
            if v is None:
                mag.append(None)
                ph.append(None)
            else:
                v = complex(v)
                mag.append(math.sqrt(v.real * v.real + v.imag * v.imag))
                ph.append(math.atan2(v.imag, v.real) * 180.0 / math.pi)
        cols[f"{h}_mag"] = mag
        cols[f"{h}_phase_deg"] = ph
    return _write(cols, filename)


def write_results(result, filename):
    """Write an AnalysisResult with the writer of its kind (main.rs:104-131)."""
    return {"op": write_op_results_to_parquet, "dc": write_dc_results_to_parquet,
            "ac": write_ac_results_to_parquet,
            "transient": write_tran_results_to_parquet}[result.kind](result.data, filename)
