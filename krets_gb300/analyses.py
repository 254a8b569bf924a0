"""Analysis specifications and krets.toml loading
(crates/krets-parser/src/analyses.rs:8-165).

`AnalysisSpec.from_file` reads the same TOML the reference CLI reads
(`circuit_path` plus one `[analysis.<op|dc|ac|transient>]` table).  The
extensions of this package (integration method, source-lag switch, precision
mode) live in an optional `[gb300]` table, so every existing krets.toml still
parses unchanged.
"""
from __future__ import annotations

import math
import tomllib
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Union

from .errors import ParseError


@dataclass
class Op:
    pass


@dataclass
class DcAnalysis:
    element: str
    start: float
    stop: float
    step_size: float


@dataclass
class Linear:
    total_points: int


@dataclass
class Decade:
    points_per_decade: int


@dataclass
class Octave:
    points_per_octave: int


AcSweep = Union[Linear, Decade, Octave]


@dataclass
class AcAnalysis:
    sweep: AcSweep
    fstart: float
    fstop: float

    def generate_frequencies(self) -> List[float]:
        return generate_frequencies(self)


@dataclass
class TransientAnalysis:
    time_step: float
    stop_time: float
    # Extensions (not in the reference, which has backward Euler only):
    method: str = "be"            # "be" (reference) or "tr" (trapezoidal)
    # The reference evaluates sources, in the first Newton iteration of a
    # step, at the previous step's time (transient.rs:49 + stampable.rs:1043).
    # None = reference behaviour for "be", no lag for "tr".
    source_lag: Optional[bool] = None


Analysis = Union[Op, DcAnalysis, AcAnalysis, TransientAnalysis]


def generate_frequencies(a: AcAnalysis) -> List[float]:
    """Frequency list of an AC sweep, restating analyses.rs:80-158.

    Decade/octave sweeps multiply a running frequency by a fixed factor (they
    do not call pow per point), append fstop when the loop steps past it, then
    sort and dedup.  The arithmetic is IEEE f64 in the same order, so the list
    is bit-identical to the reference's.
    """
    f0, f1 = a.fstart, a.fstop
    freqs: List[float] = []
    if f0 <= 0.0 or f1 <= 0.0 or f0 > f1:
        return freqs
    sw = a.sweep
    if isinstance(sw, Linear):
        tp = sw.total_points
        if tp == 1:
            freqs.append(f0)
        elif tp > 1:
            step = (f1 - f0) / float(tp - 1)
            for i in range(tp):
                freqs.append(f0 + float(i) * step)
    else:
        if isinstance(sw, Decade):
            ppx = sw.points_per_decade
            if ppx == 0:
                return freqs
            span = math.log10(f1 / f0)
            factor = 10.0 ** (1.0 / float(ppx))
        else:
            ppx = sw.points_per_octave
            if ppx == 0:
                return freqs
            span = math.log2(f1 / f0)
            factor = 2.0 ** (1.0 / float(ppx))
        total = int(_round_half_away(span * float(ppx))) + 1
        cur = f0
        for _ in range(total):
            if cur > f1 * (1.0 + 1e-9):
                break
            freqs.append(cur)
            cur *= factor
            if cur > f1 and (not freqs or freqs[-1] < f1):
                freqs.append(f1)
                break
        if not freqs or freqs[-1] < f1 * (1.0 - 1e-9):
            freqs.append(f1)
    freqs.sort()
    out: List[float] = []
    for f in freqs:
        if not out or out[-1] != f:
            out.append(f)
    return out


def _round_half_away(x: float) -> float:
    # Rust f64::round rounds half away from zero.
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def _analysis_from_table(tab: dict) -> Analysis:
    if len(tab) != 1:
        raise ParseError("exactly one analysis table expected")
    (kind, body), = tab.items()
    if kind == "op":
        return Op()
    if kind == "dc":
        return DcAnalysis(str(body["element"]), float(body["start"]), float(body["stop"]),
                          float(body["step_size"]))
    if kind == "ac":
        sw = body["sweep"]
        var = sw["variation"]
        if var == "Linear":
            sweep = Linear(int(sw["total_points"]))
        elif var == "Decade":
            sweep = Decade(int(sw["points_per_decade"]))
        elif var == "Octave":
            sweep = Octave(int(sw["points_per_octave"]))
        else:
            raise ParseError(f"unknown AC variation {var}")
        return AcAnalysis(sweep, float(body["fstart"]), float(body["fstop"]))
    if kind == "transient":
        return TransientAnalysis(float(body["time_step"]), float(body["stop_time"]))
    raise ParseError(f"unknown analysis '{kind}'")


@dataclass
class AnalysisSpec:
    circuit_path: Path
    analysis: Analysis
    extensions: dict = field(default_factory=dict)

    @staticmethod
    def from_str(text: str) -> "AnalysisSpec":
        try:
            d = tomllib.loads(text)
        except tomllib.TOMLDecodeError as e:
            raise ParseError(f"TOML deserialization error: {e}")
        ext = d.get("gb300", {})
        an = _analysis_from_table(d["analysis"])
        if isinstance(an, TransientAnalysis):
            an.method = ext.get("method", "be")
            if "source_lag" in ext:
                an.source_lag = bool(ext["source_lag"])
        return AnalysisSpec(Path(d["circuit_path"]), an, ext)

    @staticmethod
    def from_file(path) -> "AnalysisSpec":
        return AnalysisSpec.from_str(Path(path).read_text())
