"""Python mirror of krets_solver's public API over the C ABI.

    Solver(circuit, config).solve(analysis) -> AnalysisResult

as in crates/krets-solver/src/solver.rs:17-52 (dispatcher) and
crates/krets-solver/src/lib.rs:13-76 (AnalysisResult with into_op/into_dc/
into_ac/into_transient).  Results are dicts keyed like the reference's maps:
"V(<node>)", "I(<element id>)", plus "time", "frequency" or "step".  Every
solve runs on the GPU through libkrets_gpu.so; there is no CPU path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any, Dict, List

import numpy as np

from . import _lib
from .analyses import AcAnalysis, DcAnalysis, Op, TransientAnalysis, generate_frequencies
from .config import SolverConfig
from .errors import ElementNotFound, InvalidElementFormat
from .netlist import KIND_I, KIND_V, Circuit
from .table import element_table


@dataclass
class AnalysisResult:
    kind: str                 # "op" | "dc" | "ac" | "transient"
    data: Any                 # dict or list of dicts, as the reference
    array: np.ndarray         # the same values as an array [points][n] (reference numbering)
    axis: np.ndarray | None = None   # time / frequency / step values

    def into_op(self) -> Dict[str, float]:
        if self.kind != "op":
            raise TypeError("Called `into_op()` on a non-Op result")
        return self.data

    def into_dc(self) -> List[Dict[str, float]]:
        if self.kind != "dc":
            raise TypeError("Called `into_dc()` on a non-Dc result")
        return self.data

    def into_ac(self) -> List[Dict[str, complex]]:
        if self.kind != "ac":
            raise TypeError("Called `into_ac()` on a non-Ac result")
        return self.data

    def into_transient(self) -> List[Dict[str, float]]:
        if self.kind != "transient":
            raise TypeError("Called `into_transient()` on a non-Transient result")
        return self.data


def _round_half_away(x: float) -> int:
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


class Solver:
    """Owns the circuit and its compiled device topology (solver.rs:17-25)."""

    def __init__(self, circuit: Circuit, config: SolverConfig | None = None, nmos_resolved: bool = False):
        """nmos_resolved: stamp NMOS devices (the reference's stamp with its node lookups
        resolved); the default reproduces the reference, whose NMOS stamps nothing."""
        self.circuit = circuit
        self.config = config or SolverConfig()
        self.table = element_table(circuit, nmos_resolved)
        self.names = circuit.names_by_index()
        self.gpu = _lib.GpuCircuit(self.table, circuit.size, self.config)

    def _maps(self, rows: np.ndarray, extra_key=None, extra=None, cast=float):
        out = []
        for i, row in enumerate(rows):
            d = {nm: cast(row[k]) for k, nm in enumerate(self.names)}
            if extra_key is not None:
                d[extra_key] = extra[i]
            out.append(d)
        return out

    def solve(self, analysis) -> AnalysisResult:
        if isinstance(analysis, Op):
            x, _ = self.gpu.op()
            return AnalysisResult("op", self._maps(x[None, :])[0], x)
        if isinstance(analysis, DcAnalysis):
            idx = next((k for k, el in enumerate(self.circuit.elements)
                        if el.identifier == analysis.element), None)
            if idx is None:
                raise ElementNotFound(f"Element '{analysis.element}' not found in the netlist")
            if self.circuit.elements[idx].kind not in (KIND_V, KIND_I):
                raise InvalidElementFormat("DC sweep element must be a voltage or current source")
            x = self.gpu.dc(idx, analysis.start, analysis.stop, analysis.step_size)
            steps = [float(i) for i in range(len(x))]
            return AnalysisResult("dc", self._maps(x, "step", steps), x, np.array(steps))
        if isinstance(analysis, AcAnalysis):
            freqs = [f for f in generate_frequencies(analysis) if f > 0.0]
            z = self.gpu.ac(np.array(freqs)) if freqs else np.zeros((0, self.circuit.size), complex)
            data = self._maps(z, "frequency", [complex(f, 0.0) for f in freqs], cast=complex)
            return AnalysisResult("ac", data, z, np.array(freqs))
        if isinstance(analysis, TransientAnalysis):
            h = analysis.time_step
            n_steps = _round_half_away(analysis.stop_time / h)   # transient.rs:29
            lag = analysis.source_lag
            if lag is None:
                lag = analysis.method == "be"
            x = self.gpu.tran(h, n_steps, analysis.method, lag)
            times = [float(s) * h for s in range(n_steps + 1)]
            return AnalysisResult("transient", self._maps(x, "time", times), x, np.array(times))
        raise TypeError(f"unknown analysis {analysis!r}")
