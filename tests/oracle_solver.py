"""Oracle-backed stand-in for krets_gb300.Solver (test infrastructure): the same
AnalysisResult maps, computed by the CPU oracle, so the CLI and the parquet writer can
be checked on a machine without a GPU.  The product never uses it."""
import numpy as np

from krets_gb300.analyses import AcAnalysis, DcAnalysis, Op, TransientAnalysis, generate_frequencies
from krets_gb300.solver import AnalysisResult, _round_half_away
from krets_gb300.table import element_table
from oracle import oracle as O


class OracleSolver:
    def __init__(self, circuit, config=None):
        self.circuit = circuit
        self.table = element_table(circuit)
        self.names = circuit.names_by_index()

    def _maps(self, rows, key=None, vals=None, cast=float):
        out = []
        for i, row in enumerate(rows):
            d = {nm: cast(row[k]) for k, nm in enumerate(self.names)}
            if key is not None:
                d[key] = vals[i]
            out.append(d)
        return out

    def solve(self, a):
        n = self.circuit.size
        if isinstance(a, Op):
            x = O.op(self.table, n)
            return AnalysisResult("op", self._maps(x[None, :])[0], x)
        if isinstance(a, AcAnalysis):
            f = np.array([v for v in generate_frequencies(a) if v > 0.0])
            z = O.ac(self.table, n, f)
            return AnalysisResult("ac", self._maps(z, "frequency", [complex(v, 0.0) for v in f], complex), z, f)
        if isinstance(a, TransientAnalysis):
            steps = _round_half_away(a.stop_time / a.time_step)
            x = O.tran(self.table, n, a.time_step, steps, method=a.method)
            t = [s * a.time_step for s in range(steps + 1)]
            return AnalysisResult("transient", self._maps(x, "time", t), x, np.array(t))
        if isinstance(a, DcAnalysis):
            idx = next(k for k, el in enumerate(self.circuit.elements) if el.identifier == a.element)
            x = O.dc(self.table, n, idx, a.start, a.stop, a.step_size)
            st = [float(i) for i in range(len(x))]
            return AnalysisResult("dc", self._maps(x, "step", st), x, np.array(st))
        raise TypeError(a)
