"""krets_gb300 — GB300-native (sm_103a) MNA solve path for krets circuits.
"""
from .config import SolverConfig  # noqa: F401
from .analyses import (AcAnalysis, AnalysisSpec, DcAnalysis, Decade, Linear, Octave, Op,  # noqa: F401
                       TransientAnalysis, generate_frequencies)
from .netlist import Circuit, parse_circuit_description, parse_circuit_description_file  # noqa: F401
from .solver import AnalysisResult, Solver  # noqa: F401
