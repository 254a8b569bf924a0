"""SolverConfig (crates/krets-solver/src/config.rs:4-36).

`minimum_resistance` and `minimum_conductance` are declared by the reference
but never read by it; they are kept for interface parity and likewise unused.
"""
from dataclasses import dataclass


@dataclass
class SolverConfig:
    relative_tolerance: float = 0.001
    current_absolute_tolerance: float = 1e-12
    voltage_absolute_tolerance: float = 1e-6
    maximum_iterations: int = 300
    minimum_resistance: float = 1e-3
    minimum_conductance: float = 1e-12
