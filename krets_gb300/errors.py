"""Error types mirroring krets_solver::Error (crates/krets-solver/src/error.rs:4-36)
and the parser's error enum (crates/krets-parser/src/error.rs), plus the two
conditions a device path adds (a bounded wait that ran out, a CUDA failure).

Every C-ABI status code in include/krets_gpu.h maps to one class here.
"""


class KretsError(Exception):
    """Base class of every error this package raises."""


class ParseError(KretsError):
    """Netlist or krets.toml could not be parsed (parser error.rs)."""


class ElementNotFound(KretsError):
    """error.rs:8-9 — a DC sweep names an element the netlist lacks."""


class MaximumIterationsExceeded(KretsError):
    """error.rs:12-13 — Newton did not converge within maximum_iterations."""


class InvalidElementFormat(KretsError):
    """error.rs:16-17 — e.g. a DC sweep element that is not a V or I source."""


class Unexpected(KretsError):
    """error.rs:20-21."""


class DecompositionFailed(KretsError):
    """error.rs:24-25 — a zero (or non-finite) pivot during factorisation."""


class MatrixBuild(KretsError):
    """error.rs:28-29."""


class MatrixDecomposition(KretsError):
    """error.rs:32-33 (OP analysis maps factorisation failures to this)."""


class NotImplementedInReference(KretsError):
    """The reference panics with todo!() here (BJT stamps, NMOS AC stamp)."""


class DeviceTimeout(KretsError):
    """A bounded device-side wait ran out (no reference counterpart)."""


class CudaError(KretsError):
    """A CUDA runtime call failed (no reference counterpart)."""


class PivotUnstable(KretsError):
    """A static pivot grew beyond the growth limit and no fallback was allowed."""
