import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

GOLDEN = ROOT / "tests" / "golden" / "reference_cases.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    O.lib()
    return O


@pytest.fixture(scope="session")
def built_lib():
    """libkrets_gpu.so built in-tree (compiles with nvcc when missing)."""
    from krets_gb300 import build
    if not build.OUT.exists():
        build.build()
    from krets_gb300 import _lib
    return _lib


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


def circuit_from_case(case):
    from krets_gb300 import parse_circuit_description
    from krets_gb300.generators import resistor_ladder_netlist
    text = case["netlist"] if case.get("netlist") else resistor_ladder_netlist(case["ladder"])
    return parse_circuit_description(text)


def analysis_from_case(case):
    from krets_gb300.analyses import _analysis_from_table
    return _analysis_from_table(case["analysis"])
