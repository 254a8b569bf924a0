"""Build libkrets_gpu.so in-tree with nvcc for sm_103a (no cmake, one -gencode).

    python -m krets_gb300.build        # or krets_gb300.build.build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "libkrets_gpu.so"
BUILD = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def build(verbose: bool = False, extra: list | None = None) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC"] + inc + (extra or [])
    jobs = [
        [nvcc, *ARCH, "-lineinfo", *common, "-c", str(CSRC / "api.cu"), "-o", str(BUILD / "api.o")],
        [nvcc, *common, "-x", "c++", "-c", str(CSRC / "symbolic.cpp"), "-o", str(BUILD / "symbolic.o")],
    ]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=2) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    tmp = OUT.with_suffix(".so.tmp")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), str(BUILD / "api.o"), str(BUILD / "symbolic.o"),
         "-lcudart"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(OUT)
