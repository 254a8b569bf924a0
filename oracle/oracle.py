"""ctypes front of the CPU oracle (krets_oracle.c) — TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check (or time, as the CPU baseline) the device path.  The product never
imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libkrets_oracle.so"

OK, SINGULAR, MAXITER, NOTFOUND, BADELEM, NOTIMPL, NOMEM, NONFINITE = range(8)


class OracleError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"oracle {where} failed with status {code}")
        self.code = code


class Cfg(ctypes.Structure):
    _fields_ = [("reltol", ctypes.c_double), ("iabstol", ctypes.c_double),
                ("vabstol", ctypes.c_double), ("maxiter", ctypes.c_int32),
                ("faithful", ctypes.c_int32)]


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        L.ko_op.argtypes = [P, I, I, P, P, P]
        L.ko_dc.argtypes = [P, I, I, P, I, D, D, D, P, I, P]
        L.ko_ac.argtypes = [P, I, I, P, P, I, P, P]
        L.ko_tran.argtypes = [P, I, I, P, D, I, I, I, P, P]
        L.ko_assemble.argtypes = [P, I, I, I, D, I, D, P, P, P]
        L.ko_lu_solve_csc.argtypes = [I, P, P, P, P, P]
        L.ko_adjoint_tran.argtypes = [P, I, I, P, D, I, I, I, P, P]
        L.ko_tran_adaptive.argtypes = [P, I, I, P, D, D, I, D, D, D, I, P, P, P]
        L.ko_pulse.argtypes = [P, D]
        L.ko_pulse.restype = D
        L.ko_sin.argtypes = [P, D]
        L.ko_sin.restype = D
        assert L.ko_abi_elem_size() == 104
        _lib = L
    return _lib


def _cfg(config=None, faithful=False) -> Cfg:
    if config is None:
        return Cfg(0.001, 1e-12, 1e-6, 300, int(faithful))
    return Cfg(config.relative_tolerance, config.current_absolute_tolerance,
               config.voltage_absolute_tolerance, config.maximum_iterations, int(faithful))


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def op(table, n, config=None):
    x = np.zeros(n)
    it = ctypes.c_int(0)
    c = _cfg(config)
    st = lib().ko_op(_p(table), len(table), n, ctypes.byref(c), _p(x), ctypes.byref(it))
    if st:
        raise OracleError(st, "op")
    return x


def dc(table, n, sweep_index, start, stop, step, config=None):
    npts = int(abs((stop - start) / step)) + 1
    x = np.zeros((npts, n))
    got = ctypes.c_int(0)
    c = _cfg(config)
    st = lib().ko_dc(_p(table), len(table), n, ctypes.byref(c), sweep_index, start, stop, step,
                     _p(x), npts, ctypes.byref(got))
    if st:
        raise OracleError(st, "dc")
    return x


def ac(table, n, freqs, config=None):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    x = np.zeros((len(freqs), n, 2))
    kept = ctypes.c_int(0)
    c = _cfg(config)
    st = lib().ko_ac(_p(table), len(table), n, ctypes.byref(c), _p(freqs), len(freqs), _p(x),
                     ctypes.byref(kept))
    if st:
        raise OracleError(st, "ac")
    z = x[:kept.value, :, 0] + 1j * x[:kept.value, :, 1]
    return z


def tran(table, n, h, n_steps, method="be", lag=None, config=None, faithful=False,
         return_iters=False):
    m = 1 if method == "tr" else 0
    if lag is None:
        lag = (m == 0)
    x = np.zeros((n_steps + 1, n))
    iters = np.zeros(max(n_steps, 1), dtype=np.int32)
    c = _cfg(config, faithful)
    st = lib().ko_tran(_p(table), len(table), n, ctypes.byref(c), h, n_steps, m, int(bool(lag)),
                       _p(x), _p(iters))
    if st:
        raise OracleError(st, "tran")
    return (x, iters) if return_iters else x


def tran_adaptive(table, n, h0, t_stop, method="tr", lte_tol=1e-3, h_min=None, h_max=None, max_points=100000,
                  config=None):
    """Adaptive-step transient (truncation-error control): (t[points], x[points][n])."""
    m = 1 if method == "tr" else 0
    h_min = h0 * 1e-6 if h_min is None else h_min
    h_max = t_stop if h_max is None else h_max
    t = np.zeros(max_points)
    x = np.zeros((max_points, n))
    got = ctypes.c_int(0)
    c = _cfg(config)
    st = lib().ko_tran_adaptive(_p(table), len(table), n, ctypes.byref(c), h0, t_stop, m, lte_tol, h_min, h_max,
                                max_points, _p(t), _p(x), ctypes.byref(got))
    if st:
        raise OracleError(st, "tran_adaptive")
    return t[:got.value], x[:got.value]


def adjoint_tran(table, n, h, n_steps, out, method="tr", config=None):
    """Loss sum_s x_s[out]^2 and its gradient w.r.t. every element value (FP64 adjoint)."""
    loss = ctypes.c_double(0.0)
    grad = np.zeros(len(table))
    c = _cfg(config)
    st = lib().ko_adjoint_tran(_p(table), len(table), n, ctypes.byref(c), h, n_steps,
                               1 if method == "tr" else 0, out, ctypes.byref(loss), _p(grad))
    if st:
        raise OracleError(st, "adjoint_tran")
    return loss.value, grad


def assemble(table, n, mode="dc", h=0.0, method="be", freq=0.0, sol=None):
    md = {"dc": 0, "ac": 1, "tran": 2}[mode]
    w = 2 if md == 1 else 1
    A = np.zeros((n, n, w))
    b = np.zeros((n, w))
    s = np.zeros(n) if sol is None else np.ascontiguousarray(sol, dtype=np.float64)
    st = lib().ko_assemble(_p(table), len(table), n, md, h, 1 if method == "tr" else 0, freq,
                           _p(s), _p(A), _p(b))
    if st:
        raise OracleError(st, "assemble")
    if w == 2:
        return A[..., 0] + 1j * A[..., 1], b[:, 0] + 1j * b[:, 1]
    return A[..., 0], b[:, 0]


def pulse(params, t):
    w = np.ascontiguousarray(params, dtype=np.float64)
    return lib().ko_pulse(_p(w), t)


def sin(params, t):
    w = np.ascontiguousarray(params, dtype=np.float64)
    return lib().ko_sin(_p(w), t)


def lu_solve_csc(n, indptr, indices, data, b):
    ap = np.ascontiguousarray(indptr, dtype=np.int32)
    ai = np.ascontiguousarray(indices, dtype=np.int32)
    ax = np.ascontiguousarray(data, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    st = lib().ko_lu_solve_csc(n, _p(ap), _p(ai), _p(ax), _p(bb), _p(x))
    if st:
        raise OracleError(st, "lu")
    return x
