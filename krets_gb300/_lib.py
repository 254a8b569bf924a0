"""ctypes binding of libkrets_gpu.so (the C ABI in include/krets_gpu.h).

The library is built in-tree (krets_gb300/build.py).  There is no CPU fallback:
when the library is missing, `lib()` raises, and every solve reports a CUDA
error when no GPU is present.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import errors as E
from .table import ELEM_DTYPE

LIB_PATH = Path(__file__).resolve().parent / "libkrets_gpu.so"

OK = 0
ELEMENT_NOT_FOUND, MAX_ITERATIONS, INVALID_ELEMENT, UNEXPECTED = 1, 2, 3, 4
DECOMPOSITION_FAILED, MATRIX_BUILD, MATRIX_DECOMPOSITION, NOT_IMPLEMENTED = 5, 6, 7, 8
TIMEOUT, CUDA, INVALID_ARGUMENT, OUT_OF_MEMORY, PIVOT_UNSTABLE = 9, 10, 11, 12, 13

METHOD = {"be": 0, "tr": 1}
PREC_FP64, PREC_MIXED, PREC_DF = 0, 1, 2
MODE_DC, MODE_AC, MODE_TRAN = 0, 1, 2

PROG_ARRAYS = ["q", "prow", "lu_rowptr", "lu_col", "lu_diag", "a_rowptr", "a_col", "a_slot", "a_cptr",
               "a_contrib", "b_cptr", "b_contrib", "piv_ptr", "piv", "upd", "lev_ptr", "lev_rows",
               "ulev_ptr", "ulev_rows", "el_pos", "meta", "tprog", "tpoff", "sprog", "spoff", "iprog", "ipoff",
               "imap"]

_EXC = {
    ELEMENT_NOT_FOUND: E.ElementNotFound, MAX_ITERATIONS: E.MaximumIterationsExceeded,
    INVALID_ELEMENT: E.InvalidElementFormat, UNEXPECTED: E.Unexpected,
    DECOMPOSITION_FAILED: E.DecompositionFailed, MATRIX_BUILD: E.MatrixBuild,
    MATRIX_DECOMPOSITION: E.MatrixDecomposition, NOT_IMPLEMENTED: E.NotImplementedInReference,
    TIMEOUT: E.DeviceTimeout, CUDA: E.CudaError, INVALID_ARGUMENT: E.KretsError,
    OUT_OF_MEMORY: E.CudaError, PIVOT_UNSTABLE: E.PivotUnstable,
}


class Config(ctypes.Structure):
    _fields_ = [("relative_tolerance", ctypes.c_double), ("current_absolute_tolerance", ctypes.c_double),
                ("voltage_absolute_tolerance", ctypes.c_double), ("maximum_iterations", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int32
_D = ctypes.c_double


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise E.CudaError(f"{LIB_PATH} is not built (run krets_gb300.build.build()); "
                              "there is no CPU fallback")
        L = ctypes.CDLL(str(LIB_PATH))
        sig = {
            "krets_circuit_create": [_P, _I, _I, _P, _P],
            "krets_circuit_destroy": [_P],
            "krets_circuit_info": [_P, _I, _P, _P, _P, _P, _P],
            "krets_op": [_P, _P, _P],
            "krets_dc": [_P, _I, _D, _D, _D, _P, _I, _P],
            "krets_ac": [_P, _P, _I, _P, _P],
            "krets_tran": [_P, _D, _I, _I, _I, _I, _P],
            "krets_batch_tran": [_P, _I, _P, _D, _I, _I, _I, _I, _P, _P],
            "krets_batch_ac": [_P, _I, _P, _P, _I, _I, _P, _P],
            "krets_batch_tran_noalloc": [_P, _I, _P, _D, _I, _I, _I, _I, _P, _P],
            "krets_adjoint_tran": [_P, _I, _P, _D, _I, _I, _I, _I, _I, _P, _P],
            "krets_multi_create": [_I, _P, _P, _P, _I, _D, _P],
            "krets_multi_destroy": [_P],
            "krets_multi_info": [_P, _P, _I],
            "krets_multi_tran": [_P, _I, _I, _P, _P, _P],
            "krets_multi_last_timing": [_P, _P, _P],
            "krets_direct_host_access": [],
            "krets_batch_op": [_P, _I, _P, _P, _P],
            "krets_batch_dc": [_P, _I, _P, _I, _D, _D, _D, _P, _I, _P, _P],
            "krets_batch_tran_adaptive": [_P, _I, _P, _D, _D, _I, _D, _D, _D, _I, _P, _P, _P, _P],
            "krets_batch_tran_probe": [_P, _I, _P, _D, _I, _I, _I, _I, _P, _P, _P],
            "krets_last_timing": [_P, _P, _P],
            "krets_last_launch": [_P, _P, _I],
            "krets_last_refine_stats": [_P, _P, _P],
            "krets_device_alloc": [ctypes.c_size_t, _P],
            "krets_device_free": [_P],
            "krets_memcpy_h2d": [_P, _P, ctypes.c_size_t],
            "krets_memcpy_d2h": [_P, _P, ctypes.c_size_t],
            "krets_flush_l2": [_P],
            "krets_host_register": [_P, ctypes.c_size_t],
            "krets_host_unregister": [_P],
            "krets_device_synchronize": [],
            "krets_symbolic_export": [_P, _I, _I, _I, _I, _D, _D, _I, _I, _P, ctypes.c_int64, _P],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int32
        L.krets_status_string.argtypes = [_I]
        L.krets_status_string.restype = ctypes.c_char_p
        L.krets_last_error_message.argtypes = []
        L.krets_last_error_message.restype = ctypes.c_char_p
        L.krets_launch_count.argtypes = []
        L.krets_launch_count.restype = ctypes.c_int64
        _lib = L
    return _lib


def check(status: int, what: str = ""):
    if status == OK:
        return
    L = lib()
    msg = L.krets_last_error_message().decode(errors="replace")
    cls = _EXC.get(status, E.KretsError)
    raise cls(f"{what}: {L.krets_status_string(status).decode()} ({msg})")


def host_buffer(shape, dtype=np.float64) -> np.ndarray:
    """Zeroed output buffer whose pages are resident (written by the CPU): the library may
    have the GPU write host buffers in place, and a GPU first touch of fresh pages is far
    slower than the CPU's."""
    a = np.empty(shape, dtype)
    a.fill(0)
    return a


class PinnedBuffer:
    """A host array page-locked through the library (krets_host_register) until close():
    the double-float batched transient copies its results into pinned memory span by span
    with the copy engines.  Where the GPU shares the host's page tables (NVLink-C2C) an
    ordinary array written in place is faster once the buffer is reused; pinning pays for
    one call into fresh memory, or where the GPU cannot map host memory.  `.array` is the
    numpy view; its pages are touched first."""

    def __init__(self, shape, dtype=np.float64):
        self.array = host_buffer(shape, dtype)
        self._ptr = self.array.ctypes.data
        check(lib().krets_host_register(ctypes.c_void_p(self._ptr), self.array.nbytes), "host_register")

    def close(self):
        if self._ptr:
            lib().krets_host_unregister(ctypes.c_void_p(self._ptr))
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ptr(a) -> ctypes.c_void_p:
    if a is None:
        return None
    if isinstance(a, DeviceArray):
        return ctypes.c_void_p(a.ptr)
    return a.ctypes.data_as(ctypes.c_void_p)


class DeviceArray:
    """Device memory owned through the library (for callers without a CUDA binding)."""

    def __init__(self, shape, dtype=np.float64):
        self.shape = tuple(shape) if isinstance(shape, (tuple, list)) else (int(shape),)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        check(lib().krets_device_alloc(max(self.nbytes, 16), ctypes.byref(p)), "device alloc")
        self.ptr = p.value

    def upload(self, host: np.ndarray):
        h = np.ascontiguousarray(host, dtype=self.dtype)
        assert h.nbytes == self.nbytes
        check(lib().krets_memcpy_h2d(ctypes.c_void_p(self.ptr), h.ctypes.data_as(ctypes.c_void_p), self.nbytes))
        return self

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.shape, self.dtype) if out is None else out
        check(lib().krets_memcpy_d2h(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr), self.nbytes))
        return out

    def free(self):
        if self.ptr:
            lib().krets_device_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class MultiCircuit:
    """Many distinct linear circuits (tables with their own unknown counts) run together."""

    def __init__(self, tables, sizes, method="be", h=1e-9):
        self.sizes = np.asarray(sizes, dtype=np.int32)
        self.tables = [np.ascontiguousarray(t, dtype=ELEM_DTYPE) for t in tables]
        el = np.concatenate(self.tables) if self.tables else np.zeros(0, ELEM_DTYPE)
        off = np.zeros(len(self.tables) + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(t) for t in self.tables])
        self.method = method
        self.h = None
        h_ = ctypes.c_void_p()
        check(lib().krets_multi_create(len(self.tables), ptr(el), ptr(off), ptr(self.sizes), METHOD[method], h,
                                       ctypes.byref(h_)), "multi_create")
        self.h = h_

    def close(self):
        if self.h:
            lib().krets_multi_destroy(self.h)
            self.h = None

    __del__ = close

    def offsets(self, n_steps):
        off = np.zeros(len(self.sizes), dtype=np.int64)
        off[1:] = np.cumsum((n_steps + 1) * self.sizes.astype(np.int64))[:-1]
        return off

    def total(self, n_steps):
        return int((n_steps + 1) * self.sizes.astype(np.int64).sum())

    def tran(self, n_steps, lag=None, out=None):
        """Operating point then n_steps steps; returns the flat output (or fills `out`,
        a host array or DeviceArray of total(n_steps) doubles) and per-circuit status."""
        if lag is None:
            lag = self.method == "be"
        if out is None:
            out = host_buffer(self.total(n_steps))
        st = np.zeros(len(self.sizes), dtype=np.int32)
        check(lib().krets_multi_tran(self.h, n_steps, int(bool(lag)), ptr(out), None, ptr(st)), "multi_tran")
        return out, st

    def split(self, flat, n_steps):
        off = self.offsets(n_steps)
        return [flat[o:o + (n_steps + 1) * n].reshape(n_steps + 1, n) for o, n in zip(off, self.sizes)]

    def info(self):
        v = np.zeros(16, dtype=np.int64)
        check(lib().krets_multi_info(self.h, ptr(v), len(v)), "multi_info")
        return v

    def timing(self):
        k = ctypes.c_float()
        c = ctypes.c_float()
        check(lib().krets_multi_last_timing(self.h, ctypes.byref(k), ctypes.byref(c)))
        return k.value, c.value


class GpuCircuit:
    """Owns a krets_circuit handle (compiled topology on the device)."""

    def __init__(self, table: np.ndarray, n: int, config=None):
        self.table = np.ascontiguousarray(table, dtype=ELEM_DTYPE)
        self.n = int(n)
        self.ne = len(self.table)
        cfg = None
        if config is not None:
            cfg = Config(config.relative_tolerance, config.current_absolute_tolerance,
                         config.voltage_absolute_tolerance, config.maximum_iterations, 0)
        h = ctypes.c_void_p()
        check(lib().krets_circuit_create(ptr(self.table), self.ne, self.n,
                                         ctypes.byref(cfg) if cfg is not None else None, ctypes.byref(h)),
              "krets_circuit_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().krets_circuit_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- analyses
    def op(self):
        x = host_buffer(self.n)
        it = ctypes.c_int32(0)
        check(lib().krets_op(self.h, ptr(x), ctypes.byref(it)), "op")
        return x, it.value

    def dc(self, sweep_index, start, stop, step):
        npts = int(abs((stop - start) / step)) + 1
        x = host_buffer((npts, self.n))
        got = ctypes.c_int32(0)
        check(lib().krets_dc(self.h, sweep_index, start, stop, step, ptr(x), npts, ctypes.byref(got)), "dc")
        return x[:got.value]

    def ac(self, freqs):
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        x = host_buffer((max(len(f), 1), self.n, 2))
        kept = ctypes.c_int32(0)
        check(lib().krets_ac(self.h, ptr(f), len(f), ptr(x), ctypes.byref(kept)), "ac")
        return x[:kept.value, :, 0] + 1j * x[:kept.value, :, 1]

    def tran(self, h, n_steps, method="be", lag=None, refactor_each_step=False):
        m = METHOD[method]
        if lag is None:
            lag = m == 0
        x = host_buffer((n_steps + 1, self.n))
        check(lib().krets_tran(self.h, h, n_steps, m, int(bool(lag)), int(bool(refactor_each_step)), ptr(x)),
              "tran")
        return x

    def batch_op(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        ni = v.shape[0]
        x = host_buffer((ni, self.n))
        st = np.zeros(ni, dtype=np.int32)
        check(lib().krets_batch_op(self.h, ni, ptr(v), ptr(x), ptr(st)), "batch_op")
        return x

    def batch_dc(self, values, sweep_index, start, stop, step):
        """Warm-started DC sweep of every instance: [n_inst][points][n], statuses."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        ni = v.shape[0]
        npts = int(abs((stop - start) / step)) + 1
        x = host_buffer((ni, npts, self.n))
        st = np.zeros(ni, dtype=np.int32)
        got = ctypes.c_int32(0)
        check(lib().krets_batch_dc(self.h, ni, ptr(v), sweep_index, start, stop, step, ptr(x), npts,
                                   ctypes.byref(got), ptr(st)), "batch_dc")
        return x[:, :got.value], st

    def batch_tran_probe(self, values, h, n_steps, probe, method="tr", lag=None, out=None, n_inst=None):
        """Double-float batched transient writing only the unknowns in `probe` each step:
        [n_inst][n_steps+1][len(probe)]."""
        m = METHOD[method]
        if lag is None:
            lag = m == 0
        pr = np.ascontiguousarray(probe, dtype=np.int32)
        if isinstance(values, DeviceArray):
            ni = values.shape[0] if n_inst is None else n_inst
        else:
            values = np.ascontiguousarray(values, dtype=np.float64)
            ni = values.shape[0]
        if out is None:
            out = host_buffer((ni, n_steps + 1, len(pr)))
        st = np.zeros(ni, dtype=np.int32)
        check(lib().krets_batch_tran_probe(self.h, ni, ptr(values), h, n_steps, m, int(bool(lag)), len(pr), ptr(pr),
                                           ptr(out), ptr(st)), "batch_tran_probe")
        return out

    def batch_tran_adaptive(self, values, h0, t_stop, method="tr", lte_tol=1e-3, h_min=None, h_max=None,
                            max_points=20000, n_inst=None):
        """Truncation-error step control: per instance (t[points], x[points][n]) and statuses.
        values None runs one instance with the nominal values."""
        m = METHOD[method]
        h_min = h0 * 1e-6 if h_min is None else h_min
        h_max = t_stop if h_max is None else h_max
        if values is None:
            ni = 1 if n_inst is None else n_inst
        else:
            values = np.ascontiguousarray(values, dtype=np.float64)
            ni = values.shape[0]
        t = host_buffer((ni, max_points))
        x = host_buffer((ni, max_points, self.n))
        npts = np.zeros(ni, dtype=np.int32)
        st = np.zeros(ni, dtype=np.int32)
        rc = lib().krets_batch_tran_adaptive(self.h, ni, ptr(values), h0, t_stop, m, lte_tol, h_min, h_max,
                                             max_points, ptr(t), ptr(x), ptr(npts), ptr(st))
        return [(t[i, :npts[i]], x[i, :npts[i]]) for i in range(ni)], st, rc

    def batch_tran(self, values, h, n_steps, method="tr", lag=None, precision=PREC_MIXED, out=None,
                   n_inst=None):
        m = METHOD[method]
        if lag is None:
            lag = m == 0
        if isinstance(values, DeviceArray):
            ni = values.shape[0] if n_inst is None else n_inst
        elif values is None:
            ni = 1 if n_inst is None else n_inst
        else:
            values = np.ascontiguousarray(values, dtype=np.float64)
            ni = values.shape[0]
        if out is None:
            out = host_buffer((ni, n_steps + 1, self.n))
        st = np.zeros(ni, dtype=np.int32)
        check(lib().krets_batch_tran(self.h, ni, ptr(values), h, n_steps, m, int(bool(lag)), precision, ptr(out),
                                     ptr(st)), "batch_tran")
        return out

    def batch_tran_noalloc(self, d_values, h, n_steps, d_out, d_status, n_inst, method="tr", lag=None,
                           precision=PREC_MIXED):
        """krets_batch_tran_noalloc: device buffers only, no device allocation inside."""
        m = METHOD[method]
        if lag is None:
            lag = m == 0
        check(lib().krets_batch_tran_noalloc(self.h, n_inst, ptr(d_values), h, n_steps, m, int(bool(lag)),
                                             precision, ptr(d_out), ptr(d_status)), "batch_tran_noalloc")

    def adjoint_tran(self, values, h, n_steps, out_unknown, method="tr", checkpoint_every=100, gradient=True,
                     n_inst=None):
        """Loss sum_n x_out(t_n)^2 per instance and its gradient w.r.t. every element value."""
        if values is None:
            ni = 1 if n_inst is None else n_inst
        elif isinstance(values, DeviceArray):
            ni = values.shape[0]
        else:
            values = np.ascontiguousarray(values, dtype=np.float64)
            ni = values.shape[0]
        loss = host_buffer(ni)
        grad = host_buffer((ni, self.ne)) if gradient else None
        check(lib().krets_adjoint_tran(self.h, ni, ptr(values), h, n_steps, METHOD[method], out_unknown,
                                       checkpoint_every, int(bool(gradient)), ptr(loss), ptr(grad)),
              "adjoint_tran")
        return (loss, grad) if gradient else loss

    def batch_ac(self, values, freqs, precision=PREC_MIXED, out=None):
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        if values is None:
            ni = 1
        elif isinstance(values, DeviceArray):
            ni = values.shape[0]
        else:
            values = np.ascontiguousarray(values, dtype=np.float64)
            ni = values.shape[0]
        host_out = out is None
        if host_out:
            out = host_buffer((ni, len(f), self.n, 2))
        st = np.zeros(ni * len(f), dtype=np.int32)
        check(lib().krets_batch_ac(self.h, ni, ptr(values), ptr(f), len(f), precision, ptr(out), ptr(st)),
              "batch_ac")
        if host_out:
            return out[..., 0] + 1j * out[..., 1]
        return out

    # -------------------------------------------------------------- diagnostics
    def timing(self):
        k = ctypes.c_float()
        c = ctypes.c_float()
        check(lib().krets_last_timing(self.h, ctypes.byref(k), ctypes.byref(c)))
        return k.value, c.value

    def refine_stats(self):
        hist = np.zeros(8, dtype=np.int64)
        fb = ctypes.c_int32()
        check(lib().krets_last_refine_stats(self.h, ptr(hist), ctypes.byref(fb)))
        return hist, fb.value

    def info(self, mode):
        vals = [ctypes.c_int32() for _ in range(5)]
        check(lib().krets_circuit_info(self.h, mode, *[ctypes.byref(v) for v in vals]))
        return dict(zip(["n", "nnz_a", "nnz_lu", "n_levels", "n_ulevels"], [v.value for v in vals]))

    def last_launch(self):
        """Last double-float batched launch: threads per instance, instances per CTA, grid,
        how the group size was chosen ("default" / "autotuner" / "autotuner cache"), and
        where the factors were kept."""
        info = np.zeros(5, dtype=np.int32)
        check(lib().krets_last_launch(self.h, ptr(info), 5), "last_launch")
        how = {0: "default", 1: "autotuner", 2: "autotuner cache"}.get(int(info[3]), "?")
        return {"threads_per_instance": int(info[0]), "instances_per_cta": int(info[1]), "grid": int(info[2]),
                "group_size_from": how, "factors": "global memory" if info[4] else "shared memory"}

    def flush_l2(self):
        check(lib().krets_flush_l2(self.h))


def launch_count() -> int:
    return int(lib().krets_launch_count())


def symbolic_export(table, n, mode, method="be", h=1e-9, freq=1e3, ordering=-1):
    """Host symbolic pass arrays (no GPU needed): dict name -> int64 array."""
    t = np.ascontiguousarray(table, dtype=ELEM_DTYPE)
    out = {}
    m = METHOD[method] if isinstance(method, str) else method
    for which, name in enumerate(PROG_ARRAYS):
        ln = ctypes.c_int64(0)
        check(lib().krets_symbolic_export(ptr(t), len(t), n, mode, m, h, freq, ordering, which, None, 0,
                                          ctypes.byref(ln)), "symbolic_export")
        arr = np.zeros(max(ln.value, 1), dtype=np.int64)
        check(lib().krets_symbolic_export(ptr(t), len(t), n, mode, m, h, freq, ordering, which, ptr(arr),
                                          ln.value, ctypes.byref(ln)), "symbolic_export")
        out[name] = arr[:ln.value]
    return out
