"""Test infrastructure: ctypes access to the reference solver's own residual
code, compiled out of tree by oracle/Makefile into oracle/_ref/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.  See oracle/ref_harness.cpp for the entry
points and the reference functions they drive.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_P = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


_libs: dict = {}


def load(kind: str = "serial") -> ctypes.CDLL:
    """kind: 'serial' (the reference's stock single-thread build) or 'omp'."""
    if kind in _libs:
        return _libs[kind]
    path = os.path.join(REF_DIR, "libref_%s.so" % kind)
    if not os.path.exists(path):
        raise FileNotFoundError("%s missing: run `make -C oracle ref`" % path)
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    lib.refh_open.restype = ctypes.c_void_p
    lib.refh_open.argtypes = [ctypes.c_char_p]
    lib.refh_close.argtypes = [ctypes.c_void_p]
    lib.refh_dims.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 3
    lib.refh_set_threads.argtypes = [ctypes.c_int]
    lib.refh_residual.argtypes = [ctypes.c_void_p, _P, _P, ctypes.c_int]
    lib.refh_residual_inplace.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.refh_dt.argtypes = [ctypes.c_void_p, _P, ctypes.c_double, _P]
    lib.refh_metrics.argtypes = [ctypes.c_void_p, _P, _P, _P]
    lib.refh_primitives.argtypes = [ctypes.c_void_p, _P]
    lib.refh_eta_gradients.argtypes = [ctypes.c_void_p, _P]
    lib.refh_write_outputs.argtypes = [ctypes.c_void_p, _P]
    _libs[kind] = lib
    return lib


class RefCase:
    """One reference Config+Mesh+EulerEquation built from an ``.inp`` file.

    The reference reads the grid path relative to the working directory, so
    ``.inp`` files written by structured_gb300.case use absolute paths."""

    def __init__(self, inp_path: str, kind: str = "serial"):
        self.lib = load(kind)
        self.h = self.lib.refh_open(inp_path.encode())
        if not self.h:
            raise RuntimeError("reference setup failed for %s" % inp_path)
        ni, nj, nq = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.refh_dims(self.h, ctypes.byref(ni), ctypes.byref(nj), ctypes.byref(nq))
        self.ni, self.nj, self.nq = ni.value, nj.value, nq.value
        self.nic, self.njc = self.ni - 1, self.nj - 1

    def close(self):
        if self.h:
            self.lib.refh_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int) -> int:
        return self.lib.refh_set_threads(n)

    def residual(self, q: np.ndarray, lhs: bool = False) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64)
        assert q.shape == (self.nic, self.njc, self.nq)
        rhs = np.empty_like(q)
        self.lib.refh_residual(self.h, _ptr(q), _ptr(rhs), int(lhs))
        return rhs

    def residual_inplace(self, lhs: bool = False) -> None:
        self.lib.refh_residual_inplace(self.h, int(lhs))

    def dt(self, q: np.ndarray, cfl: float) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty_like(q)
        self.lib.refh_dt(self.h, _ptr(q), cfl, _ptr(out))
        return out

    def metrics(self):
        nchi = np.empty((self.ni, self.njc, 2))
        neta = np.empty((self.nic, self.nj, 2))
        vol = np.empty((self.nic, self.njc))
        self.lib.refh_metrics(self.h, _ptr(nchi), _ptr(neta), _ptr(vol))
        return nchi, neta, vol

    def primitives(self) -> np.ndarray:
        out = np.empty((5, self.nic + 2, self.njc + 2))
        self.lib.refh_primitives(self.h, _ptr(out))
        return out

    def eta_gradients(self) -> np.ndarray:
        out = np.empty((self.nic, self.nj, 4))
        self.lib.refh_eta_gradients(self.h, _ptr(out))
        return out

    def write_outputs(self, q: np.ndarray) -> None:
        """The reference's IOManager::write of state q (files under the case's io.label)."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        self.lib.refh_write_outputs(self.h, _ptr(q))
