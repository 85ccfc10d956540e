"""Test infrastructure: ctypes access to the FP64 CPU restatement
(oracle/port/port.cpp, built by ``make -C oracle port``).  Checker only."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from structured_gb300 import abi, case as C

HERE = os.path.dirname(os.path.abspath(__file__))
_P = ctypes.POINTER(ctypes.c_double)
_lib = None


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def load():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_ref", "libport.so")
        if not os.path.exists(path):
            raise FileNotFoundError("%s missing: run `make -C oracle port`" % path)
        lib = ctypes.CDLL(path)
        lib.port_create.restype = ctypes.c_void_p
        lib.port_create.argtypes = [ctypes.POINTER(abi.StCase), _P, _P]
        lib.port_destroy.argtypes = [ctypes.c_void_p]
        lib.port_set_threads.argtypes = [ctypes.c_int]
        lib.port_set_threads.restype = ctypes.c_int
        lib.port_metrics.argtypes = [ctypes.c_void_p, _P, _P, _P, _P]
        lib.port_residual.argtypes = [ctypes.c_void_p, _P, _P, _P, ctypes.c_int]
        lib.port_flux_scale.argtypes = [ctypes.c_void_p, _P, _P, _P, ctypes.c_int]
        lib.port_skin_friction.argtypes = [ctypes.c_void_p, _P, _P, _P]
        lib.port_dt.argtypes = [ctypes.c_void_p, _P, ctypes.c_double, _P]
        lib.port_jvp.argtypes = [ctypes.c_void_p, _P, _P, _P, _P, _P, ctypes.c_int]
        lib.port_vjp.argtypes = [ctypes.c_void_p, _P, _P, _P, _P, _P, ctypes.c_int]
        lib.port_objective_grad.argtypes = [ctypes.c_void_p, _P, _P]
        lib.port_set_freeze_nonlocal.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib = lib
    return _lib


class PortCase:
    def __init__(self, c: C.Case, xv=None, yv=None):
        self.lib = load()
        if xv is None:
            xv, yv = C.load_grid(c)
        self.case = c
        self.xv = np.ascontiguousarray(xv, dtype=np.float64)
        self.yv = np.ascontiguousarray(yv, dtype=np.float64)
        self.st, self._keep = abi.make_case_struct(c)
        self.h = self.lib.port_create(ctypes.byref(self.st), _ptr(self.xv), _ptr(self.yv))
        self.ni, self.nj, self.nq = c.ni, c.nj, c.nq
        self.nic, self.njc = c.ni - 1, c.nj - 1

    def __del__(self):
        try:
            if self.h:
                self.lib.port_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_threads(self, n: int) -> int:
        return self.lib.port_set_threads(n)

    def _order(self, lhs):
        return self.case.lhs_order if (lhs and self.case.lhs_order) else self.case.order

    def metrics(self):
        nchi = np.empty((self.ni, self.njc, 2)); neta = np.empty((self.nic, self.nj, 2))
        vol = np.empty((self.nic, self.njc)); wd = np.empty((self.nic, self.njc))
        self.lib.port_metrics(self.h, _ptr(nchi), _ptr(neta), _ptr(vol), _ptr(wd))
        return nchi, neta, vol, wd

    def residual(self, q, beta=None, lhs=False):
        q = np.ascontiguousarray(q, dtype=np.float64)
        rhs = np.empty_like(q)
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        self.lib.port_residual(self.h, _ptr(q), _ptr(b), _ptr(rhs), self._order(lhs))
        return rhs

    def flux_scale(self, q, beta=None, lhs=False):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty_like(q)
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        self.lib.port_flux_scale(self.h, _ptr(q), _ptr(b), _ptr(out), self._order(lhs))
        return out

    def skin_friction(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        cf = np.empty(self.nic)
        J = ctypes.c_double()
        self.lib.port_skin_friction(self.h, _ptr(q), _ptr(cf), ctypes.byref(J))
        return cf, J.value

    def dt(self, q, cfl):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty_like(q)
        self.lib.port_dt(self.h, _ptr(q), cfl, _ptr(out))
        return out

    def jvp(self, q, v, beta=None, vb=None, lhs=False):
        q = np.ascontiguousarray(q, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        vb = None if vb is None else np.ascontiguousarray(vb, dtype=np.float64)
        out = np.empty_like(q)
        self.lib.port_jvp(self.h, _ptr(q), _ptr(b), _ptr(v), _ptr(vb), _ptr(out), self._order(lhs))
        return out

    def vjp(self, q, psi, beta=None, lhs=False):
        q = np.ascontiguousarray(q, dtype=np.float64)
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        oq = np.empty_like(q)
        ob = np.zeros((self.nic, self.njc))
        self.lib.port_vjp(self.h, _ptr(q), _ptr(b), _ptr(psi), _ptr(oq), _ptr(ob), self._order(lhs))
        return oq, ob

    def freeze_nonlocal(self, on: bool = True) -> None:
        """JVPs and VJPs with the periodic and wake ghosts' tangents held at
        zero: the Jacobian's local part, without the distant coupling of those
        boundary copies."""
        self.lib.port_set_freeze_nonlocal(self.h, 1 if on else 0)

    def objective_grad(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.empty_like(q)
        self.lib.port_objective_grad(self.h, _ptr(q), _ptr(out))
        return out
