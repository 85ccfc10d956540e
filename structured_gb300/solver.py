"""Host-side mirror of the reference's residual / solver interface over the C ABI.

``EulerEquation`` mirrors src/model/eulerequation.h:16-64 (calc_residual,
calc_dt) for one grid block; the state lives on the GPU in the reference's
q[i][j][k] layout.  Every call goes through libstructured_gb300.so: there is no
CPU fallback, and a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import abi
from . import case as C

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstructured_gb300.so")
_P = ctypes.POINTER(ctypes.c_double)
_lib = None


class StructuredError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%s)" % (msg, abi.ERRORS.get(code, str(code))))
        self.code = code


def _ptr(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(_P)


def _vp(x):
    return ctypes.c_void_p(int(x)) if x is not None else None


def _f32p(a):
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous float32")
    return ctypes.c_void_p(a.ctypes.data)


def load_library() -> ctypes.CDLL:
    """Loads the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError("%s is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`"
                                % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "st_last_error": (ctypes.c_char_p, []),
        "st_version": (I, []),
        "st_create": (I, [ctypes.POINTER(abi.StCase), _P, _P, I, ctypes.POINTER(V)]),
        "st_destroy": (I, [V]),
        "st_dims": (I, [V, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]),
        "st_set_state": (I, [V, _P]),
        "st_get_state": (I, [V, _P]),
        "st_set_beta": (I, [V, _P]),
        "st_get_wall_distance": (I, [V, _P]),
        "st_residual": (I, [V, I, _P]),
        "st_residual_device": (I, [V, V, V, V, I]),
        "st_dt": (I, [V, D, _P]),
        "st_norms": (I, [V, _P]),
        "st_skin_friction": (I, [V, _P, ctypes.POINTER(D)]),
        "st_skin_friction_device": (I, [V, V, V]),
        "st_jvp_device": (I, [V, V, V, V, I]),
        "st_vjp_device": (I, [V, V, V, V, I]),
        "st_vjp": (I, [V, _P, _P, _P, I]),
        "st_residual_vjp_device": (I, [V, V, V, V, V, I]),
        "st_residual_vjp": (I, [V, _P, _P, _P, _P, I]),
        "st_fused_launch_count": (I, [V, I]),
        "st_probe_fp64": (I, [V, ctypes.POINTER(D)]),
        "st_set_residual_path": (I, [V, I, ctypes.POINTER(I)]),
        "st_probe_nr_math": (I, [V, ctypes.c_longlong, V]),
        "st_last_kernel_ms": (I, [V, ctypes.POINTER(D), ctypes.POINTER(D)]),
        "st_profile_pipeline": (I, [V, I, I, _P, I, ctypes.c_char_p, I, ctypes.POINTER(I)]),
        "st_launch_counts": (I, [V, I, ctypes.POINTER(I), ctypes.POINTER(I)]),
        "st_device_state": (I, [V, ctypes.POINTER(V), ctypes.POINTER(V), ctypes.POINTER(V)]),
        "st_jacobian_assemble": (I, [V, I]),
        "st_jacobian_blocks": (I, [V, _P]),
        "st_jacobian_apply_device": (I, [V, V, V, I]),
        "st_linear_solve_device": (I, [V, D, V, V, I, I, I, D, ctypes.POINTER(abi.StSolveStats)]),
        "st_solve": (I, [V, ctypes.POINTER(abi.StSolveParams), ctypes.POINTER(abi.StSolveStats), _P, I,
                         ctypes.POINTER(I)]),
        "st_cf_gradient_device": (I, [V, _P, V]),
        "st_adjoint_solve_device": (I, [V, V, V, D, I, I, D, ctypes.POINTER(abi.StSolveStats)]),
        "st_tangent_solve_device": (I, [V, V, V, D, I, I, D, ctypes.POINTER(abi.StSolveStats)]),
        "st_explicit_solve": (I, [V, I, D, I, D, I, V, I, ctypes.POINTER(I)]),
        "st_wall_gradients": (I, [V, V]),
        "st_mlp_param_count": (I, []),
        "st_mlp_init": (I, [V, ctypes.c_ulonglong]),
        "st_mlp_set_params": (I, [V, V]),
        "st_mlp_get_params": (I, [V, V]),
        "st_mlp_set_normalization": (I, [V, V, V]),
        "st_mlp_enable": (I, [V, I]),
        "st_mlp_train": (I, [V, V, V, ctypes.c_long, I, I, ctypes.c_float, ctypes.c_ulonglong, V]),
        "st_mlp_grad": (I, [V, V, V, ctypes.c_long, I, ctypes.c_ulonglong, I, V, V]),
        "st_sa_features": (I, [V, V]),
        "st_mlp_beta": (I, [V, V]),
        "st_precond_info": (I, [V, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(D)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int, what: str) -> None:
    if rc != abi.ST_OK:
        msg = load_library().st_last_error().decode(errors="replace")
        raise StructuredError(rc, "%s: %s" % (what, msg))


class EulerEquation:
    """One grid block on one GPU (reference: Mesh::setup + EulerEquation,
    src/utils/mesh.cpp:392-414, src/model/eulerequation.h:16-64)."""

    def __init__(self, case: C.Case, xv: np.ndarray | None = None, yv: np.ndarray | None = None,
                 device: int = -1):
        self.lib = load_library()
        if xv is None:
            xv, yv = C.load_grid(case)
        self.case = case
        self._xv = np.ascontiguousarray(xv, dtype=np.float64)
        self._yv = np.ascontiguousarray(yv, dtype=np.float64)
        if self._xv.shape != (case.ni, case.nj):
            raise ValueError("grid shape %s does not match ni, nj = %d, %d" % (self._xv.shape, case.ni, case.nj))
        self._st, self._keep = abi.make_case_struct(case)
        h = ctypes.c_void_p()
        _check(self.lib.st_create(ctypes.byref(self._st), _ptr(self._xv), _ptr(self._yv), device, ctypes.byref(h)),
               "st_create")
        self.h = h
        nic, njc, nq = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.st_dims(self.h, ctypes.byref(nic), ctypes.byref(njc), ctypes.byref(nq))
        self.nic, self.njc, self.nq = nic.value, njc.value, nq.value
        self.shape = (self.nic, self.njc, self.nq)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.st_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state --------------------------------------------------------------
    def set_state(self, q: np.ndarray) -> None:
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.shape != self.shape:
            raise ValueError("state shape %s != %s" % (q.shape, self.shape))
        _check(self.lib.st_set_state(self.h, _ptr(q)), "st_set_state")

    def get_state(self) -> np.ndarray:
        q = np.empty(self.shape)
        _check(self.lib.st_get_state(self.h, _ptr(q)), "st_get_state")
        return q

    def set_beta(self, beta: np.ndarray) -> None:
        b = np.ascontiguousarray(beta, dtype=np.float64)
        if b.shape != (self.nic, self.njc):
            raise ValueError("beta shape")
        _check(self.lib.st_set_beta(self.h, _ptr(b)), "st_set_beta")

    def wall_distance(self) -> np.ndarray:
        d = np.empty((self.nic, self.njc))
        _check(self.lib.st_get_wall_distance(self.h, _ptr(d)), "st_get_wall_distance")
        return d

    # -- reference interface -------------------------------------------------
    def calc_residual(self, q: np.ndarray | None = None, lhs: bool = False) -> np.ndarray:
        """EulerEquation::calc_residual (src/model/eulerequation.cpp:202-232)."""
        if q is not None:
            self.set_state(q)
        rhs = np.empty(self.shape)
        _check(self.lib.st_residual(self.h, int(lhs), _ptr(rhs)), "st_residual")
        return rhs

    def calc_dt(self, cfl: float) -> np.ndarray:
        """EulerEquation::calc_dt (src/model/eulerequation.cpp:237-259)."""
        dt = np.empty(self.shape)
        _check(self.lib.st_dt(self.h, float(cfl), _ptr(dt)), "st_dt")
        return dt

    def norms(self) -> np.ndarray:
        out = np.empty(self.nq)
        _check(self.lib.st_norms(self.h, _ptr(out)), "st_norms")
        return out

    def skin_friction(self):
        cf = np.empty(self.nic)
        J = ctypes.c_double()
        _check(self.lib.st_skin_friction(self.h, _ptr(cf), ctypes.byref(J)), "st_skin_friction")
        return cf, J.value

    # -- device-pointer entry points (torch tensors or raw CUDA pointers) -----
    def residual_device(self, q_ptr: int, rhs_ptr: int, beta_ptr: int | None = None, lhs: bool = False) -> None:
        _check(self.lib.st_residual_device(self.h, _vp(q_ptr), _vp(beta_ptr), _vp(rhs_ptr), int(lhs)),
               "st_residual_device")

    def jvp_device(self, v_ptr: int, jv_ptr: int, vb_ptr: int | None = None, lhs: bool = False) -> None:
        _check(self.lib.st_jvp_device(self.h, _vp(v_ptr), _vp(vb_ptr), _vp(jv_ptr), int(lhs)), "st_jvp_device")

    def vjp_device(self, psi_ptr: int, outq_ptr: int | None, outb_ptr: int | None, lhs: bool = False) -> None:
        _check(self.lib.st_vjp_device(self.h, _vp(psi_ptr), _vp(outq_ptr), _vp(outb_ptr), int(lhs)), "st_vjp_device")

    def vjp(self, psi: np.ndarray, lhs: bool = False):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        oq = np.empty(self.shape)
        ob = np.empty((self.nic, self.njc))
        _check(self.lib.st_vjp(self.h, _ptr(psi), _ptr(oq), _ptr(ob), int(lhs)), "st_vjp")
        return oq, ob

    def residual_vjp_device(self, psi_ptr: int, rhs_ptr: int, outq_ptr: int | None, outb_ptr: int | None,
                            lhs: bool = False) -> None:
        """Residual and adjoint of the context state in one sweep."""
        _check(self.lib.st_residual_vjp_device(self.h, _vp(psi_ptr), _vp(rhs_ptr), _vp(outq_ptr), _vp(outb_ptr),
                                               int(lhs)), "st_residual_vjp_device")

    def residual_vjp(self, psi: np.ndarray, lhs: bool = False):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        rhs = np.empty(self.shape)
        oq = np.empty(self.shape)
        ob = np.empty((self.nic, self.njc))
        _check(self.lib.st_residual_vjp(self.h, _ptr(psi), _ptr(rhs), _ptr(oq), _ptr(ob), int(lhs)), "st_residual_vjp")
        return rhs, oq, ob

    def fused_launch_count(self, lhs: bool = False) -> int:
        n = self.lib.st_fused_launch_count(self.h, int(lhs))
        if n < 0:
            _check(n, "st_fused_launch_count")
        return n

    def device_state(self):
        q, r, s = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(self.lib.st_device_state(self.h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(s)), "st_device_state")
        return q.value, r.value, s.value

    def set_residual_path(self, tiled: bool) -> bool:
        """Selects the tiled (TMA-staged) sweeps or the per-stage passes for
        the FP64 residual; returns whether the tiled sweeps now run."""
        act = ctypes.c_int()
        _check(self.lib.st_set_residual_path(self.h, int(tiled), ctypes.byref(act)), "st_set_residual_path")
        return bool(act.value)

    def probe_fp64_tflops(self) -> float:
        t = ctypes.c_double()
        _check(self.lib.st_probe_fp64(self.h, ctypes.byref(t)), "st_probe_fp64")
        return t.value

    def profile(self, which: str = "residual", lhs: bool = False) -> dict:
        """Per-launch device times (ms) of one residual or adjoint evaluation."""
        ms = np.zeros(32)
        buf = ctypes.create_string_buffer(1024)
        n = ctypes.c_int()
        code = {"residual": 0, "adjoint": 1, "fused": 2}[which]
        _check(self.lib.st_profile_pipeline(self.h, code, int(lhs), _ptr(ms), 32, buf,
                                            1024, ctypes.byref(n)), "st_profile_pipeline")
        names = buf.value.decode().split(",")
        out = {}
        for k, v in zip(names, ms[:n.value]):
            out[k] = out.get(k, 0.0) + float(v)
        return out

    def launch_counts(self, lhs: bool = False):
        r, v = ctypes.c_int(), ctypes.c_int()
        _check(self.lib.st_launch_counts(self.h, int(lhs), ctypes.byref(r), ctypes.byref(v)), "st_launch_counts")
        return r.value, v.value

    def last_kernel_ms(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(self.lib.st_last_kernel_ms(self.h, ctypes.byref(a), ctypes.byref(b)), "st_last_kernel_ms")
        return a.value, b.value


def solve_params(case: C.Case | None = None, **over) -> abi.StSolveParams:
    """Pseudo-time Newton parameters from a case's [solver] keys
    (src/utils/config.cpp:42-56) with keyword overrides."""
    p = abi.StSolveParams()
    p.max_steps = case.iteration_max if case else 100
    p.krylov_m, p.krylov_maxit, p.krylov_rtol = 40, 120, 1e-3
    p.cfl = case.cfl if case else 10.0
    p.cfl_max = 1e12
    p.cfl_ramp = int(case.cfl_ramp) if case else 1
    p.cfl_ramp_iteration = case.cfl_ramp_iteration if case else 5
    p.cfl_ramp_exponent = case.cfl_ramp_exponent if case else 1.2
    p.under_relaxation = case.under_relaxation if case else 1.0
    p.under_relaxation_ramp = int(case.under_relaxation_ramp) if case else 0
    p.under_relaxation_ramp_iteration = case.under_relaxation_ramp_iteration if case else 20
    p.under_relaxation_ramp_exponent = case.under_relaxation_ramp_exponent if case else 1.1
    # the reference's default tolerance (1e10, config.cpp:52) never mattered:
    # its tolerance exit is disabled (solver.cpp:145); treat it as unset
    p.tolerance = case.tolerance if (case and case.tolerance < 1e9) else 0.0
    p.rel_tolerance = 0.0
    p.ser_exponent = 0.0
    p.divergence_factor = 1e4
    p.max_failures = 20
    p.min_steps = 0
    p.cfl_growth = 0.0
    p.reject_factor = 3.0
    p.max_rel_drho = 0.3
    p.nut_floor = 0.0
    p.cfl_min = 0.1
    for k, v in over.items():
        setattr(p, k, v)
    return p


class Solver:
    """Pseudo-time Newton driver on the GPU (reference: Solver::solve,
    src/solver/solver.cpp:198-236, implicit path of Solver::step :53-196)."""

    def __init__(self, eq: EulerEquation, **params):
        self.eq = eq
        self.params = solve_params(eq.case, **params)

    def solve(self, raise_on_noconv: bool = True):
        eq = self.eq
        nq = eq.nq
        stride = 3 + nq
        hist = np.zeros(stride * (self.params.max_steps + 2))
        st = abi.StSolveStats()
        steps = ctypes.c_int()
        rc = eq.lib.st_solve(eq.h, ctypes.byref(self.params), ctypes.byref(st), _ptr(hist), hist.size,
                             ctypes.byref(steps))
        rows = []
        for k in range(0, hist.size, stride):
            if k > 0 and hist[k] == 0 and hist[k + 1] == 0:
                break
            rows.append(hist[k:k + stride].copy())
        history = np.array(rows)
        if rc != abi.ST_OK and (raise_on_noconv or rc != -4):
            _check(rc, "st_solve")
        return rc == abi.ST_OK, history


def _eq_extras():
    def jacobian_assemble(self, lhs: bool = False):
        _check(self.lib.st_jacobian_assemble(self.h, int(lhs)), "st_jacobian_assemble")

    def jacobian_blocks(self):
        b = np.empty((self.nic, self.njc, 13, self.nq, self.nq))
        _check(self.lib.st_jacobian_blocks(self.h, _ptr(b)), "st_jacobian_blocks")
        return b

    def jacobian_apply_device(self, v_ptr, out_ptr, transpose=False):
        _check(self.lib.st_jacobian_apply_device(self.h, _vp(v_ptr), _vp(out_ptr), int(transpose)),
               "st_jacobian_apply_device")

    def linear_solve_device(self, cfl, b_ptr, x_ptr, transpose=False, m=40, maxit=200, rtol=1e-8):
        st = abi.StSolveStats()
        _check(self.lib.st_linear_solve_device(self.h, float(cfl), _vp(b_ptr), _vp(x_ptr), int(transpose), m, maxit,
                                               float(rtol), ctypes.byref(st)), "st_linear_solve_device")
        return st

    def cf_gradient_device(self, w: np.ndarray, grad_ptr):
        w = np.ascontiguousarray(w, dtype=np.float64)
        _check(self.lib.st_cf_gradient_device(self.h, _ptr(w), _vp(grad_ptr)), "st_cf_gradient_device")

    def adjoint_solve_device(self, b_ptr, psi_ptr, cfl_prec=1e6, m=150, maxit=4000, rtol=1e-10):
        st = abi.StSolveStats()
        _check(self.lib.st_adjoint_solve_device(self.h, _vp(b_ptr), _vp(psi_ptr), float(cfl_prec), m, maxit,
                                                float(rtol), ctypes.byref(st)), "st_adjoint_solve_device")
        return st

    def tangent_solve_device(self, b_ptr, dq_ptr, cfl_prec=1e6, m=150, maxit=4000, rtol=1e-10):
        st = abi.StSolveStats()
        _check(self.lib.st_tangent_solve_device(self.h, _vp(b_ptr), _vp(dq_ptr), float(cfl_prec), m, maxit,
                                                float(rtol), ctypes.byref(st)), "st_tangent_solve_device")
        return st

    def explicit_solve(self, scheme: str = "rk4_jameson", cfl: float | None = None, steps: int = 1000,
                       tolerance: float = 0.0, check_every: int = 100, raise_on_noconv: bool = True):
        """Explicit marching (Solver::step's forward_euler / rk4_jameson);
        returns (steps done, history rows [step, norms...])."""
        code = {"forward_euler": 0, "rk4_jameson": 1}[scheme]
        cfl = self.case.cfl if cfl is None else cfl
        hist = np.zeros((steps // check_every + 2) * (1 + self.nq))
        done = ctypes.c_int()
        rc = self.lib.st_explicit_solve(self.h, code, float(cfl), int(steps), float(tolerance), int(check_every),
                                        _ptr(hist), hist.size, ctypes.byref(done))
        if rc and not (rc == -4 and not raise_on_noconv):
            _check(rc, "st_explicit_solve")
        rows = hist.reshape(-1, 1 + self.nq)
        return done.value, rows[rows[:, 0] > 0]

    def precond_info(self) -> dict:
        """Wake strip level of the implicit solve's preconditioner: its size,
        whether the last factorisation built it, how often, host ms of the last."""
        n, act, cnt, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(self.lib.st_precond_info(self.h, ctypes.byref(n), ctypes.byref(act), ctypes.byref(cnt),
                                        ctypes.byref(ms)), "st_precond_info")
        return {"strip_unknowns": n.value, "strip_active": bool(act.value), "strip_factorisations": cnt.value,
                "strip_host_ms": ms.value}

    def wall_gradients(self) -> np.ndarray:
        """(u_x, u_y, v_x, v_y) at the j = 0 faces of the current state, [nic][4]."""
        out = np.empty((self.nic, 4))
        _check(self.lib.st_wall_gradients(self.h, _ptr(out)), "st_wall_gradients")
        return out

    # -- learned SA correction (st_mlp_*) --------------------------------
    def mlp_init(self, seed: int) -> None:
        _check(self.lib.st_mlp_init(self.h, int(seed)), "st_mlp_init")

    def mlp_params(self) -> np.ndarray:
        out = np.empty(self.lib.st_mlp_param_count(), dtype=np.float32)
        _check(self.lib.st_mlp_get_params(self.h, _f32p(out)), "st_mlp_get_params")
        return out

    def mlp_set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.lib.st_mlp_param_count():
            raise ValueError("MLP parameter count")
        _check(self.lib.st_mlp_set_params(self.h, _f32p(p)), "st_mlp_set_params")

    def mlp_set_normalization(self, mean, std) -> None:
        m = np.ascontiguousarray(mean, dtype=np.float32)
        sd = np.ascontiguousarray(std, dtype=np.float32)
        _check(self.lib.st_mlp_set_normalization(self.h, _f32p(m), _f32p(sd)), "st_mlp_set_normalization")

    def mlp_enable(self, on: bool = True) -> None:
        _check(self.lib.st_mlp_enable(self.h, int(on)), "st_mlp_enable")

    def mlp_train(self, feat_ptr, target_ptr, n: int, steps: int, batch: int = 65536, lr: float = 1e-3,
                  seed: int = 0) -> np.ndarray:
        loss = np.zeros(steps, dtype=np.float32)
        _check(self.lib.st_mlp_train(self.h, _vp(feat_ptr), _vp(target_ptr), int(n), int(steps), int(batch),
                                     float(lr), int(seed), _f32p(loss)), "st_mlp_train")
        return loss

    def mlp_grad(self, feat_ptr, target_ptr, n: int, batch: int, seed: int, step: int = 0):
        """Gradient (FP32 master layout) and loss of the batch st_mlp_train
        draws at `step`, without an update."""
        g = np.zeros(self.lib.st_mlp_param_count(), dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(self.lib.st_mlp_grad(self.h, _vp(feat_ptr), _vp(target_ptr), int(n), int(batch), int(seed), int(step),
                                    _f32p(g), _f32p(loss)), "st_mlp_grad")
        return g, float(loss[0])

    def sa_features_device(self, out_ptr) -> None:
        _check(self.lib.st_sa_features(self.h, _vp(out_ptr)), "st_sa_features")

    def mlp_beta_device(self, out_ptr) -> None:
        _check(self.lib.st_mlp_beta(self.h, _vp(out_ptr)), "st_mlp_beta")

    for f in (jacobian_assemble, jacobian_blocks, jacobian_apply_device, linear_solve_device, cf_gradient_device,
              adjoint_solve_device, tangent_solve_device, explicit_solve, precond_info, wall_gradients, mlp_init, mlp_params, mlp_set_params,
              mlp_set_normalization, mlp_enable, mlp_train, mlp_grad, sa_features_device, mlp_beta_device):
        setattr(EulerEquation, f.__name__, f)


_eq_extras()
