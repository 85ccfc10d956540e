"""ctypes mirror of the plain-C structs in include/structured_gb300.h.

Shared by the library binding (structured_gb300.solver) and the test-side
checkers: a struct layout is plumbing, not computation."""
from __future__ import annotations

import ctypes

from . import case as _case

ST_OK = 0
ERRORS = {-1: "bad argument", -2: "CUDA failure", -3: "non-finite result",
          -4: "no convergence", -5: "device wait timed out", -6: "unsupported option"}

BC_TYPES = {"freestream": 0, "slipwall": 1, "wall": 2, "outflow": 3, "periodic": 4,
            "isothermalwall": 5, "wake": 6}
FACES = {"bottom": 0, "right": 1, "top": 2, "left": 3}
VISC = {"power": 0, "sutherland": 1}
TURB = {"none": 0, "sa": 1}
FLUX = {"roe": 0, "ausm": 1}


class StBc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("face", ctypes.c_int32), ("start", ctypes.c_int32),
                ("end", ctypes.c_int32), ("u", ctypes.c_double), ("v", ctypes.c_double),
                ("T", ctypes.c_double)]


class StCase(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int32), ("nj", ctypes.c_int32), ("order", ctypes.c_int32),
                ("lhs_order", ctypes.c_int32), ("viscosity_law", ctypes.c_int32),
                ("turbulence", ctypes.c_int32), ("nbc", ctypes.c_int32),
                ("plate_vertex", ctypes.c_int32), ("flux", ctypes.c_int32),
                ("rho_inf", ctypes.c_double), ("u_inf", ctypes.c_double), ("v_inf", ctypes.c_double),
                ("p_inf", ctypes.c_double), ("T_inf", ctypes.c_double), ("mu_inf", ctypes.c_double),
                ("pr_inf", ctypes.c_double), ("dpdx", ctypes.c_double), ("dpdy", ctypes.c_double),
                ("nu_tilde_inf", ctypes.c_double), ("plate_x_end", ctypes.c_double),
                ("bcs", ctypes.POINTER(StBc))]


class StSolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("residual0", ctypes.c_double), ("residual", ctypes.c_double)]


def make_case_struct(c: "_case.Case"):
    """Returns (StCase, keepalive) for a structured_gb300.case.Case."""
    bcs = (StBc * max(1, len(c.boundaries)))()
    for n, b in enumerate(c.boundaries):
        if b.type not in BC_TYPES:
            raise ValueError("unknown boundary type %r" % b.type)
        if b.face not in FACES:
            raise ValueError("unknown boundary face %r" % b.face)
        bcs[n] = StBc(BC_TYPES[b.type], FACES[b.face], b.start, b.end, b.u, b.v, b.T)
    s = StCase()
    s.ni, s.nj = c.ni, c.nj
    s.order = c.order
    s.lhs_order = c.lhs_order if c.lhs_order is not None else c.order
    s.viscosity_law = VISC[c.viscosity_law]
    s.turbulence = TURB[c.turbulence]
    if c.flux not in FLUX:
        raise ValueError("flux %r: roe or ausm" % c.flux)
    s.flux = FLUX[c.flux]
    s.nbc = len(c.boundaries)
    s.plate_vertex = c.i_le
    s.rho_inf, s.u_inf, s.v_inf = c.rho_inf, c.u_inf, c.v_inf
    s.p_inf, s.T_inf, s.mu_inf, s.pr_inf = c.p_inf, c.T_inf, c.mu_inf, c.pr_inf
    s.dpdx, s.dpdy = c.dpdx, c.dpdy
    s.nu_tilde_inf = c.nu_tilde_inf_ratio * c.mu_inf / c.rho_inf
    s.plate_x_end = c.plate_x_end
    s.bcs = ctypes.cast(bcs, ctypes.POINTER(StBc))
    return s, bcs


class StSolveParams(ctypes.Structure):
    _fields_ = [("max_steps", ctypes.c_int32), ("krylov_m", ctypes.c_int32), ("krylov_maxit", ctypes.c_int32),
                ("cfl_ramp", ctypes.c_int32), ("cfl_ramp_iteration", ctypes.c_int32),
                ("under_relaxation_ramp", ctypes.c_int32), ("under_relaxation_ramp_iteration", ctypes.c_int32),
                ("max_failures", ctypes.c_int32), ("min_steps", ctypes.c_int32),
                ("cfl", ctypes.c_double), ("cfl_max", ctypes.c_double), ("cfl_ramp_exponent", ctypes.c_double),
                ("under_relaxation", ctypes.c_double), ("under_relaxation_ramp_exponent", ctypes.c_double),
                ("tolerance", ctypes.c_double), ("rel_tolerance", ctypes.c_double), ("krylov_rtol", ctypes.c_double),
                ("ser_exponent", ctypes.c_double), ("divergence_factor", ctypes.c_double),
                ("cfl_growth", ctypes.c_double), ("reject_factor", ctypes.c_double),
                ("max_rel_drho", ctypes.c_double), ("nut_floor", ctypes.c_double), ("cfl_min", ctypes.c_double)]
