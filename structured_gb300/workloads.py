"""The flat-plate workloads of the residual / adjoint path as cases.

  laminar_plate     129x65, M=0.2, Re_L=1e5, Sutherland, Pr=0.72: implicit
                    pseudo-time to steady state (plain method).
  throughput_plate  513x257 / 2049x1025 / 4097x2049, M=0.3, Re=1e6, SA,
                    seeded 1 % perturbations: residual / adjoint throughput.
  turbulent_plate   545x385, first cell 1e-7 at ratio 1.05, M=0.2, Re_L=5e6,
                    SA with beta = 1; objective J = drag on x in [0, 1].
  inversion_cases   the turbulent plate at Re_L in {1e6, 3e6, 1e7} with the top
                    boundary inclined at {0, +2, -2} degrees.
  target_beta       1 + 0.3 * (sum of 8 seeded 2D Gaussians), widths 0.05-0.2
                    in x and 0.002-0.02 in y.
"""
from __future__ import annotations

import numpy as np

from . import case as C


def laminar_plate(workdir: str, ni: int = 129, nj: int = 65, write_files: bool = True) -> C.Case:
    return C.flat_plate_case(workdir, "laminar_plate_%dx%d" % (ni, nj), ni, nj, 0.2, 1e5, 1e-4, 1.08, pr=0.72,
                             viscosity_law="sutherland", write_files=write_files, order=2, lhs_order=2)


def throughput_plate(workdir: str, grid: str = "4097x2049", write_files: bool = False) -> C.Case:
    ni, nj = (int(v) for v in grid.split("x"))
    return C.flat_plate_case(workdir, "throughput_%s" % grid, ni, nj, 0.3, 1e6, 1e-4, 1.08, turbulence="sa",
                             write_files=write_files)


def turbulent_plate(workdir: str, ni: int = 545, nj: int = 385, reynolds: float = 5e6, top_angle_deg: float = 0.0,
                    h1: float = 1e-7, ratio: float = 1.05, write_files: bool = True) -> C.Case:
    name = "turbulent_plate_%dx%d_Re%.0e_a%+.0f" % (ni, nj, reynolds, top_angle_deg)
    return C.flat_plate_case(workdir, name, ni, nj, 0.2, reynolds, h1, ratio, turbulence="sa", pr=0.72,
                             viscosity_law="sutherland", top_angle_deg=top_angle_deg, write_files=write_files,
                             order=2, lhs_order=2)


def inversion_cases(workdir: str, ni: int = 545, nj: int = 385, write_files: bool = True):
    out = []
    for re_l in (1e6, 3e6, 1e7):
        for ang in (0.0, 2.0, -2.0):
            out.append(((re_l, ang), turbulent_plate(workdir, ni, nj, re_l, ang, write_files=write_files)))
    return out


def cell_centres(xv: np.ndarray, yv: np.ndarray):
    xc = 0.25 * (xv[:-1, :-1] + xv[1:, :-1] + xv[:-1, 1:] + xv[1:, 1:])
    yc = 0.25 * (yv[:-1, :-1] + yv[1:, :-1] + yv[:-1, 1:] + yv[1:, 1:])
    return xc, yc


def target_beta(xv: np.ndarray, yv: np.ndarray, seed: int = 20261203, n: int = 8) -> np.ndarray:
    """1 + 0.3 * sum of n Gaussians with centres on the plate's boundary layer
    (x in [0.05, 0.95], y in [0, 0.02]) and widths 0.05-0.2 (x), 0.002-0.02 (y)."""
    rng = np.random.default_rng(seed)
    xc, yc = cell_centres(xv, yv)
    b = np.zeros_like(xc)
    for _ in range(n):
        x0, y0 = rng.uniform(0.05, 0.95), rng.uniform(0.0, 0.02)
        sx, sy = rng.uniform(0.05, 0.2), rng.uniform(0.002, 0.02)
        amp = rng.uniform(-1.0, 1.0)
        b += amp * np.exp(-0.5 * (((xc - x0) / sx) ** 2 + ((yc - y0) / sy) ** 2))
    return 1.0 + 0.3 * b
