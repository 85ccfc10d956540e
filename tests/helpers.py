"""Shared test helpers: golden fixtures and the per-cell parity metric."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

from structured_gb300 import case as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """Residual fixtures (the reference's calc_residual / calc_dt on a seeded
    state); io_*.npz hold output files and steady_*.npz converged states
    instead."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("io_", "steady_")))


def load_golden(name: str):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = C.case_from_dict(json.loads(str(d["case"])))
    return c, {k: d[k] for k in d.files if k != "case"}


def rel_err(a: np.ndarray, b: np.ndarray, scale: np.ndarray) -> float:
    """max over cells and components of |a-b| / (sum of |face fluxes|/V):
    the per-cell relative error of a residual, which is a small difference of
    O(1) face fluxes."""
    return float(np.max(np.abs(a - b) / (scale + 1e-300)))


def flat_plate(tmp, name, ni, nj, **kw):
    args = dict(mach=0.3, reynolds=1e6, h1=1e-4, ratio=1.08)
    args.update(kw)
    return C.flat_plate_case(str(tmp), name, ni, nj, **args)


def negative_nut_state(c, seed):
    """perturbed_state with rho nu_tilde negative (-0.5..-12 x freestream, chi
    down to about -36, across fv1's pole at chi = -c_v1) in a patch touching
    the wall: exercises the SA-neg branches of mu_t, the diffusion coefficient
    and the source."""
    q = C.perturbed_state(c, seed)
    rng = np.random.default_rng(seed + 1)
    i0, i1, j1 = c.nic // 3, c.nic // 2 + 2, max(3, c.njc // 3)
    patch = q[i0:i1, :j1, 4]
    q[i0:i1, :j1, 4] = -np.abs(patch) * rng.uniform(0.5, 12.0, patch.shape)
    return q
