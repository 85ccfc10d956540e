"""End-to-end checks of the implicit solve and the discrete adjoint on the
turbulent flat plate (545x385, first cell 1e-7 at ratio 1.05, M=0.2,
Re_L=5e6, SA with beta = 1, J = drag on the plate):

  python -m structured_gb300.validate gradient [--cells 64] [--out file.json]

1. pseudo-time Newton from freestream to steady state;
2. dJ/dbeta by one adjoint solve;
3. tangent check: dJ/dbeta_c by forward-sensitivity solves on a few cells;
4. central finite differences (step 1e-6) of converged solves on seeded cells
   with |dJ/dbeta_c| >= 1e-3 max, with the round-off floor eps*|J|/(2h*|g_c|)
   of each difference stated.
"""
from __future__ import annotations

import argparse
import json
import sys
import tempfile
import time

import numpy as np


def gradient_check(ncells: int = 64, ni: int = 545, nj: int = 385, h: float = 1e-6, seed: int = 20261203,
                   ntangent: int = 8):
    import torch
    from . import case as C
    from . import inversion as inv
    from . import workloads
    from .solver import EulerEquation, Solver
    out = {}
    tmp = tempfile.mkdtemp()
    c = workloads.turbulent_plate(tmp, ni, nj, write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-7, ratio=1.05)
    xv, yv = g.xv, g.yv
    eq = EulerEquation(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    t0 = time.time()
    ok, hist = inv.converge(eq)
    out["flow_solve"] = {"converged": bool(ok), "steps": int(hist.shape[0] - 1), "wall_s": time.time() - t0,
                         "residual_initial": float(hist[0, 3:].max()), "residual_final": float(hist[-1, 3:].max())}
    if not ok:
        return out
    r0 = float(hist[0, 3:].max())
    q0 = eq.get_state()
    w = inv.plate_weights(c, xv)
    cf, J0 = eq.skin_friction()
    out["J"] = J0
    t0 = time.time()
    grad, st = inv.cf_adjoint_gradient(eq, w, rtol=1e-12)
    out["adjoint"] = {"wall_s": time.time() - t0, "gmres_iterations": int(st.iterations),
                      "converged": int(st.converged), "residual_ratio": st.residual / max(st.residual0, 1e-300)}
    rng = np.random.default_rng(seed)
    # seeded cells among those whose gradient carries signal (>= 1e-3 of the
    # largest: the plate's boundary layer); the rest are below FD resolution
    cand = np.argwhere(np.abs(grad) >= 1e-3 * np.abs(grad).max())
    pick = rng.choice(len(cand), size=min(ncells, len(cand)), replace=False)
    cells = [tuple(int(t) for t in cand[k]) for k in pick]
    # tangent check
    tan = []
    gq = torch.zeros(eq.shape, dtype=torch.float64, device="cuda")
    eq.cf_gradient_device(w, gq.data_ptr())
    zero = torch.zeros(eq.shape, dtype=torch.float64, device="cuda")
    for (i, j) in cells[:ntangent]:
        vb = torch.zeros((c.nic, c.njc), dtype=torch.float64, device="cuda")
        vb[i, j] = 1.0
        b = torch.empty_like(zero)
        eq.jvp_device(zero.data_ptr(), b.data_ptr(), vb.data_ptr())  # dR/dbeta e_c
        b = -b
        dq = torch.zeros_like(b)
        eq.tangent_solve_device(b.data_ptr(), dq.data_ptr(), rtol=1e-12)
        torch.cuda.synchronize()
        t = float((gq * dq).sum())
        tan.append({"cell": [i, j], "tangent": t, "adjoint": float(grad[i, j]),
                    "rel": abs(t - grad[i, j]) / max(abs(t), 1e-300)})
    out["tangent"] = tan
    # finite differences
    fd = []
    t0 = time.time()
    for (i, j) in cells:
        Js = []
        for sgn in (1.0, -1.0):
            beta = np.ones((c.nic, c.njc))
            beta[i, j] += sgn * h
            eq.set_beta(beta)
            ok, _ = inv.converge(eq, q0, warm=True, tol_abs=1e-13 * r0, min_steps=3, cfl=1e12, cfl_ramp=0,
                                 krylov_rtol=1e-12)
            Js.append(eq.skin_friction()[1] if ok else np.nan)
        d = (Js[0] - Js[1]) / (2 * h)
        floor = np.finfo(float).eps * abs(J0) / (2 * h * max(abs(grad[i, j]), 1e-300))
        fd.append({"cell": [i, j], "fd": d, "adjoint": float(grad[i, j]),
                   "rel": abs(d - grad[i, j]) / max(abs(grad[i, j]), 1e-300), "roundoff_floor": floor})
    eq.set_beta(np.ones((c.nic, c.njc)))
    out["fd"] = fd
    out["fd_wall_s"] = time.time() - t0
    rels = np.array([e["rel"] for e in fd])
    floors = np.array([e["roundoff_floor"] for e in fd])
    out["fd_summary"] = {"cells": len(fd), "median_rel": float(np.median(rels)), "max_rel": float(rels.max()),
                         "cells_within_10x_floor": int((rels <= 10 * floors + 1e-8).sum()),
                         "median_floor": float(np.median(floors))}
    out["tangent_max_rel"] = max(e["rel"] for e in tan)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["gradient"])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--ni", type=int, default=545)
    ap.add_argument("--nj", type=int, default=385)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    res = gradient_check(a.cells, a.ni, a.nj)
    s = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s)
    summary = {k: v for k, v in res.items() if k not in ("fd", "tangent")}
    print(json.dumps(summary, indent=1))


if __name__ == "__main__":
    sys.exit(main())
