"""End-to-end checks of the implicit solve and the discrete adjoint on the
turbulent flat plate (545x385, first cell 1e-7 at ratio 1.05, M=0.2,
Re_L=5e6, SA with beta = 1, J = drag on the plate):

  python -m structured_gb300.validate gradient [--cells 64] [--out file.json]
  python -m structured_gb300.validate inversion [--ni --nj --iters] [--out dir]
  python -m structured_gb300.validate mlp --data dir [--steps] [--out file.json]
  python -m structured_gb300.validate closure --data dirs [--steps] [--out file.json]
  python -m structured_gb300.validate heldout [--ni --nj --iters --study] [--out file.json]

1. pseudo-time Newton from freestream to steady state;
2. dJ/dbeta by one adjoint solve;
3. tangent check: dJ/dbeta_c = (dJ/dQ) dQ/dbeta_c by one forward-sensitivity
   linear solve per cell on the first `ntangent` cells (an independent solve
   with the untransposed operator);
4. central finite differences (step 1e-6) on seeded cells with
   |dJ/dbeta_c| >= 1e-3 max.  Each perturbed state is one exact Newton step
   from the converged state (the perturbation enters linearly; the step's
   O(h^2) remainder is below the noise).  Each cell's round-off floor
   eps |J| / (2h |g_c|) is stated: a difference quotient of step 1e-6 on a
   state converged to round-off resolves the gradient only to a few times
   that.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np


# the right-hand side of a perturbed step is dominated by h dR/dbeta_c, so a
# 1e-7 linear solve keeps the step's error far below the noise of J
FD_STEP = dict(warm=True, tol_abs=0.0, min_steps=1, max_steps=1, cfl=1e12, cfl_ramp=0, krylov_rtol=1e-7,
               reject_factor=1e30, krylov_maxit=3000)


def gradient_check(ncells: int = 64, ni: int = 545, nj: int = 385, h: float = 1e-6, seed: int = 20261203,
                   ntangent: int = 8, out_path: str | None = None, log=print):
    import torch
    from . import case as C
    from . import inversion as inv
    from . import workloads
    from .solver import EulerEquation, Solver
    out = {}

    def save(stage):
        log("[%s] %s" % (stage, json.dumps({k: v for k, v in out.items() if k not in ("fd", "tangent")})))
        if out_path:
            with open(out_path, "w") as f:
                json.dump(out, f, indent=1)
    tmp = tempfile.mkdtemp()
    c = workloads.turbulent_plate(tmp, ni, nj, write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-7, ratio=1.05)
    xv, yv = g.xv, g.yv
    eq = EulerEquation(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    t0 = time.time()
    ok, hist = inv.converge(eq)
    if hist is None:
        out["flow_solve"] = {"converged": False, "diverged": True, "wall_s": time.time() - t0}
        save("flow solve")
        return out
    out["flow_solve"] = {"converged": bool(ok), "steps": int(hist.shape[0] - 1), "wall_s": time.time() - t0,
                         "residual_initial": float(hist[0, 3:].max()), "residual_final": float(hist[-1, 3:].max())}
    save("flow solve")
    if not ok:
        return out
    r0 = float(hist[0, 3:].max())
    q0 = eq.get_state()
    w = inv.plate_weights(c, xv)
    cf, J0 = eq.skin_friction()
    out["J"] = J0
    t0 = time.time()
    grad, st = inv.cf_adjoint_gradient(eq, w, rtol=1e-12, maxit=6000)
    out["adjoint"] = {"wall_s": time.time() - t0, "gmres_iterations": int(st.iterations),
                      "converged": int(st.converged), "residual_ratio": st.residual / max(st.residual0, 1e-300)}
    save("adjoint")
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
        ts = eq.tangent_solve_device(b.data_ptr(), dq.data_ptr(), rtol=1e-10, maxit=4000)
        torch.cuda.synchronize()
        t = float((gq * dq).sum())
        tan.append({"cell": [i, j], "tangent": t, "adjoint": float(grad[i, j]), "gmres_iterations": int(ts.iterations),
                    "converged": int(ts.converged), "rel": abs(t - grad[i, j]) / max(abs(t), 1e-300)})
        log("tangent %s" % json.dumps(tan[-1]))
    out["tangent"] = tan
    # finite differences
    def perturbed_J(beta):
        eq.set_beta(beta)
        inv.converge(eq, q0, **FD_STEP)
        return eq.skin_friction()[1]
    t0 = time.time()
    fd = []
    for (i, j) in cells:
        Js = []
        for sgn in (1.0, -1.0):
            beta = np.ones((c.nic, c.njc))
            beta[i, j] += sgn * h
            Js.append(perturbed_J(beta))
        d = (Js[0] - Js[1]) / (2 * h)
        gc = max(abs(grad[i, j]), 1e-300)
        fd.append({"cell": [i, j], "fd": d, "adjoint": float(grad[i, j]), "rel": abs(d - grad[i, j]) / gc,
                   "roundoff_floor": np.finfo(float).eps * abs(J0) / (2 * h * gc)})
        log("fd %d/%d %s  (%.0f s)" % (len(fd), len(cells), json.dumps(fd[-1]), time.time() - t0))
        if len(fd) % 8 == 0:
            out["fd"] = fd
            save("fd")
    eq.set_beta(np.ones((c.nic, c.njc)))
    out["fd"] = fd
    out["fd_wall_s"] = time.time() - t0
    rels = np.array([e["rel"] for e in fd])
    floors = np.array([e["roundoff_floor"] for e in fd])
    out["fd_summary"] = {"cells": len(fd), "step": h, "median_rel": float(np.median(rels)),
                         "max_rel": float(rels.max()), "cells_within_1e-8": int((rels <= 1e-8).sum()),
                         "cells_within_10x_floor": int((rels <= 10 * floors).sum()),
                         "median_floor": float(np.median(floors))}
    out["tangent_summary"] = {"cells": len(tan), "max_rel": max(e["rel"] for e in tan),
                              "all_converged": all(e["converged"] for e in tan)}
    save("done")
    return out


def inversions(ni: int, nj: int, iters: int, out_dir: str | None, only: str | None = None, log=print):
    """The nine field inversions (Re_L in {1e6, 3e6, 1e7} x top angle in
    {0, +2, -2} degrees); per case a JSON summary line and, with out_dir, an
    .npz of the fields."""
    import os
    from . import inversion as inv
    summaries = []
    for re_l in (1e6, 3e6, 1e7):
        for ang in (0.0, 2.0, -2.0):
            tag = "Re%.0e_a%+.0f" % (re_l, ang)
            if only and tag not in only.split(","):
                continue
            summary, arrays = inv.run_case(re_l, ang, ni, nj, max_iter=iters, log=log)
            summaries.append(summary)
            log("[case] " + json.dumps(summary))
            if out_dir:
                os.makedirs(out_dir, exist_ok=True)
                # what training and the held-out comparison read: the inverted
                # beta (FP64), the inverted state for the features (FP32), the
                # wall Cf arrays and the inversion's history; the grid is
                # regenerated from the case
                keep = {k: arrays[k] for k in ("beta_inv", "cf_target", "cf_inv", "cf_base", "iter_wall_s", "iter_cf",
                                               "inversion_wall_s")}
                keep["q_inv"] = arrays["q_inv"].astype(np.float32)
                np.savez_compressed(os.path.join(out_dir, "inversion_%s_%dx%d.npz" % (tag, ni, nj)), **keep)
                with open(os.path.join(out_dir, "inversions_%dx%d.json" % (ni, nj)), "w") as f:
                    json.dump(summaries, f, indent=1)
    return summaries


def closure(data_dirs, steps: int, out_path: str | None, log=print):
    """The learned-correction study over the inversion files of data_dirs:
    the inversions' summaries, then training on all other cases that matched
    their targets, on those at the held-out case's Reynolds number only, and on
    the held-out case itself (the feature set's upper bound), each followed by
    the held-out comparison of plain SA, the inverted-beta solve and the
    learned solve."""
    import glob
    import shutil
    import tempfile
    from . import mlp
    work = tempfile.mkdtemp()
    summaries = []
    for d in data_dirs:
        for p in glob.glob(os.path.join(d, "inversion_*.npz")):
            shutil.copy(p, work)
        for p in glob.glob(os.path.join(d, "inversions_*.json")):
            summaries += json.load(open(p))
    out = {"inversions": summaries, "training": {}}
    for mode in ("all", "same_re", "self"):
        res, params, loss = mlp.run(work, steps=steps, train_mode=mode, log=log)
        out["training"][mode] = res
        if out_path:
            with open(out_path, "w") as f:
                json.dump(out, f, indent=1)
            np.save(os.path.splitext(out_path)[0] + "_%s_params.npy" % mode, params)
    if out_path:
        # the held-out case's wall Cf: of its inverted-beta solution and its target
        held = glob.glob(os.path.join(work, "inversion_%s_*.npz" % mlp.HELD_OUT))[0]
        d = np.load(held)
        np.savez(os.path.splitext(out_path)[0] + "_heldout.npz", cf_inv=d["cf_inv"], cf_target=d["cf_target"],
                 name=os.path.basename(held))
    return out


def heldout(ni: int, nj: int, iters: int, study: str, out_path: str | None, log=print):
    """The learned-correction workload's held-out case (Re_L 3e6, top inclined
    at -2 deg) on an ni x nj grid.  Plain SA and the learned solve both start
    from freestream and are timed.  The learned solve uses the network of the
    study `study`, trained on the eight other cases' inversions at the
    study's grid.  Then the case's own field inversion runs, and the plate Cf
    of both solves is compared with the inverted-beta solution and with the
    target Cf the inversion aims for (max and mean over the plate faces).
    out_path (a JSON) is written after each stage, and an .npz beside it holds
    the wall Cf arrays."""
    import torch
    from . import case as C
    from . import inversion as inv
    from . import workloads
    from .solver import EulerEquation
    re_l, ang = 3e6, -2.0
    res = json.load(open(study + ".json"))["training"]["all"]
    params = np.load(study + "_all_params.npy")
    out = {"case": "turbulent plate %dx%d, Re_L %.0e, top %+.0f deg (held out)" % (ni, nj, re_l, ang),
           "network": os.path.basename(study) + "_all_params.npy", "network_train_cases": res["train_cases"]}

    def save():
        if out_path:
            with open(out_path, "w") as f:
                json.dump(out, f, indent=1)

    c = workloads.turbulent_plate(tempfile.mkdtemp(), ni, nj, re_l, ang, write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-7, ratio=1.05, top_angle_deg=ang)
    mask = inv.plate_mask(c, g.xv)
    eq = EulerEquation(c, g.xv, g.yv)
    cfs = {}
    for label, learned in (("plain_sa", False), ("learned", True)):
        if learned:
            eq.mlp_init(0)
            eq.mlp_set_params(params.astype(np.float32))
            eq.mlp_set_normalization(np.array(res["feature_mean"], np.float32), np.array(res["feature_std"], np.float32))
            eq.mlp_enable(True)
        eq.set_state(C.freestream_state(c))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ok, hist = inv.converge(eq)
        wall = time.perf_counter() - t0
        cfs[label] = eq.skin_friction()[0]
        out[label] = {"solve_s": wall, "converged": bool(ok),
                      "steps": int(hist.shape[0] - 1) if hist is not None else None}
        log("%s: %s" % (label, json.dumps(out[label])))
        save()
    eq.mlp_enable(False)
    eq.close()
    summary, arrays = inv.run_case(re_l, ang, ni, nj, max_iter=iters, log=log)
    cf_inv, cf_t = arrays["cf_inv"], arrays["cf_target"]
    err = lambda cf, ref: np.abs((cf - ref)[mask] / ref[mask])
    out["inversion"] = summary
    for label in ("plain_sa", "learned"):
        e_inv, e_t = err(cfs[label], cf_inv), err(cfs[label], cf_t)
        out[label].update(cf_err_vs_inverted=float(e_inv.max()), cf_err_vs_target=float(e_t.max()),
                          cf_err_vs_target_mean=float(e_t.mean()))
    log("[heldout] " + json.dumps(out))
    save()
    if out_path:
        np.savez_compressed(os.path.splitext(out_path)[0] + ".npz", cf_inv=cf_inv, cf_target=arrays["cf_target"],
                            cf_plain=cfs["plain_sa"], cf_learned=cfs["learned"], iter_wall_s=arrays["iter_wall_s"],
                            iter_cf=arrays["iter_cf"])
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["gradient", "inversion", "mlp", "closure", "heldout"])
    ap.add_argument("--data", default=None)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--iters", type=int, default=15)
    ap.add_argument("--only", default=None)
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--ni", type=int, default=545)
    ap.add_argument("--nj", type=int, default=385)
    ap.add_argument("--tangent", type=int, default=8)
    ap.add_argument("--out", default=None)
    ap.add_argument("--train", default="all", choices=["all", "same_re", "self"])
    ap.add_argument("--study", default=os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                    "results", "closure_273x193"))
    a = ap.parse_args(argv)
    if a.what == "heldout":
        heldout(a.ni, a.nj, a.iters, a.study, a.out, log=lambda m: print(m, flush=True))
        return 0
    if a.what == "inversion":
        inversions(a.ni, a.nj, a.iters, a.out, a.only, log=lambda m: print(m, flush=True))
        return 0
    if a.what == "closure":
        closure(a.data.split(","), a.steps, a.out, log=lambda m: print(m, flush=True))
        return 0
    if a.what == "mlp":
        from . import mlp
        res, params, loss = mlp.run(a.data, steps=a.steps, train_mode=a.train, log=lambda m: print(m, flush=True))
        print(json.dumps(res, indent=1))
        if a.out:
            with open(a.out, "w") as f:
                json.dump(res, f, indent=1)
            np.save(os.path.splitext(a.out)[0] + "_params.npy", params)
            np.save(os.path.splitext(a.out)[0] + "_loss.npy", loss)
        return 0
    res = gradient_check(a.cells, a.ni, a.nj, ntangent=a.tangent, out_path=a.out, log=lambda m: print(m, flush=True))
    summary = {k: v for k, v in res.items() if k not in ("fd", "tangent")}
    print(json.dumps(summary, indent=1))


if __name__ == "__main__":
    sys.exit(main())
