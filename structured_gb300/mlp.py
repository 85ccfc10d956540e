"""Learned SA correction: training data from field inversions, training, and
the held-out comparison of plain SA, the inverted-beta solve and the learned
solve.  The reference has no turbulence model, adjoint or learning; this
module is new.

    python -m structured_gb300.validate mlp --data DIR [--out file.json]

DIR holds the inversion_<tag>_<ni>x<nj>.npz files the inversion run writes.
Training pairs are (features of the inverted state, inverted beta) over all
cells of the cases other than Re_L = 3e6 at -2 degrees whose inversion matched
its target (plate Cf within `max_cf_err`, 5 %): an inversion that stalled far
from its target leaves a beta field that contradicts the others.
"""
from __future__ import annotations

import glob
import os
import re
import tempfile
import time

import numpy as np

HELD_OUT = "Re3e+06_a-2"


def _case_of(path: str):
    from . import workloads
    m = re.search(r"inversion_(Re([0-9.e+]+)_a([+-][0-9]+))_(\d+)x(\d+)\.npz$", os.path.basename(path))
    if not m:
        raise ValueError("not an inversion file: %s" % path)
    tag, re_l, ang, ni, nj = m.group(1), float(m.group(2)), float(m.group(3)), int(m.group(4)), int(m.group(5))
    return tag, workloads.turbulent_plate(tempfile.mkdtemp(), ni, nj, re_l, ang, write_files=False)


class _Case:
    """An inversion file's arrays, with the grid (regenerated from the case
    when the file does not hold it) and the inverted state in FP64."""

    def __init__(self, path, c):
        from . import case as C
        self._d = dict(np.load(path))
        if "xv" not in self._d:
            m = re.search(r"_a([+-][0-9]+)_", os.path.basename(path))
            g = C.flat_plate_grid(c.ni, c.nj, h1=1e-7, ratio=1.05, top_angle_deg=float(m.group(1)))
            self._d["xv"], self._d["yv"] = g.xv, g.yv
        self._d["q_inv"] = np.ascontiguousarray(self._d["q_inv"], dtype=np.float64)
        self.files = list(self._d)

    def __getitem__(self, k):
        return self._d[k]


def _eq_for(path: str):
    from .solver import EulerEquation
    tag, c = _case_of(path)
    d = _Case(path, c)
    return tag, c, d, EulerEquation(c, d["xv"], d["yv"])


def training_set(paths):
    """Device tensors (features [N][4] float32, targets [N] float32)."""
    import torch
    feats, targets = [], []
    for path in paths:
        tag, c, d, eq = _eq_for(path)
        eq.set_state(d["q_inv"])
        eq.set_beta(d["beta_inv"])
        f = torch.empty((eq.nic * eq.njc, 4), dtype=torch.float32, device="cuda")
        eq.sa_features_device(f.data_ptr())
        feats.append(f)
        targets.append(torch.tensor(d["beta_inv"].reshape(-1), dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    return torch.cat(feats), torch.cat(targets)


def cf_error(cf, cf_ref, mask):
    return float(np.abs((cf - cf_ref)[mask] / cf_ref[mask]).max())


def inversion_cf_error(path: str) -> float:
    from . import inversion as inv
    _, c = _case_of(path)
    d = _Case(path, c)
    return cf_error(d["cf_inv"], d["cf_target"], inv.plate_mask(c, d["xv"]))


def _re_of(path: str) -> str:
    return re.search(r"inversion_(Re[0-9.e+]+)_", os.path.basename(path)).group(1)


def run(data_dir: str, steps: int = 2000, batch: int = 65536, lr: float = 1e-3, seed: int = 20261203,
        max_cf_err: float = 0.05, train_mode: str = "all", log=print):
    """train_mode: "all" (every other case whose inversion matched its target
    within max_cf_err), "same_re" (those of them at the held-out case's
    Reynolds number) or "self" (the held-out case's own inversion: the
    feature set's upper bound, not a generalisation result)."""
    import torch
    from . import inversion as inv
    paths = sorted(glob.glob(os.path.join(data_dir, "inversion_*.npz")))
    test_paths = [p for p in paths if HELD_OUT in os.path.basename(p)]
    others = [p for p in paths if HELD_OUT not in os.path.basename(p)]
    errs = {os.path.basename(p): inversion_cf_error(p) for p in others}
    train_paths = [p for p in others if errs[os.path.basename(p)] <= max_cf_err]
    if train_mode == "same_re" and test_paths:
        train_paths = [p for p in train_paths if _re_of(p) == _re_of(test_paths[0])]
    elif train_mode == "self":
        train_paths = list(test_paths)
    if not train_paths or not test_paths:
        raise FileNotFoundError("need the held-out case %s and training cases in %s" % (HELD_OUT, data_dir))
    out = {"train_mode": train_mode, "train_cases": [os.path.basename(p) for p in train_paths],
           "held_out": os.path.basename(test_paths[0]),
           "excluded": {k: v for k, v in errs.items() if v > max_cf_err}}
    t0 = time.time()
    feat, target = training_set(train_paths)
    f_np = feat.cpu().numpy()
    mean, std = f_np.mean(axis=0), f_np.std(axis=0) + 1e-6
    out["samples"] = int(feat.shape[0])
    out["feature_mean"], out["feature_std"] = mean.tolist(), std.tolist()
    # train on the held-out case's context (any SA context holds the network)
    tag, c, d, eq = _eq_for(test_paths[0])
    eq.mlp_set_normalization(mean, std)
    eq.mlp_init(seed)
    torch.cuda.synchronize()
    t1 = time.time()
    loss = eq.mlp_train(feat.data_ptr(), target.data_ptr(), int(feat.shape[0]), steps, batch=batch, lr=lr, seed=seed)
    out["train"] = {"steps": steps, "batch": batch, "lr": lr, "wall_s": time.time() - t1,
                    "loss_first": float(loss[0]), "loss_last": float(loss[-20:].mean())}
    log("[train] %s" % out["train"])
    params = eq.mlp_params()
    # held-out comparison against the inverted-beta FP64 solution
    mask = inv.plate_mask(c, d["xv"])
    cf_inv, cf_target = d["cf_inv"], d["cf_target"]
    from . import case as C

    def solve(label, beta=None, learned=False, chunk=4, max_steps=200):
        """From freestream, in chunks of Newton steps (the CFL carried over);
        after each chunk the plate Cf is compared with the inverted-beta
        solution and the first time it is within 1 % is recorded."""
        eq.mlp_enable(False)
        eq.set_beta(np.ones((c.nic, c.njc)) if beta is None else beta)
        if learned:
            eq.mlp_enable(True)
        eq.set_state(C.freestream_state(c))
        torch.cuda.synchronize()
        ts = time.time()
        steps, cfl, tol, ok, t_hit, steps_hit, diverged = 0, inv.SOLVE_COLD["cfl"], None, False, None, None, False
        while steps < max_steps and not ok:
            ok, hist = inv.converge(eq, None, tol_abs=tol, cfl=cfl, max_steps=chunk)
            if hist is None:
                diverged = True
                break
            if tol is None:
                tol = 1e-12 * float(hist[0, 3:].max())
            steps += int(hist.shape[0] - 1)
            cfl = float(hist[-1, 1]) * inv.SOLVE_COLD["cfl_growth"]
            cf, _ = eq.skin_friction()
            if t_hit is None and cf_error(cf, cf_inv, mask) <= 0.01:
                t_hit, steps_hit = time.time() - ts, steps
        wall = time.time() - ts
        cf, J = eq.skin_friction()
        eq.mlp_enable(False)
        res = {"converged": bool(ok), "diverged": diverged, "steps": steps, "wall_s": wall,
               "time_to_cf_err_1pct_s": t_hit, "steps_to_cf_err_1pct": steps_hit,
               "cf_err_vs_inverted": cf_error(cf, cf_inv, mask), "cf_err_vs_target": cf_error(cf, cf_target, mask),
               "J": J}
        log("[%s] %s" % (label, res))
        return res, cf

    if "inversion_wall_s" in d.files:
        # the held-out case's own field inversion: total wall time, and the
        # time to its first iterate whose Cf is within 1 % of its final Cf
        tw = d["iter_wall_s"]
        within = [float(t) for t, cf in zip(tw, d["iter_cf"]) if cf_error(cf, cf_inv, mask) <= 0.01]
        out["field_inversion"] = {"wall_s": float(d["inversion_wall_s"]),
                                  "wall_s_to_cf_err_1pct": within[0] if within else float(d["inversion_wall_s"]),
                                  "iterations": int(len(tw) - 1)}
    out["plain_sa"], _ = solve("plain SA")
    out["inverted_beta"], _ = solve("inverted beta", beta=d["beta_inv"])
    out["learned"], cf_l = solve("learned", learned=True)
    b = torch.empty(c.nic * c.njc, dtype=torch.float64, device="cuda")
    eq.mlp_beta_device(b.data_ptr())
    torch.cuda.synchronize()
    bl = b.cpu().numpy().reshape(c.nic, c.njc)
    bl_err = bl - d["beta_inv"]
    out["learned_beta_rms_err_vs_inverted"] = float(np.sqrt((bl_err ** 2).mean()))
    out["wall_s"] = time.time() - t0
    return out, params, loss
