"""Adjoint-driven field inversion of the SA production multiplier beta.

Objective (per case):  f(beta) = sum_i ((Cf_i - Cf*_i) / s)^2 + lam * sum_c (beta_c - 1)^2,
Cf over the no-slip plate's wall faces, s the plate-mean |Cf*| (with Cf ~ 4e-3
an unscaled misfit is ~1e-5 and lam = 1e-4 would hold beta at 1).  Gradient by the discrete adjoint:
    (dR/dQ)^T psi = (df/dQ)^T,      df/dbeta = 2 lam (beta - 1) - (dR/dbeta)^T psi,
every piece on the GPU through the C ABI (flow solve: st_solve; df/dQ:
st_cf_gradient_device; adjoint: st_adjoint_solve_device; (dR/dbeta)^T psi:
st_vjp_device).  The optimiser is L-BFGS (two-loop recursion, Armijo
backtracking) on the host over the beta field.  The reference has no
adjoint, objective or inversion; this module is new.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from .solver import EulerEquation, Solver, StructuredError


def plate_weights(case, xv) -> np.ndarray:
    """dx of each bottom face on the plate (zero elsewhere): drag J = sum w Cf."""
    w = np.zeros(case.nic)
    lo = max(case.i_le, 0)
    for i in range(lo, case.nic):
        xm = 0.5 * (xv[i, 0] + xv[i + 1, 0])
        if xm <= case.plate_x_end:
            w[i] = xv[i + 1, 0] - xv[i, 0]
    return w


def plate_mask(case, xv) -> np.ndarray:
    return plate_weights(case, xv) > 0


def cell_areas(xv: np.ndarray, yv: np.ndarray) -> np.ndarray:
    """Cell areas [nic][njc] from the vertices (half the cross product of the
    diagonals)."""
    return 0.5 * np.abs((xv[1:, 1:] - xv[:-1, :-1]) * (yv[:-1, 1:] - yv[1:, :-1])
                        - (xv[:-1, 1:] - xv[1:, :-1]) * (yv[1:, 1:] - yv[:-1, :-1]))


SOLVE_COLD = dict(max_steps=300, cfl=5.0, cfl_growth=2.0, rel_tolerance=1e-12, krylov_rtol=1e-4, krylov_m=150,
                  krylov_maxit=300)
# Warm restarts after a change of beta: the SA residual that beta drives is
# ~1e-8 of the momentum residual's round-off floor, so a norm test alone would
# accept the old state; at least two near-Newton steps with tight linear solves
# carry the change into the state.  (Measured on the SA plates: pseudo-time
# steps at CFL <= 1e2 from a converged state let the residual grow, even with
# beta unchanged; pure Newton (CFL 1e12) converges only for changes of beta of
# about 1e-3; this schedule, CFL 1e5 growing x10, carries the line search's
# trial steps, and a failed warm solve falls back to a cold one.)
SOLVE_WARM = dict(max_steps=60, cfl=1e5, cfl_growth=10.0, min_steps=2, rel_tolerance=1e-12, krylov_rtol=1e-8,
                  krylov_m=150, krylov_maxit=600, max_failures=40)


def converge(eq: EulerEquation, q0=None, warm=False, tol_abs=None, **over):
    """Pseudo-time Newton to steady state; returns (ok, history), history None
    when the solve diverged."""
    if q0 is not None:
        eq.set_state(q0)
    params = dict(SOLVE_WARM if warm else SOLVE_COLD)
    if tol_abs is not None:
        params.update(tolerance=tol_abs, rel_tolerance=0.0)
    params.update(over)
    try:
        return Solver(eq, **params).solve(raise_on_noconv=False)
    except StructuredError as e:
        if e.code != -3:  # ST_ERR_NONFINITE: diverged
            raise
        return False, None


def cf_adjoint_gradient(eq: EulerEquation, w: np.ndarray, rtol: float = 1e-10, maxit: int = 4000):
    """d(sum_i w_i Cf_i)/dbeta at the converged state of eq (beta as set).
    Returns (grad [nic][njc], adjoint stats)."""
    import torch
    shape = eq.shape
    g = torch.zeros(shape, dtype=torch.float64, device="cuda")
    eq.cf_gradient_device(w, g.data_ptr())
    psi = torch.zeros_like(g)
    st = eq.adjoint_solve_device(g.data_ptr(), psi.data_ptr(), rtol=rtol, maxit=maxit)
    oq = torch.empty_like(g)
    ob = torch.empty((eq.nic, eq.njc), dtype=torch.float64, device="cuda")
    eq.vjp_device(psi.data_ptr(), oq.data_ptr(), ob.data_ptr())
    torch.cuda.synchronize()
    return -ob.cpu().numpy(), st


def lbfgs_direction(g: np.ndarray, S: list, Y: list, first_step: float = 1e-2, metric=None) -> np.ndarray:
    """-H g by the L-BFGS two-loop recursion over the pairs (s_k, y_k), oldest
    first, with the initial inverse Hessian gamma M (M = `metric`, a positive
    diagonal, or the identity; gamma = s.y / y.M.y of the newest pair); without
    pairs, -M g scaled so that its largest entry is `first_step`."""
    M = 1.0 if metric is None else metric
    d = -g.copy()
    alphas = []
    for s, y in reversed(list(zip(S, Y))):
        a = (s * d).sum() / (y * s).sum()
        alphas.append(a)
        d -= a * y
    if S:
        s, y = S[-1], Y[-1]
        d = M * d * ((s * y).sum() / (y * M * y).sum())
    else:
        d = M * d
        d *= first_step / max(np.abs(d).max(), 1e-300)
    for (s, y), a in zip(zip(S, Y), reversed(alphas)):
        b = (y * d).sum() / (y * s).sum()
        d += (a - b) * s
    return d


def lbfgs_minimize(evaluate, x0: np.ndarray, max_iter: int, m: int = 10, first_step: float = 0.05,
                   gtol: float = 0.0, log=print, on_accept=None, metric=None, backtrack: float | None = None,
                   max_ls: int = 10, curvature_check: bool = True):
    """L-BFGS on f(x), evaluate(x) -> (f, g, aux) with g None where f is not
    defined (a diverged flow solve).  Armijo backtracking, at most max_ls
    trials: by a fixed factor `backtrack`, or (None) by quadratic
    interpolation of f along the direction (the new step is the parabola's
    minimiser through f(0), f'(0) and f(step), kept within [0.1, 0.5] of the
    step tried); with curvature_check a pair (s, y) enters the memory only
    with positive curvature s.y > 1e-10 |s| |y|.  A failed line search drops the memory and retries
    once along steepest descent, scaled so that its largest entry is
    first_step; a second failure ends the run.  metric: the positive diagonal
    of the initial inverse Hessian (lbfgs_direction).  on_accept(it, x, f,
    aux, step) is called at every accepted iterate.  Returns (x, f, g, aux,
    iterations)."""
    x = np.array(x0, dtype=float)
    f, g, aux = evaluate(x)
    if g is None:
        raise RuntimeError("objective undefined at the starting point")
    S, Y = [], []
    it = 0
    for it in range(1, max_iter + 1):
        accepted = False
        for attempt in range(2):
            d = lbfgs_direction(g, S, Y, first_step, metric)
            gd = float((g * d).sum())
            if gd >= 0:
                S, Y = [], []
                d = lbfgs_direction(g, S, Y, first_step, metric)
                gd = float((g * d).sum())
            step = 1.0
            for _ls in range(max_ls):
                xn = x + step * d
                fn, gn, auxn = evaluate(xn)
                if gn is not None and fn <= f + 1e-4 * step * gd:
                    accepted = True
                    break
                if backtrack is not None:
                    step *= backtrack
                    continue
                if gn is None or not np.isfinite(fn):
                    step *= 0.1
                    continue
                den = 2.0 * (fn - f - gd * step)
                trial = -gd * step * step / den if den > 0 else 0.5 * step
                step = min(0.5 * step, max(0.1 * step, trial))
            if accepted or not S:
                break
            log("inversion: line search failed at iteration %d; restarting along steepest descent" % it)
            S, Y = [], []
        if not accepted:
            log("inversion: line search failed at iteration %d" % it)
            it -= 1
            break
        s_, y_ = xn - x, gn - g
        if not curvature_check or float((s_ * y_).sum()) > 1e-10 * np.sqrt(float((s_ * s_).sum()) * float((y_ * y_).sum())):
            S.append(s_)
            Y.append(y_)
            if len(S) > m:
                S.pop(0)
                Y.pop(0)
        x, f, g, aux = xn, fn, gn, auxn
        if on_accept:
            on_accept(it, x, f, aux, step)
        if np.abs(g).max() < gtol:
            break
    return x, f, g, aux, it


@dataclasses.dataclass
class InversionResult:
    beta: np.ndarray
    q: np.ndarray
    cf: np.ndarray
    f_history: list
    misfit_history: list
    iterations: int
    wall_s: float
    flow_solves: int
    iter_wall_s: list = dataclasses.field(default_factory=list)   # wall time at each accepted iterate
    iter_cf: list = dataclasses.field(default_factory=list)       # wall Cf of each accepted iterate


def invert(eq: EulerEquation, xv: np.ndarray, cf_target: np.ndarray, q_start: np.ndarray, lam: float = 1e-4,
           max_iter: int = 40, m: int = 10, gtol: float = 1e-10, log=print, tol_abs: float | None = None,
           adj_rtol: float = 1e-8, first_step: float = 0.01, yv: np.ndarray | None = None,
           area_metric: bool = False) -> InversionResult:
    """L-BFGS over beta for f = |(Cf - Cf*) / s|^2 + lam |beta - 1|^2 on the
    plate faces, s = mean |Cf*| there.  tol_abs: absolute residual tolerance
    of the warm-started flow solves; adj_rtol: relative tolerance of the
    adjoint solves (the gradient needs a few digits, not round-off);
    area_metric (with yv, the grid's y vertices): an L-BFGS metric weighting
    each cell by 1/area; off by default (the Euclidean metric is the one
    measured to converge on the plate inversions).  The line search backtracks
    by 0.3 per trial, at most 8 trials; first_step is the largest change of
    beta on a steepest-descent step.  A failed line search drops the curvature
    pairs and retries along the steepest descent direction once before the
    inversion stops."""
    case = eq.case
    mask = plate_mask(case, xv)
    cf_scale = float(np.abs(cf_target[mask]).mean())
    t0 = time.time()
    solves = [0]
    state = {"q": q_start.copy()}

    def evaluate(beta):
        eq.set_beta(beta)
        ok, _ = converge(eq, state["q"], warm=True, tol_abs=tol_abs)
        solves[0] += 1
        if not ok:
            ok, _ = converge(eq, state["q"], warm=False, tol_abs=tol_abs)
            solves[0] += 1
            if not ok:
                return np.inf, None, None, None
        q = eq.get_state()
        cf, _ = eq.skin_friction()
        r = np.where(mask, cf - cf_target, 0.0) / cf_scale
        misfit = float((r * r).sum())
        f = misfit + lam * float(((beta - 1.0) ** 2).sum())
        g, st = cf_adjoint_gradient(eq, 2.0 * r / cf_scale, rtol=adj_rtol)
        if not st.converged:
            log("inversion: adjoint solve reached %.1e of its right-hand side" % (st.residual / st.residual0))
        g = g + 2.0 * lam * (beta - 1.0)
        return f, g, q, (misfit, cf)

    fh, mh, iter_wall, iter_cf = [], [], [], []

    def accept(it, beta, f, aux, step):
        q, (misfit, cf) = aux
        state["q"] = q
        fh.append(f)
        mh.append(misfit)
        iter_wall.append(time.time() - t0)
        iter_cf.append(cf)
        if it > 0:
            log("inversion it %3d  f %.6e  misfit %.6e  step %.2e  solves %d" % (it, f, misfit, step, solves[0]))

    def objective(beta):
        f, g, q, extra = evaluate(beta)
        return f, g, (None if g is None else (q, extra))

    beta0 = np.ones((case.nic, case.njc))
    f0, g0, aux0 = objective(beta0)
    if g0 is None:
        raise RuntimeError("flow solve failed at beta = 1")
    accept(0, beta0, f0, aux0, 0.0)
    cache = {"first": (f0, g0, aux0)}

    def objective_cached(beta):
        if "first" in cache:  # the starting point was just evaluated
            return cache.pop("first")
        return objective(beta)

    # cell areas span orders of magnitude on the stretched grids (first cell
    # 1e-7): the gradient per cell scales with its area, so the metric 1/area
    # (normalised to mean 1) gives the L-BFGS the grid-independent steepest
    # descent of the beta field instead of one that only moves large cells
    metric = None
    if area_metric and yv is not None:
        metric = 1.0 / cell_areas(xv, yv)
        metric /= metric.mean()
    beta, f, g, _, it = lbfgs_minimize(objective_cached, beta0, max_iter, m=m, first_step=first_step, gtol=gtol,
                                       log=log, on_accept=accept, metric=metric, backtrack=0.3, max_ls=8,
                                       curvature_check=False)
    eq.set_beta(beta)
    eq.set_state(state["q"])
    cf, _ = eq.skin_friction()
    return InversionResult(beta=beta, q=state["q"], cf=cf, f_history=fh, misfit_history=mh, iterations=it,
                           wall_s=time.time() - t0, flow_solves=solves[0], iter_wall_s=iter_wall, iter_cf=iter_cf)


def run_case(re_l: float, angle_deg: float, ni: int, nj: int, max_iter: int = 15, lam: float = 1e-4,
             seed: int = 20261203, log=print) -> tuple[dict, dict]:
    """One field inversion of the turbulent plate family: the target Cf is the
    solver's own Cf with beta = target_beta(seed); L-BFGS starts from beta = 1.
    Returns (summary, arrays)."""
    import tempfile
    from . import case as C
    from . import workloads
    c = workloads.turbulent_plate(tempfile.mkdtemp(), ni, nj, re_l, angle_deg, write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-7, ratio=1.05, top_angle_deg=angle_deg)
    xv, yv = g.xv, g.yv
    eq = EulerEquation(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    t0 = time.time()
    ok, hist = converge(eq)
    if not ok:
        raise RuntimeError("baseline solve failed (Re %.0e, %+.0f deg)" % (re_l, angle_deg))
    t_base = time.time() - t0
    r0 = float(hist[0, 3:].max())
    tol = 1e-12 * r0
    q_base = eq.get_state()
    cf_base, J_base = eq.skin_friction()
    beta_true = workloads.target_beta(xv, yv, seed)
    eq.set_beta(beta_true)
    ok, _ = converge(eq, q_base, warm=True, tol_abs=tol)
    if not ok:  # a large change of beta: the freestream start of the baseline solve
        ok, _ = converge(eq, C.freestream_state(c), warm=False, tol_abs=tol)
    if not ok:
        raise RuntimeError("target solve failed")
    q_true = eq.get_state()
    cf_target, J_target = eq.skin_friction()
    eq.set_beta(np.ones_like(beta_true))
    res = invert(eq, xv, cf_target, q_base, lam=lam, max_iter=max_iter, log=log, tol_abs=tol, yv=yv)
    mask = plate_mask(c, xv)
    rel_cf = lambda cf, ref=cf_target: float(np.abs((cf - ref)[mask] / ref[mask]).max())
    # the inversion's own wall time to a Cf within 1 % of the Cf it ends with
    t_1pct = next((t for t, cf in zip(res.iter_wall_s, res.iter_cf) if rel_cf(cf, res.cf) <= 0.01), res.wall_s)
    summary = {"Re_L": re_l, "angle_deg": angle_deg, "grid": [ni, nj], "baseline_solve_s": t_base,
               "baseline_steps": int(hist.shape[0] - 1), "J_base": J_base, "J_target": J_target,
               "cf_err_base": rel_cf(cf_base), "cf_err_inverted": rel_cf(res.cf),
               "misfit_initial": res.misfit_history[0], "misfit_final": res.misfit_history[-1],
               "iterations": res.iterations, "flow_solves": res.flow_solves, "wall_s": res.wall_s,
               "wall_s_to_1pct_of_final_cf": t_1pct}
    arrays = {"xv": xv, "yv": yv, "beta_true": beta_true, "beta_inv": res.beta, "q_inv": res.q, "q_true": q_true,
              "q_base": q_base, "cf_target": cf_target, "cf_inv": res.cf, "cf_base": cf_base,
              "iter_wall_s": np.array(res.iter_wall_s), "iter_cf": np.array(res.iter_cf),
              "inversion_wall_s": np.array(res.wall_s)}
    return summary, arrays
