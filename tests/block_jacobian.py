"""The implicit solver's block Jacobian restated in numpy over the oracle's
exact JVPs (test infrastructure; the product assembles on the GPU,
structured_gb300/csrc/st_solver.cu).

Layout, as on the device:
- regular blocks ``[nic][njc][13][nq][nq]`` for the 13-point stencil offsets
  OFFSETS, assembled from JVPs over a 5x5 (second order) or 3x3 (first order)
  cell colouring, with the wake ghosts' tangents held at zero so that the
  colouring sees only local dependencies;
- wake partner blocks ``[nic][4][nq][nq]``: the wake cut (bc.cpp:224-263)
  makes the bottom ghost below column a a copy of cell (nic-1-a, 0), and that
  ghost reaches rows (a-1, 0), (a, 0), (a+1, 0) and (a, 1).  Slot t of row
  column i holds d R(i, j_t) / d q(nic-1-(i-d_t), 0) for SLOTS[t] = (j_t, d_t).
  They are assembled by seeding the row-0 source cells of one half of the grid
  whose column is congruent to k mod 3 (ghost windows three columns apart
  never share a row), and reading the rows next to their mirror ghosts on the
  other half, where the seeds have no local effect."""
from __future__ import annotations

import numpy as np

OFFSETS = ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-2, 0), (2, 0), (0, -2), (0, 2),
           (-1, -1), (-1, 1), (1, -1), (1, 1))
SLOTS = ((0, -1), (0, 0), (0, 1), (1, 0))
MIN_SIDE_GAP = 6


def wake_columns(c) -> np.ndarray:
    """Mask of the columns whose bottom ghost is a wake copy (both halves of
    each bottom wake range, padded start..end -> columns start-1..end-1 and
    nic-end..nic-start)."""
    nic = c.ni - 1
    m = np.zeros(nic, dtype=bool)
    for b in c.boundaries:
        if b.type != "wake":
            continue
        if b.face != "bottom":
            raise ValueError("wake cut on the %s face" % b.face)
        end = b.end if b.end >= 0 else nic + 2 + b.end
        if b.start < 1:
            raise ValueError("wake range starts on the corner ghost")
        for ip in range(b.start, end + 1):
            m[ip - 1] = True
            m[nic - ip] = True
    return m


def side_of(i: int, nic: int) -> int:
    return 1 if 2 * i > nic - 1 else 0


def check_sides(mask: np.ndarray) -> None:
    """The two halves of the cut must be apart: a seed's own stencil (two
    columns) never reaches the rows next to another seed's mirror ghost."""
    nic = mask.size
    cols = np.nonzero(mask)[0]
    if cols.size == 0:
        return
    left = [i for i in cols if side_of(i, nic) == 0]
    right = [i for i in cols if side_of(i, nic) == 1]
    if not left or not right or min(right) - max(left) < MIN_SIDE_GAP:
        raise ValueError("wake halves closer than %d columns" % MIN_SIDE_GAP)


def assemble_regular(port, q, order: int, freeze: bool = True) -> np.ndarray:
    nic, njc, nq = q.shape
    cs = 3 if order == 1 else 5
    half = cs // 2
    jac = np.zeros((nic, njc, len(OFFSETS), nq, nq))
    ii, jj = np.meshgrid(np.arange(nic), np.arange(njc), indexing="ij")
    port.freeze_wake(freeze)
    try:
        for ci in range(cs):
            for cj in range(cs):
                on = (ii % cs == ci) & (jj % cs == cj)
                mi = (ci - ii) % cs
                mj = (cj - jj) % cs
                di = np.where(mi > half, mi - cs, mi)
                dj = np.where(mj > half, mj - cs, mj)
                for comp in range(nq):
                    v = np.zeros_like(q)
                    v[on, comp] = 1.0
                    jv = port.jvp(q, v, lhs=(order == 1))
                    for o, (oi, oj) in enumerate(OFFSETS):
                        sel = (di == oi) & (dj == oj)
                        ic, jc = ii + oi, jj + oj
                        sel &= (ic >= 0) & (ic < nic) & (jc >= 0) & (jc < njc)
                        jac[sel, o, :, comp] = jv[sel]
    finally:
        port.freeze_wake(False)
    return jac


def assemble_partners(port, q, mask: np.ndarray, order: int) -> np.ndarray:
    nic, njc, nq = q.shape
    W = np.zeros((nic, len(SLOTS), nq, nq))
    for side in (0, 1):
        for k in range(3):
            seeds = [s for s in range(nic) if mask[s] and side_of(s, nic) == side and s % 3 == k]
            if not seeds:
                continue
            for comp in range(nq):
                v = np.zeros_like(q)
                v[seeds, 0, comp] = 1.0
                jv = port.jvp(q, v, lhs=(order == 1))
                for i in range(nic):
                    for t, (j, d) in enumerate(SLOTS):
                        a = i - d
                        if a < 0 or a >= nic or not mask[a]:
                            continue
                        src = nic - 1 - a
                        if side_of(src, nic) != side or src % 3 != k:
                            continue
                        W[i, t, :, comp] = jv[i, j]
    return W


def apply(jac, W, x, trans: bool = False) -> np.ndarray:
    """J x (or J^T x) from the regular blocks and the wake partners."""
    nic, njc, nq = x.shape
    y = np.zeros_like(x)
    for o, (oi, oj) in enumerate(OFFSETS):
        for i in range(nic):
            ic = i + oi
            if ic < 0 or ic >= nic:
                continue
            for j in range(njc):
                jc = j + oj
                if jc < 0 or jc >= njc:
                    continue
                if trans:
                    y[ic, jc] += jac[i, j, o].T @ x[i, j]
                else:
                    y[i, j] += jac[i, j, o] @ x[ic, jc]
    if W is not None:
        for i in range(nic):
            for t, (j, d) in enumerate(SLOTS):
                a = i - d
                if a < 0 or a >= nic:
                    continue
                pc = nic - 1 - a
                if trans:
                    y[pc, 0] += W[i, t].T @ x[i, j]
                else:
                    y[i, j] += W[i, t] @ x[pc, 0]
    return y


def to_sparse(jac, W):
    """The same operator as a scipy CSR matrix over (i*njc + j)*nq + k."""
    import scipy.sparse as sp
    nic, njc, noff, nq, _ = jac.shape
    rows, cols, vals = [], [], []
    kk, ll = np.meshgrid(np.arange(nq), np.arange(nq), indexing="ij")
    for i in range(nic):
        for j in range(njc):
            r0 = (i * njc + j) * nq
            for o, (oi, oj) in enumerate(OFFSETS):
                ic, jc = i + oi, j + oj
                if 0 <= ic < nic and 0 <= jc < njc:
                    rows.append(r0 + kk.ravel()); cols.append((ic * njc + jc) * nq + ll.ravel())
                    vals.append(jac[i, j, o].ravel())
    if W is not None:
        for i in range(nic):
            for t, (j, d) in enumerate(SLOTS):
                a = i - d
                if 0 <= a < nic and np.any(W[i, t]):
                    r0 = (i * njc + j) * nq
                    rows.append(r0 + kk.ravel()); cols.append(((nic - 1 - a) * njc) * nq + ll.ravel())
                    vals.append(W[i, t].ravel())
    n = nic * njc * nq
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def steady_newton(port, c, q, cfl=1.0, growth=1.5, cfl_max=1e8, max_rel_drho=0.2, tol=1e-10, max_steps=80):
    """Steady state of the oracle's residual by pseudo-time Newton: each step
    solves (I/dt - J) dq = R, the implicit solver's system, exactly (sparse LU
    of the full second-order Jacobian with the wake partners), damped so that
    no density changes by more than ``max_rel_drho``; CFL grows by ``growth``
    per step.  Returns the state and the max-over-components L2 norms."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    mask = wake_columns(c)
    has_wake = bool(mask.any())
    if has_wake:
        check_sides(mask)
    q = q.copy()
    hist = []
    for _ in range(max_steps):
        R = port.residual(q)
        hist.append(np.sqrt((R ** 2).sum(axis=(0, 1))).max())
        if not np.isfinite(hist[-1]) or hist[-1] < tol:
            break
        jac = assemble_regular(port, q, 2)
        W = assemble_partners(port, q, mask, 2) if has_wake else None
        M = sp.diags(1.0 / port.dt(q, cfl).ravel()) - to_sparse(jac, W)
        dq = spla.spsolve(M.tocsc(), R.ravel()).reshape(q.shape)
        rel = np.abs(dq[..., 0] / q[..., 0]).max()
        q = q + min(1.0, max_rel_drho / rel) * dq
        cfl = min(cfl * growth, cfl_max)
    return q, np.array(hist)
