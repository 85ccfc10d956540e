"""The implicit solver's block Jacobian restated in numpy over the oracle's
exact JVPs (test infrastructure; the product assembles on the GPU,
structured_gb300/csrc/st_solver.cu and st_partner.cuh).

Layout, as on the device:
- regular blocks ``[nic][njc][13][nq][nq]`` for the 13-point stencil offsets
  OFFSETS, assembled from JVPs over a 5x5 (second order) or 3x3 (first order)
  cell colouring, with the tangents of the non-local boundary copies (wake
  cut, periodic) held at zero so that the colouring sees only local
  dependencies;
- partner blocks per family of copied ghosts, ``[line length][4][nq][nq]``:
  FAM_WAKE (bc.cpp:224-263: the bottom ghost below column b copies cell
  (nic-1-b, 0)), FAM_LEFT and FAM_RIGHT (bc.cpp:329-365: the ghost left of
  row b copies cell (nic-1, b), the one right of it cell (0, b)).  Ghost b
  reaches the rows at line positions b-1, b, b+1 next to its boundary and the
  row at b one further in; slot t of line position p holds the block of row
  fam_row(f, p, t) against the source of ghost p - SLOTS[t][1].  A partner pass
  seeds the sources of the ghosts b = k mod 3 of one family and keeps the
  difference of a full and a frozen JVP: the part the copies carry."""
from __future__ import annotations

import numpy as np

OFFSETS = ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-2, 0), (2, 0), (0, -2), (0, 2),
           (-1, -1), (-1, 1), (1, -1), (1, 1))
SLOTS = ((0, -1), (0, 0), (0, 1), (1, 0))  # (distance from the boundary, row position - ghost position)
FAM_WAKE, FAM_LEFT, FAM_RIGHT = 0, 1, 2


def fam_len(f, nic, njc):
    return nic if f == FAM_WAKE else njc


def fam_row(f, p, t, nic):
    l = SLOTS[t][0]
    if f == FAM_WAKE:
        return p, l
    return (l, p) if f == FAM_LEFT else (nic - 1 - l, p)


def fam_src(f, b, nic):
    if f == FAM_WAKE:
        return nic - 1 - b, 0
    return (nic - 1, b) if f == FAM_LEFT else (0, b)


def partner_masks(c):
    """Ghost masks of the non-local copies and which families occur; ValueError
    for the boundary lists the layout cannot hold."""
    nic, njc = c.ni - 1, c.nj - 1
    masks = [np.zeros(nic, dtype=bool), np.zeros(njc, dtype=bool), np.zeros(njc, dtype=bool)]
    on = [False, False, False]
    for b in c.boundaries:
        if b.type not in ("wake", "periodic"):
            continue
        bt = b.face in ("bottom", "top")
        end = b.end if b.end >= 0 else (nic if bt else njc) + 2 + b.end
        if b.start > end:
            continue
        if b.type == "wake":
            if b.face != "bottom":
                raise ValueError("wake cut on the %s face" % b.face)
            if b.start < 1 or end > nic:
                raise ValueError("wake range on a corner ghost")
            for ip in range(b.start, end + 1):
                masks[FAM_WAKE][ip - 1] = True
                masks[FAM_WAKE][nic - ip] = True
            on[FAM_WAKE] = True
        else:
            if bt:
                raise ValueError("periodic boundaries on the %s face" % b.face)
            if b.start > 1 or end < njc:
                raise ValueError("periodic range not covering every row")
            masks[FAM_LEFT][:] = True
            masks[FAM_RIGHT][:] = True
            on[FAM_LEFT] = on[FAM_RIGHT] = True
    if on[FAM_WAKE] and on[FAM_LEFT]:
        raise ValueError("a wake cut together with periodic boundaries")
    if (on[FAM_WAKE] or on[FAM_LEFT]) and (nic < 2 or njc < 2):
        raise ValueError("fewer than two cells across")
    return masks, on


def assemble_regular(port, q, order: int, freeze: bool = True) -> np.ndarray:
    nic, njc, nq = q.shape
    cs = 3 if order == 1 else 5
    half = cs // 2
    jac = np.zeros((nic, njc, len(OFFSETS), nq, nq))
    ii, jj = np.meshgrid(np.arange(nic), np.arange(njc), indexing="ij")
    port.freeze_nonlocal(freeze)
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
        port.freeze_nonlocal(False)
    return jac


def assemble_partners(port, q, masks, on, order: int):
    """Partner blocks per family (None where the family is absent)."""
    nic, njc, nq = q.shape
    W = [None, None, None]
    for f in range(3):
        if not on[f]:
            continue
        n = fam_len(f, nic, njc)
        Wf = np.zeros((n, len(SLOTS), nq, nq))
        for k in range(3):
            ghosts = [b for b in range(k, n, 3) if masks[f][b]]
            if not ghosts:
                continue
            for comp in range(nq):
                v = np.zeros_like(q)
                for b in ghosts:
                    v[fam_src(f, b, nic) + (comp,)] = 1.0
                full = port.jvp(q, v, lhs=(order == 1))
                port.freeze_nonlocal(True)
                try:
                    frozen = port.jvp(q, v, lhs=(order == 1))
                finally:
                    port.freeze_nonlocal(False)
                for p in range(n):
                    for t, (l, d) in enumerate(SLOTS):
                        b = p - d
                        if 0 <= b < n and masks[f][b] and b % 3 == k:
                            r = fam_row(f, p, t, nic)
                            Wf[p, t, :, comp] = full[r] - frozen[r]
        W[f] = Wf
    return W


def _partner_terms(W, nic, njc):
    """(row cell, source cell, block) of every partner block."""
    for f in range(3):
        if W is None or W[f] is None:
            continue
        n = fam_len(f, nic, njc)
        for p in range(n):
            for t, (l, d) in enumerate(SLOTS):
                b = p - d
                if 0 <= b < n:
                    yield fam_row(f, p, t, nic), fam_src(f, b, nic), W[f][p, t]


def apply(jac, W, x, trans: bool = False) -> np.ndarray:
    """J x (or J^T x) from the regular blocks and the partner blocks."""
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
    for r, src, w in _partner_terms(W, nic, njc):
        if trans:
            y[src] += w.T @ x[r]
        else:
            y[r] += w @ x[src]
    return y


def fold(jac, W):
    """The preconditioner's copy of the regular blocks with the partner blocks
    whose source lies in the row's 3x3 neighbourhood (the ILU(0) pattern)
    added, as st_solver.cu prepares it."""
    out = jac.copy()
    nic, njc = jac.shape[:2]
    for (ri, rj), (si, sj), w in _partner_terms(W, nic, njc):
        di, dj = si - ri, sj - rj
        if abs(di) <= 1 and abs(dj) <= 1:
            out[ri, rj, OFFSETS.index((di, dj))] += w
    return out


def to_sparse(jac, W):
    """The same operator as a scipy CSR matrix over (i*njc + j)*nq + k
    (duplicate entries are summed)."""
    import scipy.sparse as sp
    nic, njc, noff, nq, _ = jac.shape
    rows, cols, vals = [], [], []
    kk, ll = np.meshgrid(np.arange(nq), np.arange(nq), indexing="ij")
    ii, jj = np.meshgrid(np.arange(nic), np.arange(njc), indexing="ij")
    for o, (oi, oj) in enumerate(OFFSETS):
        ic, jc = ii + oi, jj + oj
        ok = (ic >= 0) & (ic < nic) & (jc >= 0) & (jc < njc)
        r0 = ((ii * njc + jj) * nq)[ok]
        c0 = ((ic * njc + jc) * nq)[ok]
        rows.append((r0[:, None] + kk.ravel()[None, :]).ravel())
        cols.append((c0[:, None] + ll.ravel()[None, :]).ravel())
        vals.append(jac[:, :, o][ok].reshape(-1, nq * nq).ravel())
    for (ri, rj), (si, sj), w in _partner_terms(W, nic, njc):
        if np.any(w):
            rows.append((ri * njc + rj) * nq + kk.ravel())
            cols.append((si * njc + sj) * nq + ll.ravel())
            vals.append(w.ravel())
    n = nic * njc * nq
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def block_ilu0(M, nic: int, njc: int, nq: int):
    """Block ILU(0) of a sparse matrix over the 3x3 neighbourhood in natural
    cell order (the preconditioner st_solver.cu factors, here in FP64);
    returns the solve v -> (LU)^-1 v."""
    M = M.tocsr()
    n = nic * njc
    nbrs = []
    for c in range(n):
        i, j = divmod(c, njc)
        nbrs.append(sorted(ii * njc + jj for ii in (i - 1, i, i + 1) for jj in (j - 1, j, j + 1)
                           if 0 <= ii < nic and 0 <= jj < njc))
    blk = {(r, c): M[r * nq:(r + 1) * nq, c * nq:(c + 1) * nq].toarray() for r in range(n) for c in nbrs[r]}
    inv = [None] * n
    for r in range(n):
        for k in nbrs[r]:
            if k >= r:
                break
            blk[(r, k)] = blk[(r, k)] @ inv[k]
            for j in nbrs[k]:
                if j > k and (r, j) in blk:
                    blk[(r, j)] = blk[(r, j)] - blk[(r, k)] @ blk[(k, j)]
        inv[r] = np.linalg.inv(blk[(r, r)])

    def solve(v):
        y = np.asarray(v, dtype=float).reshape(n, nq).copy()
        for r in range(n):
            for k in nbrs[r]:
                if k >= r:
                    break
                y[r] -= blk[(r, k)] @ y[k]
        for r in range(n - 1, -1, -1):
            for j in nbrs[r]:
                if j > r:
                    y[r] -= blk[(r, j)] @ y[j]
            y[r] = inv[r] @ y[r]
        return y.ravel()
    return solve


def steady_newton(port, c, q, cfl=1.0, growth=1.5, cfl_max=1e8, max_rel_drho=0.2, tol=1e-10, max_steps=80):
    """Steady state of the oracle's residual by pseudo-time Newton: each step
    solves (I/dt - J) dq = R, the implicit solver's system, exactly (sparse LU
    of the full second-order Jacobian with the partner blocks), damped so that
    no density changes by more than ``max_rel_drho``; CFL grows by ``growth``
    per step.  Returns the state and the max-over-components L2 norms."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    masks, on = partner_masks(c)
    q = q.copy()
    hist = []
    for _ in range(max_steps):
        R = port.residual(q)
        hist.append(np.sqrt((R ** 2).sum(axis=(0, 1))).max())
        if not np.isfinite(hist[-1]) or hist[-1] < tol:
            break
        jac = assemble_regular(port, q, 2)
        W = assemble_partners(port, q, masks, on, 2)
        M = sp.diags(1.0 / port.dt(q, cfl).ravel()) - to_sparse(jac, W)
        dq = spla.spsolve(M.tocsc(), R.ravel()).reshape(q.shape)
        rel = np.abs(dq[..., 0] / q[..., 0]).max()
        q = q + min(1.0, max_rel_drho / rel) * dq
        cfl = min(cfl * growth, cfl_max)
    return q, np.array(hist)
