"""Non-local boundary copies in the implicit solver's Jacobian, on CPU against
the oracle: the wake cut of a NACA 0012 C-grid (bc.cpp:224-263) and the
periodic channel (bc.cpp:329-365).  Where their coupling lands, the block
layout the GPU assembles (regular 13-point blocks from a frozen colouring plus
four partner slots per ghost, tests/block_jacobian.py) reproducing the
oracle's exact JVP and VJP, Newton on it converging superlinearly, and the
device source of the partner pass (structured_gb300/csrc/st_partner.cuh,
compiled for the host by tests/partner_kernels_host.cpp) matching the numpy
layout without touching memory outside its buffers."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import block_jacobian as BJ
from structured_gb300 import case as C

VARIANTS = [("none", "roe", 2), ("sa", "roe", 2), ("none", "ausm", 2), ("none", "roe", 1), ("sa", "roe", 1)]


def naca(tmp_path, turbulence="none", flux="roe", ni=41, nj=9, tail=11):
    from oracle.port import PortCase
    c = C.naca0012_case(str(tmp_path), "naca", ni=ni, nj=nj, tail=tail)
    c.turbulence, c.flux = turbulence, flux
    xv, yv = C.load_grid(c)
    return c, PortCase(c, xv, yv)


def channel(tmp_path, ni=3, nj=11, turbulence="none", flux="roe"):
    from oracle.port import PortCase
    c = C.channel_case(str(tmp_path), "ch", nj=nj, ni=ni)
    c.turbulence, c.flux = turbulence, flux
    c.lhs_order = 1  # lhs=True evaluates the first-order residual, as in the NACA case
    xv, yv = C.load_grid(c)
    return c, PortCase(c, xv, yv)


def dense_blocks(port, q, order):
    """max |entry| of every (row cell, column cell) block of the Jacobian."""
    nic, njc, nq = q.shape
    B = np.zeros((nic, njc, nic, njc))
    for i in range(nic):
        for j in range(njc):
            for k in range(nq):
                v = np.zeros_like(q)
                v[i, j, k] = 1.0
                B[:, :, i, j] = np.maximum(B[:, :, i, j], np.abs(port.jvp(q, v, lhs=(order == 1))).max(axis=2))
    return B


def off_stencil(B):
    out = []
    for ri, rj, ci, cj in zip(*np.nonzero(B)):
        if (ci - ri, cj - rj) not in BJ.OFFSETS:
            out.append((int(ri), int(rj), int(ci), int(cj)))
    return out


def copy_part(port, q, order):
    """(row cell, column cell) pairs where the full and the frozen Jacobian differ."""
    nic, njc, nq = q.shape
    out = set()
    for i in range(nic):
        for j in range(njc):
            for k in range(nq):
                v = np.zeros_like(q)
                v[i, j, k] = 1.0
                full = port.jvp(q, v, lhs=(order == 1))
                port.freeze_nonlocal(True)
                try:
                    frozen = port.jvp(q, v, lhs=(order == 1))
                finally:
                    port.freeze_nonlocal(False)
                for ri, rj in zip(*np.nonzero(np.abs(full - frozen).max(axis=2))):
                    out.add(((int(ri), int(rj)), (i, j)))
    return out


def slot_pairs(c, nic, njc):
    masks, on = BJ.partner_masks(c)
    pairs = set()
    for f in range(3):
        if not on[f]:
            continue
        n = BJ.fam_len(f, nic, njc)
        for p in range(n):
            for t, (l, d) in enumerate(BJ.SLOTS):
                b = p - d
                if 0 <= b < n and masks[f][b]:
                    pairs.add((BJ.fam_row(f, p, t, nic), BJ.fam_src(f, b, nic)))
    return pairs


@pytest.mark.parametrize("which,turbulence,order", [("naca", "none", 2), ("naca", "sa", 2), ("naca", "none", 1),
                                                     ("channel2", "none", 2), ("channel6", "sa", 2),
                                                     ("channel6", "none", 1)])
def test_copy_coupling_lands_in_the_partner_slots(port_built, tmp_path, which, turbulence, order):
    if which == "naca":
        c, port = naca(tmp_path, turbulence)
    else:
        c, port = channel(tmp_path, ni=3 if which == "channel2" else 7, turbulence=turbulence)
    q = C.perturbed_state(c, 7)
    nic, njc, _ = q.shape
    part = copy_part(port, q, order)
    assert part
    assert part <= slot_pairs(c, nic, njc)
    # with the copies frozen only the 13-point stencil is left
    port.freeze_nonlocal(True)
    try:
        assert off_stencil(dense_blocks(port, q, order)) == []
    finally:
        port.freeze_nonlocal(False)


def products_match(c, port, q, order):
    masks, on = BJ.partner_masks(c)
    jac = BJ.assemble_regular(port, q, order)
    W = BJ.assemble_partners(port, q, masks, on, order)
    x = np.random.default_rng(3).standard_normal(q.shape)
    jv = port.jvp(q, x, lhs=(order == 1))
    vj, _ = port.vjp(q, x, lhs=(order == 1))
    assert np.abs(BJ.apply(jac, W, x) - jv).max() < 1e-14 * np.abs(jv).max()
    assert np.abs(BJ.apply(jac, W, x, trans=True) - vj).max() < 1e-14 * np.abs(vj).max()
    # the partners carry a first-order share of the product on these grids
    assert np.abs(BJ.apply(jac, None, x) - jv).max() > 1e-3 * np.abs(jv).max()
    A = BJ.to_sparse(jac, W)
    assert np.abs(A @ x.ravel() - jv.ravel()).max() < 1e-14 * np.abs(jv).max()


@pytest.mark.parametrize("turbulence,flux,order", VARIANTS)
def test_wake_layout_reproduces_oracle_products(port_built, tmp_path, turbulence, flux, order):
    c, port = naca(tmp_path, turbulence, flux)
    products_match(c, port, C.perturbed_state(c, 11), order)


@pytest.mark.parametrize("ni", [3, 4, 8])
@pytest.mark.parametrize("turbulence,order", [("none", 2), ("sa", 2), ("none", 1)])
def test_periodic_layout_reproduces_oracle_products(port_built, tmp_path, ni, turbulence, order):
    c, port = channel(tmp_path, ni=ni, turbulence=turbulence)
    products_match(c, port, C.perturbed_state(c, 12), order)


def test_layout_refuses_what_it_cannot_hold(tmp_path):
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    c.boundaries[3].start = 0
    with pytest.raises(ValueError):
        BJ.partner_masks(c)
    c.boundaries[3].start, c.boundaries[3].face = 1, "top"
    with pytest.raises(ValueError):
        BJ.partner_masks(c)
    ch = C.channel_case(str(tmp_path), "ch", nj=11)
    ch.boundaries[2].face = "bottom"
    with pytest.raises(ValueError):
        BJ.partner_masks(ch)
    ch.boundaries[2].face, ch.boundaries[2].start = "left", 2
    with pytest.raises(ValueError):
        BJ.partner_masks(ch)
    ch.boundaries[2].start = 0
    ch.boundaries.append(C.Boundary("wake", "bottom", 1, 1))
    with pytest.raises(ValueError):
        BJ.partner_masks(ch)


def test_newton_on_the_wake_coupled_jacobian_converges_superlinearly(port_built, tmp_path):
    c, port = naca(tmp_path, ni=61, nj=17, tail=13)
    q, hist = BJ.steady_newton(port, c, C.freestream_state(c))
    assert hist[-1] < 1e-10, hist
    # each of the last steps cuts the residual by more than the one before (the
    # pseudo-time term 1/dt, CFL ~1e5 here, keeps it from being purely
    # quadratic); an inexact Jacobian settles at a fixed factor
    f = hist[-4:][1:] / hist[-4:][:-1]
    assert (np.diff(f) < 0).all() and f[-1] < 0.05, hist[-4:]


def test_newton_on_the_periodic_channel_converges(port_built, tmp_path):
    c, port = channel(tmp_path, nj=21)
    q, hist = BJ.steady_newton(port, c, C.freestream_state(c), cfl=10.0, growth=2.0, tol=1e-11)
    assert hist[-1] < 1e-11, hist  # round-off floor ~2e-12 (1e-13 of the first residual)
    # the steps above the round-off floor cut the residual by 1e-2 and more
    f = hist[-4:][1:] / hist[-4:][:-1]
    assert f[:2].max() < 0.02, hist[-4:]


# ---------------------------------------------------------------------------
# the device source on the host
# ---------------------------------------------------------------------------
GUARD = 64


def guarded(n, fill=0.0, dtype=np.float64):
    """Buffer of n elements inside NaN (or -7) guard bands; returns (whole, view)."""
    g = np.full(n + 2 * GUARD, np.nan if dtype == np.float64 else -7, dtype=dtype)
    g[GUARD:GUARD + n] = fill
    return g, g[GUARD:GUARD + n]


def guards_intact(g):
    a, b = g[:GUARD], g[-GUARD:]
    if g.dtype == np.float64:
        return bool(np.isnan(a).all() and np.isnan(b).all())
    return bool((a == -7).all() and (b == -7).all())


@pytest.fixture(scope="module")
def partner_host(tmp_path_factory):
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path_factory.mktemp("partner_host") / "libpartner_host.so")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wno-unknown-pragmas", "-shared", "-fPIC", "-o", so,
                    os.path.join(here, "partner_kernels_host.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P = ctypes.c_void_p
    I = ctypes.c_int
    lib.ph_masks.argtypes = [I, I, P, I, P, P, P, P]
    lib.ph_seed.argtypes = [I, I, I, I, P, I, I, P]
    lib.ph_extract.argtypes = [I, I, I, I, P, I, I, P, P, P]
    lib.ph_apply.argtypes = [I, I, I, I, I, P, P, P, ctypes.c_double]
    lib.ph_off13.argtypes = [I, I]
    lib.ph_fold.argtypes = [I, I, I, I, P, P]
    D = ctypes.c_double
    lib.ph_strip_cells.argtypes = [I, I, P, P]
    lib.ph_strip_matrix.argtypes = [I, I, I, I, P, P, P, P, D, D, P]
    lib.ph_dense_invert.argtypes = [I, P, P]
    lib.ph_strip_gather.argtypes = [I, I, P, P, P, P, P]
    lib.ph_strip_residual.argtypes = [I, I, I, I, P, P, P, P, D, D, P, P, P]
    lib.ph_strip_update.argtypes = [I, I, P, P, P, P]
    return lib


def host_masks(lib, c):
    from structured_gb300 import abi
    s, keep = abi.make_case_struct(c)
    nic, njc = c.ni - 1, c.nj - 1
    bufs = [guarded(nic, 0, np.int32), guarded(njc, 0, np.int32), guarded(njc, 0, np.int32)]
    on = np.full(3, -1, dtype=np.int32)
    rc = lib.ph_masks(nic, njc, ctypes.cast(s.bcs, ctypes.c_void_p), s.nbc, bufs[0][1].ctypes.data,
                      bufs[1][1].ctypes.data, bufs[2][1].ctypes.data, on.ctypes.data)
    assert all(guards_intact(g) for g, _ in bufs)
    return rc, [m.astype(bool) for _, m in bufs], [bool(v) for v in on]


def test_host_build_of_masks_agrees(partner_host, tmp_path):
    cases = []
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    cases.append(c)
    cases.append(C.channel_case(str(tmp_path), "ch", nj=11))
    for c in cases:
        rc, m, on = host_masks(partner_host, c)
        masks, on_ref = BJ.partner_masks(c)
        assert rc == 0 and on == on_ref
        for f in range(3):
            assert np.array_equal(m[f], masks[f])
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    c.boundaries[3].start = 0
    assert host_masks(partner_host, c)[0] == -6
    c.boundaries[3].start, c.boundaries[3].face = 1, "top"
    assert host_masks(partner_host, c)[0] == -6
    c.boundaries[3].type = "freestream"
    rc, m, on = host_masks(partner_host, c)
    assert rc == 0 and on == [False, False, False]
    ch = C.channel_case(str(tmp_path), "ch", nj=11)
    ch.boundaries[2].face = "top"
    assert host_masks(partner_host, ch)[0] == -6
    ch.boundaries[2].face, ch.boundaries[2].end = "left", 5
    assert host_masks(partner_host, ch)[0] == -6
    ch.boundaries[2].end = -1
    ch.boundaries.append(C.Boundary("wake", "bottom", 1, 1))
    assert host_masks(partner_host, ch)[0] == -6


@pytest.mark.parametrize("which,turbulence,order", [("naca", "none", 2), ("naca", "sa", 1),
                                                     ("channel2", "none", 2), ("channel5", "sa", 2)])
def test_host_build_of_partner_pass_matches_restatement(port_built, partner_host, tmp_path, which, turbulence,
                                                        order):
    """The device source's seeds, extraction and products (run on the host over
    the oracle's JVPs) equal the numpy layout and touch nothing outside their
    buffers."""
    if which == "naca":
        c, port = naca(tmp_path, turbulence)
    else:
        c, port = channel(tmp_path, ni=3 if which == "channel2" else 6, turbulence=turbulence)
    q = C.perturbed_state(c, 13)
    nic, njc, nq = q.shape
    rc, m, on = host_masks(partner_host, c)
    assert rc == 0
    ref = BJ.assemble_partners(port, q, *BJ.partner_masks(c), order)
    zero = np.zeros((nic, njc, len(BJ.OFFSETS), nq, nq))
    rng = np.random.default_rng(5)
    for f in range(3):
        if not on[f]:
            continue
        n = BJ.fam_len(f, nic, njc)
        mask = np.ascontiguousarray(m[f].astype(np.int32))
        gW, W = guarded(n * 4 * nq * nq)
        for k in range(3):
            for comp in range(nq):
                gv, v = guarded(q.size, 0.0)
                partner_host.ph_seed(nq, f, nic, njc, mask.ctypes.data, k, comp, v.ctypes.data)
                assert guards_intact(gv)
                seed = np.ascontiguousarray(v.reshape(q.shape))
                full = port.jvp(q, seed, lhs=(order == 1))
                port.freeze_nonlocal(True)
                frozen = port.jvp(q, seed, lhs=(order == 1))
                port.freeze_nonlocal(False)
                gf, jf = guarded(q.size)
                jf[:] = full.ravel()
                gz, jz = guarded(q.size)
                jz[:] = frozen.ravel()
                partner_host.ph_extract(nq, f, nic, njc, mask.ctypes.data, k, comp, jf.ctypes.data, jz.ctypes.data,
                                        W.ctypes.data)
                assert guards_intact(gf) and guards_intact(gz) and guards_intact(gW)
        assert np.array_equal(W.reshape(ref[f].shape), ref[f])
        only = [None, None, None]
        only[f] = ref[f]
        for trans in (0, 1):
            gx, x = guarded(q.size)
            x[:] = rng.standard_normal(q.size)
            gy, y = guarded(q.size)
            y0 = rng.standard_normal(q.size)
            y[:] = y0
            partner_host.ph_apply(nq, trans, f, nic, njc, W.ctypes.data, x.ctypes.data, y.ctypes.data, -1.5)
            assert guards_intact(gx) and guards_intact(gy) and guards_intact(gW)
            want = y0 - 1.5 * BJ.apply(zero, only, x.reshape(q.shape), trans=bool(trans)).ravel()
            assert np.abs(y - want).max() < 1e-14 * np.abs(want).max()


def test_newton_on_the_channel_example_gives_poiseuille(port_built, tmp_path):
    """The reference's implicit channel example (examples/laminar/channel/
    implicit.inp: 3 x 101, h = 0.1, mu = 1e-2, dp/dx = -0.02592, periodic in x,
    isothermal walls) by Newton through the periodic partner blocks: the
    velocity has the Poiseuille shape (-dp/dx) / (2 mu) y (h - y) up to a
    uniform offset (1 % of u_max on this grid, from the discretisation of the
    walls), and v = 0."""
    from oracle.port import PortCase
    c = C.channel_case(str(tmp_path), "ch", nj=101)
    xv, yv = C.load_grid(c)
    q, hist = BJ.steady_newton(PortCase(c, xv, yv), c, C.freestream_state(c), cfl=10.0, growth=2.0, tol=3e-10)
    assert hist[-1] < 3e-10, hist[-3:]  # round-off floor ~1.2e-10
    u = q[:, :, 1] / q[:, :, 0]
    yc = 0.25 * (yv[:-1, :-1] + yv[1:, :-1] + yv[:-1, 1:] + yv[1:, 1:])
    exact = (-c.dpdx) / (2.0 * c.mu_inf) * yc * (0.1 - yc)
    d = u - exact
    assert d.max() - d.min() < 1e-5 * exact.max()
    assert 0.0 < d.mean() < 0.02 * exact.max()
    assert np.abs(q[:, :, 2] / q[:, :, 0]).max() < 1e-12 * exact.max()


def test_host_build_of_offset_index_matches_the_layout(partner_host):
    for o, (di, dj) in enumerate(BJ.OFFSETS):
        assert partner_host.ph_off13(di, dj) == o
    assert partner_host.ph_off13(2, 1) == -1 and partner_host.ph_off13(-1, 2) == -1


@pytest.mark.parametrize("which,turbulence", [("channel2", "none"), ("channel3", "sa"), ("naca", "none")])
def test_host_build_of_fold_matches_restatement(port_built, partner_host, tmp_path, which, turbulence):
    """Partner blocks inside the ILU(0) pattern are added to the
    preconditioner's blocks, nothing outside the buffer changes.  Two cells
    across every partner is inside; three across only the slots one cell in,
    which are zero at first order; none for the wake cut of this grid."""
    if which == "naca":
        c, port = naca(tmp_path, turbulence)
    else:
        c, port = channel(tmp_path, ni=3 if which == "channel2" else 4, turbulence=turbulence)
    q = C.perturbed_state(c, 17)
    nic, njc, nq = q.shape
    masks, on = BJ.partner_masks(c)
    jac = BJ.assemble_regular(port, q, 1)
    W = BJ.assemble_partners(port, q, masks, on, 1)
    ref = BJ.fold(jac, W)
    gj, flat = guarded(jac.size)
    flat[:] = jac.ravel()
    for f in range(3):
        if on[f]:
            partner_host.ph_fold(nq, f, nic, njc, np.ascontiguousarray(W[f]).ctypes.data, flat.ctypes.data)
    assert guards_intact(gj)
    assert np.array_equal(flat.reshape(jac.shape), ref)
    changed = not np.array_equal(ref, jac)
    assert changed == (which == "channel2")


@pytest.mark.parametrize("turbulence", ["none", "sa"])
def test_host_build_of_wake_strip_level_matches_restatement(port_built, partner_host, tmp_path, turbulence):
    """The wake strip level (rows 0-1 of the columns next to the cut): its
    cells, the dense strip block of P = psd D + sj (J1 + W1) and its inverse,
    and the correction z_S += A_SS^-1 (v - P z)_S, from the device source run on
    the host, against numpy on the oracle's blocks."""
    import scipy.sparse as sp
    c, port = naca(tmp_path, turbulence)
    q = C.perturbed_state(c, 19)
    nic, njc, nq = q.shape
    masks, on = BJ.partner_masks(c)
    jac1 = BJ.assemble_regular(port, q, 1)
    W1 = BJ.assemble_partners(port, q, masks, on, 1)
    mask = np.ascontiguousarray(masks[0].astype(np.int32))
    gcells, cells_buf = guarded(2 * nic, 0, np.int32)
    ns = partner_host.ph_strip_cells(nic, njc, mask.ctypes.data, cells_buf.ctypes.data)
    assert guards_intact(gcells)
    cells = np.ascontiguousarray(cells_buf[:ns])
    want = sorted(i * njc + j for i in range(nic) for j in (0, 1)
                  if masks[0][max(i - 1, 0):i + 2].any())
    assert cells.tolist() == want
    dt = port.dt(q, 30.0)
    # gather
    gjs, jac_s = guarded(ns * 13 * nq * nq)
    gds, dt_s = guarded(ns * nq)
    jflat = np.ascontiguousarray(jac1.ravel())
    dflat = np.ascontiguousarray(dt.ravel())
    partner_host.ph_strip_gather(nq, ns, cells.ctypes.data, jflat.ctypes.data, dflat.ctypes.data,
                                 jac_s.ctypes.data, dt_s.ctypes.data)
    assert guards_intact(gjs) and guards_intact(gds)
    cell_ij = [(int(cl) // njc, int(cl) % njc) for cl in cells]
    assert np.array_equal(jac_s.reshape(ns, 13, nq, nq), np.stack([jac1[i, j] for i, j in cell_ij]))
    assert np.array_equal(dt_s.reshape(ns, nq), np.stack([dt[i, j] for i, j in cell_ij]))
    # strip block of P
    psd, sj = 1.0, -1.0
    P = (sp.diags(psd / dt.ravel()) + sj * BJ.to_sparse(jac1, W1)).tocsr()
    idx = np.array([int(cl) * nq + k for cl in cells for k in range(nq)])
    A_ref = P[idx][:, idx].toarray()
    n = ns * nq
    gA, A = guarded(n * n)
    w1 = np.ascontiguousarray(W1[0])
    partner_host.ph_strip_matrix(nic, njc, nq, ns, cells.ctypes.data, jac_s.ctypes.data, dt_s.ctypes.data,
                                 w1.ctypes.data, psd, sj, A.ctypes.data)
    assert guards_intact(gA)
    assert np.abs(A.reshape(n, n) - A_ref).max() <= 1e-14 * np.abs(A_ref).max()
    gI, inv = guarded(n * n)
    assert partner_host.ph_dense_invert(n, A.ctypes.data, inv.ctypes.data) == 1
    assert guards_intact(gI)
    I_err = np.abs(inv.reshape(n, n) @ A_ref - np.eye(n)).max()
    assert I_err < 1e-9, I_err
    # correction
    rng = np.random.default_rng(8)
    v = np.ascontiguousarray(rng.standard_normal(q.size))
    gz, z = guarded(q.size)
    z0 = rng.standard_normal(q.size)
    z[:] = z0
    gr, res = guarded(n)
    partner_host.ph_strip_residual(nq, nic, njc, ns, cells.ctypes.data, jflat.ctypes.data, w1.ctypes.data,
                                   dflat.ctypes.data, psd, sj, v.ctypes.data, z.ctypes.data, res.ctypes.data)
    assert guards_intact(gr) and guards_intact(gz)
    res_ref = (v - P @ z0)[idx]
    assert np.abs(res - res_ref).max() <= 1e-13 * np.abs(res_ref).max()
    partner_host.ph_strip_update(nq, ns, cells.ctypes.data, inv.ctypes.data, res.ctypes.data, z.ctypes.data)
    assert guards_intact(gz)
    z_ref = z0.copy()
    z_ref[idx] += inv.reshape(n, n) @ res_ref
    assert np.abs(z - z_ref).max() <= 1e-12 * np.abs(z_ref).max()
    # after the correction the strip rows of P z equal v
    assert np.abs((P @ z)[idx] - v[idx]).max() <= 1e-9 * np.abs(v).max()


def test_wake_strip_level_cuts_gmres_iterations(port_built, tmp_path):
    """On a converged C-grid state at high CFL, GMRES preconditioned by block
    ILU(0) of the first-order blocks needs markedly fewer iterations once the
    wake strip correction follows the ILU sweep (the preconditioner of forward
    solves with a wake cut)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    c, port = naca(tmp_path, ni=41, nj=13, tail=11)
    c.lhs_order = 1
    q, _ = BJ.steady_newton(port, c, C.freestream_state(c), tol=1e-8)
    nic, njc, nq = q.shape
    masks, on = BJ.partner_masks(c)
    D = sp.diags(1.0 / port.dt(q, 1e6).ravel())
    A = (D - BJ.to_sparse(BJ.assemble_regular(port, q, 2), BJ.assemble_partners(port, q, masks, on, 2))).tocsc()
    J1 = BJ.assemble_regular(port, q, 1)
    W1 = BJ.assemble_partners(port, q, masks, on, 1)
    P = (D - BJ.to_sparse(J1, W1)).tocsr()
    ilu = BJ.block_ilu0(D - BJ.to_sparse(J1, None), nic, njc, nq)
    cols = set()
    for a in np.nonzero(masks[0])[0]:
        cols |= {a - 1, a, a + 1}
    idx = np.array([(i * njc + j) * nq + k for i in sorted(cols) if 0 <= i < nic for j in (0, 1) for k in range(nq)])
    Ainv = np.linalg.inv(P[idx][:, idx].toarray())

    def strip(v):
        z = ilu(v)
        z[idx] += Ainv @ (v - P @ z)[idx]
        return z

    b = np.random.default_rng(2).standard_normal(A.shape[0])
    counts = []
    for M in (ilu, strip):
        its = []
        spla.gmres(A, b, M=spla.LinearOperator(A.shape, matvec=M), rtol=1e-6, restart=200, maxiter=5,
                   callback=lambda r: its.append(r), callback_type="pr_norm")
        counts.append(len(its))
    assert counts[1] < 0.75 * counts[0], counts
