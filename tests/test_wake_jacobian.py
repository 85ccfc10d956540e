"""The wake cut in the implicit solver's Jacobian, on CPU against the oracle:
where the cut's distant coupling lands (bc.cpp:224-263 makes the bottom ghost
of column a a copy of cell (nic-1-a, 0)), and the block layout the GPU
assembles (regular 13-point blocks from a frozen-wake colouring plus four wake
partner slots per column, tests/block_jacobian.py) reproducing the oracle's
exact JVP and VJP, and Newton on it converging quadratically on a NACA 0012
C-grid."""
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
    nic, njc = B.shape[:2]
    out = []
    for ri, rj, ci, cj in zip(*np.nonzero(B)):
        if (ci - ri, cj - rj) not in BJ.OFFSETS:
            out.append((int(ri), int(rj), int(ci), int(cj)))
    return out


@pytest.mark.parametrize("turbulence,order", [("none", 2), ("sa", 2), ("none", 1)])
def test_wake_coupling_lands_in_the_four_partner_slots(port_built, tmp_path, turbulence, order):
    c, port = naca(tmp_path, turbulence)
    q = C.perturbed_state(c, 7)
    nic = q.shape[0]
    extra = off_stencil(dense_blocks(port, q, order))
    mask = BJ.wake_columns(c)
    assert extra
    slots = set()
    for ri, rj, ci, cj in extra:
        a = nic - 1 - ci        # the ghost column that copies the column cell
        assert cj == 0 and mask[a], (ri, rj, ci, cj)
        slots.add((rj, ri - a))
    assert slots <= set(BJ.SLOTS)
    if order == 2:
        assert slots == set(BJ.SLOTS)
    # with the ghosts' tangents frozen only the 13-point stencil is left
    port.freeze_wake(True)
    try:
        assert off_stencil(dense_blocks(port, q, order)) == []
    finally:
        port.freeze_wake(False)


@pytest.mark.parametrize("turbulence,flux,order", VARIANTS)
def test_block_layout_reproduces_oracle_products(port_built, tmp_path, turbulence, flux, order):
    c, port = naca(tmp_path, turbulence, flux)
    q = C.perturbed_state(c, 11)
    mask = BJ.wake_columns(c)
    BJ.check_sides(mask)
    jac = BJ.assemble_regular(port, q, order)
    W = BJ.assemble_partners(port, q, mask, order)
    x = np.random.default_rng(3).standard_normal(q.shape)
    jv = port.jvp(q, x, lhs=(order == 1))
    vj, _ = port.vjp(q, x, lhs=(order == 1))
    assert np.abs(BJ.apply(jac, W, x) - jv).max() < 1e-14 * np.abs(jv).max()
    assert np.abs(BJ.apply(jac, W, x, trans=True) - vj).max() < 1e-14 * np.abs(vj).max()
    # the partners carry a first-order share of the product on this grid
    assert np.abs(BJ.apply(jac, None, x) - jv).max() > 1e-3 * np.abs(jv).max()
    A = BJ.to_sparse(jac, W)
    assert np.abs(A @ x.ravel() - jv.ravel()).max() < 1e-14 * np.abs(jv).max()


def test_wake_layout_refuses_what_it_cannot_hold(tmp_path):
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    c.boundaries[3].start = 0
    with pytest.raises(ValueError):
        BJ.wake_columns(c)
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    c.boundaries[3].end = 18        # columns 0..17 and 22..39: five apart
    with pytest.raises(ValueError):
        BJ.check_sides(BJ.wake_columns(c))
    c.boundaries[3].face = "top"
    with pytest.raises(ValueError):
        BJ.wake_columns(c)


def test_newton_on_the_wake_coupled_jacobian_converges_quadratically(port_built, tmp_path):
    c, port = naca(tmp_path, ni=61, nj=17, tail=13)
    q, hist = BJ.steady_newton(port, c, C.freestream_state(c))
    assert hist[-1] < 1e-10, hist
    # superlinear: each of the last steps cuts the residual by more than the
    # one before (the pseudo-time term 1/dt, CFL ~1e5 here, keeps it from
    # being purely quadratic); an inexact Jacobian settles at a fixed factor
    f = hist[-4:][1:] / hist[-4:][:-1]
    assert (np.diff(f) < 0).all() and f[-1] < 0.05, hist[-4:]


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
def wake_host(tmp_path_factory):
    """tests/wake_kernels_host.cpp: the device source of the wake pass built
    for the host."""
    import ctypes
    import os
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path_factory.mktemp("wake_host") / "libwake_host.so")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wno-unknown-pragmas", "-shared", "-fPIC", "-o", so,
                    os.path.join(here, "wake_kernels_host.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P = ctypes.c_void_p
    I = ctypes.c_int
    lib.wh_columns.argtypes = [I, I, P, I, P, P]
    lib.wh_seed.argtypes = [I, I, I, P, I, I, I, P]
    lib.wh_extract.argtypes = [I, I, I, P, I, I, I, P, P]
    lib.wh_apply.argtypes = [I, I, I, I, P, P, P, ctypes.c_double]
    return lib


def host_columns(lib, c):
    import ctypes
    from structured_gb300 import abi
    s, keep = abi.make_case_struct(c)
    nic = c.ni - 1
    gm, m = guarded(nic, 0, np.int32)
    anyw = ctypes.c_int(-1)
    rc = lib.wh_columns(nic, c.nj - 1, ctypes.cast(s.bcs, ctypes.c_void_p), s.nbc, m.ctypes.data,
                        ctypes.byref(anyw))
    assert guards_intact(gm)
    return rc, m.astype(bool), anyw.value


def test_host_build_of_wake_mask_agrees(wake_host, tmp_path):
    c = C.naca0012_case(str(tmp_path), "n", ni=41, nj=9, tail=11, write_files=False)
    rc, m, anyw = host_columns(wake_host, c)
    assert rc == 0 and anyw == 1
    assert np.array_equal(m, BJ.wake_columns(c))
    c.boundaries[3].end = 18
    assert host_columns(wake_host, c)[0] == -6
    c.boundaries[3].end, c.boundaries[3].start = 10, 0
    assert host_columns(wake_host, c)[0] == -6
    c.boundaries[3].start, c.boundaries[3].face = 1, "top"
    assert host_columns(wake_host, c)[0] == -6
    c.boundaries[3].type = "freestream"
    rc, m, anyw = host_columns(wake_host, c)
    assert rc == 0 and anyw == 0 and not m.any()
    ch = C.channel_case(str(tmp_path), "ch", nj=11)
    assert host_columns(wake_host, ch)[0] == -6          # periodic


@pytest.mark.parametrize("turbulence,order", [("none", 2), ("sa", 2), ("sa", 1)])
def test_host_build_of_wake_pass_matches_restatement(port_built, wake_host, tmp_path, turbulence, order):
    """The device source's seeds, extraction and products (run on the host over
    the oracle's JVPs) equal the numpy layout, and touch nothing outside their
    buffers."""
    c, port = naca(tmp_path, turbulence)
    q = C.perturbed_state(c, 13)
    nic, njc, nq = q.shape
    rc, m, _ = host_columns(wake_host, c)
    assert rc == 0
    mask = np.ascontiguousarray(m.astype(np.int32))
    gW, W = guarded(nic * 4 * nq * nq)
    for side in (0, 1):
        for k in range(3):
            for comp in range(nq):
                gv, v = guarded(q.size, 5.0)
                wake_host.wh_seed(nq, nic, njc, mask.ctypes.data, side, k, comp, v.ctypes.data)
                assert guards_intact(gv)
                jv = port.jvp(q, np.ascontiguousarray(v.reshape(q.shape)), lhs=(order == 1))
                gj, jvb = guarded(q.size)
                jvb[:] = jv.ravel()
                wake_host.wh_extract(nq, nic, njc, mask.ctypes.data, side, k, comp, jvb.ctypes.data, W.ctypes.data)
                assert guards_intact(gj) and guards_intact(gW)
    ref = BJ.assemble_partners(port, q, BJ.wake_columns(c), order)
    assert np.array_equal(W.reshape(ref.shape), ref)
    zero = np.zeros((nic, njc, len(BJ.OFFSETS), nq, nq))
    rng = np.random.default_rng(5)
    for trans in (0, 1):
        gx, x = guarded(q.size)
        x[:] = rng.standard_normal(q.size)
        gy, y = guarded(q.size)
        y0 = rng.standard_normal(q.size)
        y[:] = y0
        wake_host.wh_apply(nq, trans, nic, njc, W.ctypes.data, x.ctypes.data, y.ctypes.data, -1.5)
        assert guards_intact(gx) and guards_intact(gy) and guards_intact(gW)
        want = y0 - 1.5 * BJ.apply(zero, ref, x.reshape(q.shape), trans=bool(trans)).ravel()
        assert np.abs(y - want).max() < 1e-14 * np.abs(want).max()
