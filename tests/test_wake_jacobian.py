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
