"""Implicit solve on the GPU: block Jacobian, GMRES + line preconditioner,
pseudo-time Newton, objective gradient, adjoint solve and dJ/dbeta."""
import numpy as np
import pytest

from helpers import flat_plate
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu


def eq_for(case, xv, yv):
    from structured_gb300.solver import EulerEquation
    return EulerEquation(case, xv, yv)


def rel(a, b):
    return float(np.abs(a - b).max() / (np.abs(b).max() + 1e-300))


@pytest.mark.parametrize("turb", ["none", "sa"])
@pytest.mark.parametrize("lhs", [False, True])
def test_block_jacobian_matches_jvp_and_vjp(gpu_lib, tmp_path, turb, lhs):
    import torch
    c = flat_plate(tmp_path, "jac", 37, 23, turbulence=turb, lhs_order=1)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 70)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    eq.jacobian_assemble(lhs=lhs)
    rng = np.random.default_rng(71)
    v = torch.tensor(rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1)), device="cuda")
    jv_ref = torch.empty_like(v)
    eq.jvp_device(v.data_ptr(), jv_ref.data_ptr(), None, lhs=lhs)
    jv = torch.empty_like(v)
    eq.jacobian_apply_device(v.data_ptr(), jv.data_ptr())
    torch.cuda.synchronize()
    assert rel(jv.cpu().numpy(), jv_ref.cpu().numpy()) < 1e-12
    psi = rng.standard_normal(q.shape)
    oq, _ = eq.vjp(psi, lhs=lhs)
    pt = torch.tensor(psi, device="cuda")
    jt = torch.empty_like(pt)
    eq.jacobian_apply_device(pt.data_ptr(), jt.data_ptr(), transpose=True)
    torch.cuda.synchronize()
    assert rel(jt.cpu().numpy(), oq) < 1e-11


@pytest.mark.parametrize("transpose", [False, True])
def test_linear_solve_reaches_tolerance(gpu_lib, tmp_path, transpose):
    import torch
    c = flat_plate(tmp_path, "lin", 49, 33, turbulence="sa")
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 72)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    eq.jacobian_assemble(lhs=True)
    cfl = 50.0
    dt = eq.calc_dt(cfl)
    b = torch.tensor(np.random.default_rng(73).standard_normal(q.shape), device="cuda")
    x = torch.zeros_like(b)
    st = eq.linear_solve_device(cfl, b.data_ptr(), x.data_ptr(), transpose=transpose, m=60, maxit=600, rtol=1e-10)
    assert st.converged == 1
    jx = torch.empty_like(x)
    eq.jacobian_apply_device(x.data_ptr(), jx.data_ptr(), transpose=transpose)
    torch.cuda.synchronize()
    ax = x.cpu().numpy() / dt - jx.cpu().numpy()
    bb = b.cpu().numpy()
    assert np.linalg.norm(ax - bb) <= 1e-9 * np.linalg.norm(bb)


def test_laminar_plate_converges_to_blasius(gpu_lib, tmp_path):
    """Laminar flat plate (129x65, M=0.2, Re_L=1e5) to a 1e-10 relative residual
    drop; mid-plate Cf within 5 % of Blasius 0.664/sqrt(Re_x)."""
    from structured_gb300 import workloads
    from structured_gb300.solver import Solver
    c = workloads.laminar_plate(str(tmp_path))
    xv, yv = C.load_grid(c)
    eq = eq_for(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    ok, hist = Solver(eq, max_steps=200, cfl=5.0, cfl_ramp=1, cfl_ramp_iteration=3, cfl_ramp_exponent=1.3,
                      rel_tolerance=1e-10, krylov_rtol=1e-4).solve()
    assert ok, hist[-5:]
    cf, J = eq.skin_friction()
    xw = 0.5 * (xv[:-1, 0] + xv[1:, 0]) - xv[c.i_le, 0]
    sel = (xw > 0.25) & (xw < 0.75)
    blasius = 0.664 / np.sqrt(1e5 * xw[sel])
    assert np.abs(cf[sel] / blasius - 1.0).max() < 0.05


def test_adjoint_gradient_matches_finite_differences(gpu_lib, tmp_path):
    """SA plate: dJ/dbeta from the adjoint solve vs central differences of
    converged solves (step 1e-6) on seeded cells, to 1e-5 relative above the
    difference quotient's round-off floor."""
    import torch
    from structured_gb300.solver import Solver
    c = flat_plate(tmp_path, "fd", 49, 41, turbulence="sa", mach=0.2, reynolds=1e6, h1=1e-5, ratio=1.12,
                   lhs_order=2)
    xv, yv = C.load_grid(c)
    eq = eq_for(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    params = dict(max_steps=300, cfl=5.0, cfl_growth=2.0, rel_tolerance=1e-12, krylov_rtol=1e-6)
    ok, hist = Solver(eq, **params).solve()
    assert ok, hist[-5:]
    r0 = hist[0, 3:].max()
    q0 = eq.get_state()
    beta0 = np.ones((c.nic, c.njc))
    _, J0 = eq.skin_friction()
    # adjoint: (dR/dQ)^T psi = dJ/dQ ;  dJ/dbeta = -(dR/dbeta)^T psi
    w = np.zeros(c.nic)
    for i in range(max(c.i_le, 0), c.nic):
        w[i] = xv[i + 1, 0] - xv[i, 0]
    g = torch.zeros(q0.shape, dtype=torch.float64, device="cuda")
    eq.cf_gradient_device(w, g.data_ptr())
    psi = torch.zeros_like(g)
    st = eq.adjoint_solve_device(g.data_ptr(), psi.data_ptr(), rtol=1e-12)
    assert st.converged == 1
    oq = torch.empty_like(g)
    ob = torch.empty((c.nic, c.njc), dtype=torch.float64, device="cuda")
    eq.vjp_device(psi.data_ptr(), oq.data_ptr(), ob.data_ptr())
    torch.cuda.synchronize()
    grad = -ob.cpu().numpy()
    # seeded cells among those whose gradient carries signal (>= 1 % of the largest)
    rng = np.random.default_rng(74)
    cand = np.argwhere(np.abs(grad) >= 1e-2 * np.abs(grad).max())
    cells = [tuple(int(t) for t in cand[k]) for k in rng.choice(len(cand), size=4, replace=False)]
    h = 1e-6
    for (i, j) in cells:
        Js = []
        for sgn in (1.0, -1.0):
            b = beta0.copy()
            b[i, j] += sgn * h
            eq.set_beta(b)
            eq.set_state(q0)
            ok, hs = Solver(eq, **dict(params, cfl=1e12, cfl_growth=1.0, max_steps=20, min_steps=3, rel_tolerance=0.0,
                                        tolerance=1e-12 * r0, krylov_rtol=1e-12)).solve()
            assert ok, hs
            Js.append(eq.skin_friction()[1])
        fd = (Js[0] - Js[1]) / (2 * h)
        # round-off floor of the difference quotient: J to ~200 ulp over 2h
        floor = 200 * np.finfo(float).eps * abs(J0) / (2 * h)
        assert abs(fd - grad[i, j]) <= 1e-5 * abs(grad[i, j]) + floor, (i, j, fd, grad[i, j], floor)
    eq.set_beta(beta0)


def test_turbulent_plate_converges(gpu_lib, tmp_path):
    """SA plate with a 1e-7 first cell (y+ < 1) from freestream: the robust
    Newton strategy (step rejection, CFL growth, density damping, SA floor)
    reaches a 1e-11 relative residual."""
    from structured_gb300 import workloads
    from structured_gb300.solver import Solver
    c = workloads.turbulent_plate(str(tmp_path), 69, 49)
    xv, yv = C.load_grid(c)
    eq = eq_for(c, xv, yv)
    eq.set_state(C.freestream_state(c))
    ok, hist = Solver(eq, max_steps=200, cfl=5.0, cfl_growth=2.0, rel_tolerance=1e-11, krylov_rtol=1e-4).solve()
    assert ok, hist[-5:]
    cf, J = eq.skin_friction()
    assert 1e-3 < J < 1e-2
