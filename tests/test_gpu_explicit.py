"""Explicit marching on the GPU (Solver::step's forward_euler and rk4_jameson,
src/solver/solver.cpp:12-26, 103-116): trajectories against the same stages
computed from the oracle's residual and time step, and the channel's
known answer (plane Poiseuille flow)."""
import numpy as np
import pytest

from helpers import flat_plate
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu


def oracle_march(port, q, cfl, steps, scheme):
    q = q.copy()
    for _ in range(steps):
        dt = port.dt(q, cfl).reshape(q.shape)
        if scheme == "forward_euler":
            q = q + port.residual(q) * dt
        else:
            qt = q.copy()
            for s in range(4):
                qt = q + port.residual(qt) * dt / (4.0 - s)
            q = qt
    return q


@pytest.mark.parametrize("scheme", ["forward_euler", "rk4_jameson"])
@pytest.mark.parametrize("which", ["channel", "plate"])
def test_explicit_trajectory_matches_oracle(gpu_lib, port_built, tmp_path, scheme, which):
    from oracle.port import PortCase
    from structured_gb300.solver import EulerEquation
    if which == "channel":
        c = C.channel_case(str(tmp_path), "ch", nj=21)
        cfl = 0.5
    else:
        c = flat_plate(tmp_path, "fp", 33, 21)
        cfl = 0.5
    xv, yv = C.load_grid(c)
    q0 = C.perturbed_state(c, 61)
    eq = EulerEquation(c, xv, yv)
    eq.set_state(q0)
    done, hist = eq.explicit_solve(scheme, cfl=cfl, steps=20, check_every=10)
    assert done == 20 and hist.shape[0] == 2
    q_gpu = eq.get_state()
    q_ref = oracle_march(PortCase(c, xv, yv), q0, cfl, 20, scheme)
    d_ref = q_ref - q0
    scale = np.abs(d_ref).max(axis=(0, 1)) + 1e-300
    assert (np.abs((q_gpu - q0) - d_ref).max(axis=(0, 1)) / scale).max() < 1e-9


def oracle_steady(port, q, iters=20):
    """Steady state of the oracle by Newton with its exact dense Jacobian
    (columns from the dual-number JVP); small grids only."""
    n = q.size
    for _ in range(iters):
        R = port.residual(q)
        if np.abs(R).max() < 1e-13:
            break
        J = np.empty((n, n))
        for col in range(n):
            v = np.zeros(n)
            v[col] = 1.0
            J[:, col] = port.jvp(q, v.reshape(q.shape)).ravel()
        q = q + np.linalg.solve(-J, R.ravel()).reshape(q.shape)
    return q


def test_channel_reaches_poiseuille(gpu_lib, port_built, tmp_path):
    """Pressure-driven channel (h = 0.1, mu = 1e-2, dp/dx = -0.02592, periodic
    in x, isothermal walls), RK4 from freestream to a 1e-10 residual:
    - the velocity profile has the Poiseuille shape (-dp/dx) / (2 mu) y (h - y)
      exactly, up to a uniform offset (2.4 % of u_max on this grid) that the
      reference's discretisation of the walls carries;
    - it equals the oracle's steady state (Newton on the FP64 restatement).
    CFL 0.5: the time-step formula counts 2 mu / l^2 only, and the thermal
    diffusivity (gamma / Pr = 2x) puts RK4 past its real-axis limit near 0.8."""
    from oracle.port import PortCase
    from structured_gb300.solver import EulerEquation
    h = 0.1
    c = C.channel_case(str(tmp_path), "pois", nj=41, height=h, dx=h / 20)
    xv, yv = C.load_grid(c)
    eq = EulerEquation(c, xv, yv)
    q0 = C.freestream_state(c)
    eq.set_state(q0)
    done, hist = eq.explicit_solve("rk4_jameson", cfl=0.5, steps=40000, tolerance=1e-10, check_every=200)
    q = eq.get_state()
    u = q[:, :, 1] / q[:, :, 0]
    yc = 0.25 * (yv[:-1, :-1] + yv[1:, :-1] + yv[:-1, 1:] + yv[1:, 1:])
    exact = (-c.dpdx) / (2.0 * c.mu_inf) * yc * (h - yc)
    umax = exact.max()
    d = u - exact
    assert d.max() - d.min() < 1e-4 * umax, (done, d.min() / umax, d.max() / umax)
    assert abs(d.mean()) < 0.03 * umax
    qo = oracle_steady(PortCase(c, xv, yv), q0)
    uo = qo[:, :, 1] / qo[:, :, 0]
    assert np.abs(u - uo).max() < 1e-6 * umax
    assert np.abs(q[:, :, 2] / q[:, :, 0]).max() < 1e-6 * umax
