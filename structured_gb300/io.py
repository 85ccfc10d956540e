"""The reference's output files, written from a GB300 solution.

Restated from IOManager (src/utils/io.cpp) so that a run here leaves the same
files a run of the reference leaves, in the same formats:

  <label>.out      restart: q[nic][njc][nq+ntrans] raw FP64 (io.cpp:135-180)
  <label>.npz      xc, yc, q (first 4 components), rho, u, v, p, T (io.cpp:106-131)
  <label>.tec      tecplot point format, cell centres and q (io.cpp:50-103)
  <label>.surface  x, Cp, Cf per wall face; Cl/Cd returned (io.cpp:182-255)
  <label>.history  the convergence log line of Solver::step (solver.cpp:38,141,189)

Numbers are printed as C++ streams print a double by default (printf %g);
primitives follow FluidModel::primvars (src/model/fluid.cpp:48-64) operation
for operation.  Two properties of the reference are kept: the surface loop runs
over faces [tail-1, tail-1+nb), nb = ni - 2 tail + 1 (mesh.cpp:349-350), so a
case with tail = 0 writes an empty surface file; Cp averages the pressures of
the first two cell rows (io.cpp:219).  The ten q_aux columns of the tecplot
file are never set by the reference; they are written as 0 here.  The npz
`q` holds the four flow components; with SA the reference passes its
5-component buffer under a 4-component shape, which mixes components.
"""
from __future__ import annotations

import math

import numpy as np

GAMMA = 1.4


def cell_centres(xv: np.ndarray, yv: np.ndarray):
    """Mesh::calc_metrics centroids (mesh.cpp:199-200)."""
    xc = 0.25 * (xv[:-1, :-1] + xv[1:, :-1] + xv[:-1, 1:] + xv[1:, 1:])
    yc = 0.25 * (yv[:-1, :-1] + yv[1:, :-1] + yv[:-1, 1:] + yv[1:, 1:])
    return xc, yc


def primitives(q: np.ndarray, case):
    """rho, u, v, p, T of FluidModel::primvars; R = p_ref / rho_ref / T_ref."""
    R = case.p_inf / case.rho_inf / case.T_inf
    rho = q[:, :, 0]
    u = q[:, :, 1] / rho
    v = q[:, :, 2] / rho
    p = (q[:, :, 3] - 0.5 * rho * (u * u + v * v)) * (GAMMA - 1.0)
    T = p / rho / R
    return rho.copy(), u, v, p, T


def write_restart(path: str, q: np.ndarray) -> None:
    np.ascontiguousarray(q, dtype=np.float64).tofile(path)


def read_restart(path: str, nic: int, njc: int, nq: int) -> np.ndarray:
    """IOManager::read_restart: the file must hold exactly nic*njc*nq doubles."""
    q = np.fromfile(path, dtype=np.float64)
    if q.size != nic * njc * nq:
        raise ValueError("restart %s holds %d values, expected %d" % (path, q.size, nic * njc * nq))
    return q.reshape(nic, njc, nq)


def write_npz(path: str, xc, yc, q, prim) -> None:
    rho, u, v, p, T = prim
    np.savez(path, xc=xc, yc=yc, q=np.ascontiguousarray(q[:, :, :4]), rho=rho, u=u, v=v, p=p, T=T)


def _g(x: float) -> str:
    return "%g" % x


def write_tecplot(path: str, xc, yc, q, nq: int = 4, naux: int = 10) -> None:
    """IOManager::write_tecplot: header, `zone i=, j=, f=point`, rows j-major."""
    names = ["rho", "rhou", "rhov", "rhoE"][:nq]
    ntrans = q.shape[2] - nq
    nic, njc = xc.shape
    head = 'variables = "x" "y"' + "".join(' "%s"' % n for n in names) + ' "psi_0"' * ntrans + \
        "".join(' "q_aux_%d"' % k for k in range(naux))
    lines = ['title = "Solution"', head, "zone i=%d, j=%d, f=point" % (nic, njc)]
    aux = "0 " * naux
    for j in range(njc):
        for i in range(nic):
            vals = [xc[i, j], yc[i, j]] + list(q[i, j, :nq]) + list(q[i, j, nq:])
            lines.append("".join(_g(v) + " " for v in vals) + aux)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_surface(path: str, case, xv, yv, q, wall_grad) -> dict:
    """IOManager::write_surface.  wall_grad [nic][4]: (u_x, u_y, v_x, v_y) at
    the j = 0 faces (the reference's grad_u_eta / grad_v_eta row 0; from
    st_wall_gradients here).  Returns the pressure, viscous and total Cl, Cd
    the reference logs."""
    xc, _ = cell_centres(xv, yv)
    _, _, _, p, _ = primitives(q, case)
    ni = xv.shape[0]
    j1 = case.tail - 1
    nb = ni - 2 * case.tail + 1
    qinf = 0.5 * case.rho_inf * (case.u_inf * case.u_inf + case.v_inf * case.v_inf)
    mu = case.mu_inf
    fn_p = fc_p = fn_v = fc_v = 0.0
    lines = []
    if j1 >= 0:  # the reference's unsigned start wraps for tail = 0 and writes nothing
        for i in range(j1, j1 + nb):
            cp = (0.5 * (p[i, 0] + p[i, 1]) - case.p_inf) / qinf
            ux, uy, vx, vy = (float(t) for t in wall_grad[i])
            tau = mu * (uy - vx) / qinf
            lines.append("%s %s %s" % (_g(xc[i, 0]), _g(cp), _g(tau)))
            dx = xv[i + 1, 0] - xv[i, 0]
            dy = yv[i + 1, 0] - yv[i, 0]
            fn_p = fn_p - cp * dx
            fc_p = fc_p + cp * dy
            sfdiv = 2.0 / 3.0 * (ux + vy)
            sxx = mu * (2.0 * ux - sfdiv) / qinf
            syy = mu * (2.0 * vy - sfdiv) / qinf
            fn_v = fn_v - tau * dy + syy * dx
            fc_v = fc_v + tau * dx - sxx * dy
    with open(path, "w") as f:
        f.write("".join(line + "\n" for line in lines))
    aoa = case.aoa * math.pi / 180.0
    ca, sa = math.cos(aoa), math.sin(aoa)
    out = {"cl_pressure": -fc_p * sa + fn_p * ca, "cd_pressure": fc_p * ca + fn_p * sa,
           "cl_viscous": -fc_v * sa + fn_v * ca, "cd_viscous": fc_v * ca + fn_v * sa}
    out["cl"] = out["cl_viscous"] + out["cl_pressure"]
    out["cd"] = out["cd_viscous"] + out["cd_pressure"]
    return out


def history_line(step: int, t: float, wall: float, cfl: float, norms) -> str:
    """The convergence log line of Solver::step: step, time, wall time, CFL and
    the first four residual norms."""
    n = list(norms)[:4] + [0.0] * max(0, 4 - len(norms))
    return "%08d %.2e %.2e %.2e %.2e %.2e %.2e %.2e" % (step, t, wall, cfl, n[0], n[1], n[2], n[3])


def write_history(path: str, rows) -> None:
    """rows: (step, t, wall, cfl, norms) tuples, one line each."""
    with open(path, "w") as f:
        for r in rows:
            f.write(history_line(*r) + "\n")


def write_outputs(eq, label: str) -> dict:
    """IOManager::write for the solution held by an EulerEquation: the four
    files under `label`; returns the surface Cl/Cd."""
    c = eq.case
    q = eq.get_state()
    xc, yc = cell_centres(eq._xv, eq._yv)
    prim = primitives(q, c)
    write_tecplot(label + ".tec", xc, yc, q)
    write_npz(label + ".npz", xc, yc, q, prim)
    write_restart(label + ".out", q)
    return write_surface(label + ".surface", c, eq._xv, eq._yv, q, eq.wall_gradients())
