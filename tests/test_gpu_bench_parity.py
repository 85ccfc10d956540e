"""Parity on the residual-throughput workload's own grids: 2049x1025 and
4097x2049 vertices (flat plate, M=0.3, Re=1e6, first cell 1e-4 at ratio 1.08,
seeded 1 % perturbations), the grids the throughput figures are measured on.

- residual (SA and laminar) against the oracle's FP64 restatement, per cell at
  1e-12 of the cell's sum of |face flux| / V (the reference's calc_residual,
  src/model/eulerequation.cpp:202-232, is what the oracle restates);
- the fused residual + adjoint sweep (st_residual_vjp_device, the measured
  step) at 4097x2049: its residual against the oracle at the same bar, and its
  products by the dot-product identity psi.(J v) = (J^T psi).v + (dR/dbeta^T psi).vb
  against the device's forward-mode JVP, to 1e-11 of sum |psi (J v)|."""
import numpy as np
import pytest

from helpers import rel_err
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
TOL = 1e-12
SEED = 20261203


def throughput_case(ni, nj, turbulence):
    import tempfile
    c = C.flat_plate_case(tempfile.gettempdir(), "tp", ni, nj, 0.3, 1e6, 1e-4, 1.08, turbulence=turbulence,
                          write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-4, ratio=1.08)
    return c, g.xv, g.yv, C.perturbed_state(c, SEED)


@pytest.mark.parametrize("turb", ["sa", "none"])
@pytest.mark.parametrize("grid", [(2049, 1025), (4097, 2049)])
def test_residual_matches_oracle_at_throughput_grids(gpu_lib, port_built, grid, turb):
    from oracle.port import PortCase
    from structured_gb300.solver import EulerEquation
    c, xv, yv, q = throughput_case(grid[0], grid[1], turb)
    eq = EulerEquation(c, xv, yv)
    rhs = eq.calc_residual(q)
    eq.close()
    port = PortCase(c, xv, yv)
    err = rel_err(rhs, port.residual(q), port.flux_scale(q))
    print("residual %dx%d %s: max per-cell error %.2e" % (grid[0], grid[1], turb, err))
    assert err < TOL


def test_fused_residual_adjoint_at_4097x2049(gpu_lib, port_built):
    import torch
    from oracle.port import PortCase
    from structured_gb300.solver import EulerEquation
    c, xv, yv, q = throughput_case(4097, 2049, "sa")
    eq = EulerEquation(c, xv, yv)
    eq.set_state(q)
    rng = np.random.default_rng(SEED + 1)
    shape = q.shape
    psi = torch.tensor(rng.standard_normal(shape), device="cuda")
    v = torch.tensor(rng.standard_normal(shape) * np.abs(q).mean(axis=(0, 1)), device="cuda")
    vb = torch.tensor(rng.standard_normal(shape[:2]), device="cuda")
    rhs = torch.empty_like(psi)
    oq = torch.empty_like(psi)
    ob = torch.empty_like(vb)
    eq.residual_vjp_device(psi.data_ptr(), rhs.data_ptr(), oq.data_ptr(), ob.data_ptr())
    jv = torch.empty_like(psi)
    eq.jvp_device(v.data_ptr(), jv.data_ptr(), vb.data_ptr())
    torch.cuda.synchronize()
    lhs = float((psi * jv).sum())
    rhs_dot = float((oq * v).sum() + (ob * vb).sum())
    mag = float((psi * jv).abs().sum())
    dot_err = abs(lhs - rhs_dot) / mag
    r = rhs.cpu().numpy()
    del psi, v, vb, rhs, oq, ob, jv
    eq.close()
    port = PortCase(c, xv, yv)
    err = rel_err(r, port.residual(q), port.flux_scale(q))
    print("fused 4097x2049: residual error %.2e, dot-product identity %.2e" % (err, dot_err))
    assert err < TOL
    assert dot_err <= 1e-11
