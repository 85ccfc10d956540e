"""GPU residual parity through the C ABI.

Laminar cases compare with the reference's own calc_residual (golden fixtures
made by tests/golden/make_golden.py from the compiled reference); SA cases
compare with the FP64 restatement in oracle/.  Tolerance: 1e-12 relative per
cell, relative to the cell's sum of |face flux| / V (tests/helpers.rel_err)."""
import numpy as np
import pytest

from helpers import flat_plate, golden_names, load_golden, negative_nut_state, rel_err
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
TOL = 1e-12


def eq_for(case, xv, yv):
    from structured_gb300.solver import EulerEquation
    return EulerEquation(case, xv, yv)


@pytest.mark.parametrize("name", golden_names())
def test_residual_matches_reference(gpu_lib, name):
    c, g = load_golden(name)
    eq = eq_for(c, g["xv"], g["yv"])
    rhs = eq.calc_residual(g["q"])
    assert rel_err(rhs, g["rhs"], g["scale"]) < TOL
    rhs_l = eq.calc_residual(g["q"], lhs=True)
    assert rel_err(rhs_l, g["rhs_lhs"], g["scale_lhs"]) < TOL
    dt = eq.calc_dt(float(g["cfl"]))
    np.testing.assert_allclose(dt, g["dt"], rtol=1e-13)


@pytest.mark.parametrize("law", ["power", "sutherland"])
@pytest.mark.parametrize("shape", [(41, 21), (67, 35)])
def test_sa_residual_matches_oracle(gpu_lib, port_built, tmp_path, law, shape):
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "sa", shape[0], shape[1], turbulence="sa", viscosity_law=law, reynolds=5e6,
                   h1=1e-6, ratio=1.15)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 21)
    beta = 1.0 + 0.2 * np.random.default_rng(4).standard_normal((c.nic, c.njc))
    port = PortCase(c, xv, yv)
    eq = eq_for(c, xv, yv)
    np.testing.assert_allclose(eq.wall_distance(), port.metrics()[3], rtol=1e-14)
    eq.set_beta(beta)
    rhs = eq.calc_residual(q)
    ref = port.residual(q, beta)
    assert rel_err(rhs, ref, port.flux_scale(q, beta)) < TOL


def test_norms_and_skin_friction(gpu_lib, port_built, tmp_path):
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "nrm", 65, 33, turbulence="sa")
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 22)
    eq = eq_for(c, xv, yv)
    rhs = eq.calc_residual(q)
    np.testing.assert_allclose(eq.norms(), np.sqrt((rhs ** 2).sum(axis=(0, 1))), rtol=1e-13)
    cf, J = eq.skin_friction()
    cf_ref, J_ref = PortCase(c, xv, yv).skin_friction(q)
    np.testing.assert_allclose(cf, cf_ref, rtol=1e-10, atol=1e-12 * np.abs(cf_ref).max())
    assert abs(J - J_ref) <= 1e-11 * abs(J_ref)
    # the asynchronous form writes the same Cf and J (device reduction) to device buffers
    import ctypes
    import torch
    cf_d = torch.zeros(c.nic, dtype=torch.float64, device="cuda")
    J_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert eq.lib.st_skin_friction_device(eq.h, ctypes.c_void_p(cf_d.data_ptr()), ctypes.c_void_p(J_d.data_ptr())) == 0
    _, _, stream = eq.device_state()
    torch.cuda.ExternalStream(stream).synchronize()
    assert np.array_equal(cf_d.cpu().numpy(), cf) and float(J_d.item()) == J


def test_uniform_flow_preserved_on_device(gpu_lib, tmp_path):
    c = flat_plate(tmp_path, "uni", 129, 65, top_angle_deg=2.0)
    c.mu_inf = 0.0
    c.boundaries = [C.Boundary("freestream", f, 0, -1) for f in ("bottom", "top", "left", "right")]
    xv, yv = C.load_grid(c)
    eq = eq_for(c, xv, yv)
    r = eq.calc_residual(C.freestream_state(c))
    assert np.abs(r).max() < 1e-11


@pytest.mark.parametrize("turb,flux", [("none", "roe"), ("sa", "roe"), ("none", "ausm"), ("sa", "ausm")])
def test_jvp_matches_oracle(gpu_lib, port_built, tmp_path, turb, flux):
    import torch
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "jvp", 33, 21, turbulence=turb)
    c.flux = flux
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 23)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1))
    vb = rng.standard_normal(q.shape[:2])
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    vt = torch.tensor(v, device="cuda")
    vbt = torch.tensor(vb, device="cuda")
    jv = torch.empty_like(vt)
    eq.jvp_device(vt.data_ptr(), jv.data_ptr(), vbt.data_ptr())
    ref = PortCase(c, xv, yv).jvp(q, v, None, vb)
    scale = np.abs(ref).max(axis=(0, 1))
    assert (np.abs(jv.cpu().numpy() - ref) / scale).max() < 1e-11


def test_full_size_residual_matches_oracle(gpu_lib, port_built, tmp_path):
    """513x257 grid of the residual-throughput workload, SA, seeded 1 %
    perturbations: whole-grid parity."""
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "big", 513, 257, turbulence="sa")
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 20261203)
    eq = eq_for(c, xv, yv)
    port = PortCase(c, xv, yv)
    rhs = eq.calc_residual(q)
    assert rel_err(rhs, port.residual(q), port.flux_scale(q)) < TOL


def test_bad_arguments_raise(gpu_lib, tmp_path):
    from structured_gb300.solver import StructuredError
    c = flat_plate(tmp_path, "bad", 17, 9)
    xv, yv = C.load_grid(c)
    c.boundaries = [C.Boundary("slipwall", "bottom", 0, -1)]
    with pytest.raises(StructuredError):
        eq_for(c, xv, yv)
    c.boundaries = [C.Boundary("freestream", "bottom", 0, 99)]
    with pytest.raises(StructuredError):
        eq_for(c, xv, yv)


def test_sa_neg_residual_and_jvp_match_oracle(gpu_lib, port_built, tmp_path):
    """Negative nu_tilde near the wall: the SA-neg mu_t, diffusion and source
    branches on the device against the oracle (residual and dual JVP)."""
    import torch
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "neg", 45, 29, turbulence="sa", viscosity_law="sutherland", reynolds=5e6, h1=1e-6,
                   ratio=1.15, mach=0.2)
    xv, yv = C.load_grid(c)
    q = negative_nut_state(c, 24)
    assert (q[:, :, 4] < 0).sum() > 50
    rng = np.random.default_rng(6)
    beta = 1.0 + 0.2 * rng.standard_normal((c.nic, c.njc))
    port = PortCase(c, xv, yv)
    eq = eq_for(c, xv, yv)
    eq.set_beta(beta)
    assert rel_err(eq.calc_residual(q), port.residual(q, beta), port.flux_scale(q, beta)) < TOL
    v = rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1))
    vb = rng.standard_normal(q.shape[:2])
    eq.set_state(q)
    vt = torch.tensor(v, device="cuda")
    vbt = torch.tensor(vb, device="cuda")
    jv = torch.empty_like(vt)
    eq.jvp_device(vt.data_ptr(), jv.data_ptr(), vbt.data_ptr())
    ref = port.jvp(q, v, beta, vb)
    scale = np.abs(ref).max(axis=(0, 1))
    assert (np.abs(jv.cpu().numpy() - ref) / scale).max() < 1e-11
