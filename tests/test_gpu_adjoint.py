"""Hand-written discrete adjoint on the GPU: (dR/dQ)^T psi and (dR/dbeta)^T psi.

Checked against the oracle's exact transposed products (coloured dual-number
JVPs of the FP64 restatement, which is pinned to the reference's residual), and
by the dot-product identity psi . (J v) = (J^T psi) . v with the GPU's own
forward-mode JVP at full size."""
import numpy as np
import pytest

from helpers import flat_plate, golden_names, load_golden, negative_nut_state
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
TOL = 1e-10


def close(a, b, tol=TOL):
    """max over components of max|a-b| / max|b|."""
    a = a.reshape(-1, a.shape[-1]) if a.ndim == 3 else a.reshape(-1, 1)
    b = b.reshape(a.shape)
    scale = np.abs(b).max(axis=0) + 1e-300
    return float((np.abs(a - b).max(axis=0) / scale).max())


def eq_for(case, xv, yv):
    from structured_gb300.solver import EulerEquation
    return EulerEquation(case, xv, yv)


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("lhs", [False, True])
def test_vjp_matches_oracle_on_fixtures(gpu_lib, port_built, name, lhs):
    from oracle.port import PortCase
    c, g = load_golden(name)
    eq = eq_for(c, g["xv"], g["yv"])
    port = PortCase(c, g["xv"], g["yv"])
    eq.set_state(g["q"])
    psi = np.random.default_rng(31).standard_normal(g["q"].shape)
    oq, ob = eq.vjp(psi, lhs=lhs)
    rq, rb = port.vjp(g["q"], psi, lhs=lhs)
    assert close(oq, rq) < TOL
    assert np.abs(ob).max() == 0.0


@pytest.mark.parametrize("law", ["power", "sutherland"])
@pytest.mark.parametrize("top", [0.0, 2.0])
def test_sa_vjp_matches_oracle(gpu_lib, port_built, tmp_path, law, top):
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "sav", 45, 29, turbulence="sa", viscosity_law=law, reynolds=5e6, h1=1e-6,
                   ratio=1.15, top_angle_deg=top, mach=0.2)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 41)
    rng = np.random.default_rng(42)
    beta = 1.0 + 0.2 * rng.standard_normal((c.nic, c.njc))
    psi = rng.standard_normal(q.shape)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    eq.set_beta(beta)
    oq, ob = eq.vjp(psi)
    rq, rb = PortCase(c, xv, yv).vjp(q, psi, beta)
    assert close(oq, rq) < TOL
    assert close(ob, rb) < TOL


@pytest.mark.parametrize("turb", ["none", "sa"])
def test_dot_product_identity_full_size(gpu_lib, tmp_path, turb):
    """513x257 grid of the throughput workload: psi.(Jv) == (J^T psi).v with the
    device JVP (dual numbers) and the hand-written VJP."""
    import torch
    c = flat_plate(tmp_path, "dot", 513, 257, turbulence=turb)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 20261203)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    rng = np.random.default_rng(43)
    v = torch.tensor(rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1)), device="cuda")
    vb = torch.tensor(rng.standard_normal((c.nic, c.njc)), device="cuda")
    psi = torch.tensor(rng.standard_normal(q.shape), device="cuda")
    jv = torch.empty_like(v)
    eq.jvp_device(v.data_ptr(), jv.data_ptr(), vb.data_ptr())
    oq = torch.empty_like(v)
    ob = torch.empty_like(vb)
    eq.vjp_device(psi.data_ptr(), oq.data_ptr(), ob.data_ptr())
    torch.cuda.synchronize()
    lhs = float((psi * jv).sum())
    rhs = float((oq * v).sum() + (ob * vb).sum())
    mag = float((psi * jv).abs().sum())
    assert abs(lhs - rhs) <= 1e-11 * mag


def test_vjp_is_deterministic(gpu_lib, tmp_path):
    c = flat_plate(tmp_path, "det", 129, 65, turbulence="sa")
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 44)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    psi = np.random.default_rng(45).standard_normal(q.shape)
    a = eq.vjp(psi)
    b = eq.vjp(psi)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("turb", ["none", "sa"])
def test_fused_residual_adjoint_matches_separate_calls(gpu_lib, port_built, tmp_path, turb):
    """st_residual_vjp (one sweep) gives the same residual as st_residual and
    the same products as st_vjp."""
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "fused", 67, 41, turbulence=turb)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 46)
    eq = eq_for(c, xv, yv)
    psi = np.random.default_rng(47).standard_normal(q.shape)
    rhs_a = eq.calc_residual(q)
    oq_a, ob_a = eq.vjp(psi)
    rhs_b, oq_b, ob_b = eq.residual_vjp(psi)
    port = PortCase(c, xv, yv)
    from helpers import rel_err
    assert rel_err(rhs_b, rhs_a, port.flux_scale(q)) < 1e-13
    assert rel_err(rhs_b, port.residual(q), port.flux_scale(q)) < 1e-12
    assert np.array_equal(oq_a, oq_b) and np.array_equal(ob_a, ob_b)


def test_sa_neg_vjp_matches_oracle(gpu_lib, port_built, tmp_path):
    """The hand-written reverse of the SA-neg branches (mu_t = 0, rho nu_tilde
    f_n in the diffusion coefficient, the negative source) against the
    oracle's exact transposed products."""
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "negv", 45, 29, turbulence="sa", viscosity_law="sutherland", reynolds=5e6, h1=1e-6,
                   ratio=1.15, mach=0.2)
    xv, yv = C.load_grid(c)
    q = negative_nut_state(c, 47)
    rng = np.random.default_rng(48)
    beta = 1.0 + 0.2 * rng.standard_normal((c.nic, c.njc))
    psi = rng.standard_normal(q.shape)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    eq.set_beta(beta)
    oq, ob = eq.vjp(psi)
    rq, rb = PortCase(c, xv, yv).vjp(q, psi, beta)
    assert close(oq, rq) < TOL
    assert close(ob, rb) < TOL


@pytest.mark.parametrize("mach", [0.3, 1.6])
def test_ausm_sa_vjp_matches_oracle_and_jvp(gpu_lib, port_built, tmp_path, mach):
    """The hand-written reverse of the AUSM flux (the reference's default,
    src/model/flux.cpp:148-224) with SA, subsonic and supersonic (both branches
    of the split Mach numbers and pressures): against the oracle's exact
    transposed products, and by the dot-product identity with the device JVP."""
    import torch
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "ausm", 45, 29, turbulence="sa", reynolds=5e6, h1=1e-6, ratio=1.15, mach=mach)
    c.flux = "ausm"
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 48)
    rng = np.random.default_rng(49)
    beta = 1.0 + 0.2 * rng.standard_normal((c.nic, c.njc))
    psi = rng.standard_normal(q.shape)
    eq = eq_for(c, xv, yv)
    eq.set_state(q)
    eq.set_beta(beta)
    oq, ob = eq.vjp(psi)
    rq, rb = PortCase(c, xv, yv).vjp(q, psi, beta)
    assert close(oq, rq) < TOL
    assert close(ob, rb) < TOL
    v = torch.tensor(rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1)), device="cuda")
    vb = torch.tensor(rng.standard_normal((c.nic, c.njc)), device="cuda")
    jv = torch.empty_like(v)
    eq.jvp_device(v.data_ptr(), jv.data_ptr(), vb.data_ptr())
    torch.cuda.synchronize()
    lhs = float((torch.tensor(psi, device="cuda") * jv).sum())
    rhs = float((torch.tensor(oq, device="cuda") * v).sum() + (torch.tensor(ob, device="cuda") * vb).sum())
    mag = float((torch.tensor(psi, device="cuda") * jv).abs().sum())
    assert abs(lhs - rhs) <= 1e-11 * mag
