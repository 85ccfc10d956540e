"""CPU checks of the oracle (the FP64 restatement) and the case setup."""
import os

import numpy as np
import pytest

from helpers import flat_plate, golden_names, load_golden, negative_nut_state, rel_err
from structured_gb300 import case as C


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden(port_built, name):
    """The restatement reproduces the reference's calc_residual / calc_dt on
    the committed fixtures (bit-exact on x86; 1e-13 relative allows for FMA
    contraction in other host compilers)."""
    from oracle.port import PortCase
    c, g = load_golden(name)
    p = PortCase(c, g["xv"], g["yv"])
    rhs = p.residual(g["q"])
    assert rel_err(rhs, g["rhs"], g["scale"]) < 1e-13
    rhs_l = p.residual(g["q"], lhs=True)
    assert rel_err(rhs_l, g["rhs_lhs"], g["scale_lhs"]) < 1e-13
    dt = p.dt(g["q"], float(g["cfl"]))
    np.testing.assert_allclose(dt, g["dt"], rtol=1e-14)


def test_port_matches_reference_live(port_built, ref_available, tmp_path):
    if not ref_available:
        pytest.skip("reference sources not mounted here")
    from oracle.port import PortCase
    from oracle.refcase import RefCase
    c = flat_plate(tmp_path, "live", 49, 25)
    q = C.perturbed_state(c, 3)
    ref = RefCase(os.path.join(str(tmp_path), "live.inp"))
    p = PortCase(c)
    assert rel_err(p.residual(q), ref.residual(q), p.flux_scale(q)) < 1e-13


@pytest.mark.parametrize("turb", ["none", "sa", "sa_neg", "ausm"])
def test_port_jvp_matches_central_fd(port_built, tmp_path, turb):
    """sa_neg: a patch of negative nu_tilde (the SA-neg branches); ausm: the
    AUSM flux (laminar)."""
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "jvp_" + turb, 25, 17, turbulence={"sa": "sa", "sa_neg": "sa"}.get(turb, "none"))
    if turb == "ausm":
        c.flux = "ausm"
    p = PortCase(c)
    q = negative_nut_state(c, 5) if turb == "sa_neg" else C.perturbed_state(c, 5)
    rng = np.random.default_rng(1)
    v = rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1))
    beta = 1.0 + 0.1 * rng.standard_normal(q.shape[:2])
    vb = rng.standard_normal(q.shape[:2])
    jv = p.jvp(q, v, beta, vb)
    h = 1e-6
    fd = (p.residual(q + h * v, beta + h * vb) - p.residual(q - h * v, beta - h * vb)) / (2 * h)
    assert np.abs(jv - fd).max() <= 1e-8 * np.abs(fd).max()


@pytest.mark.parametrize("turb", ["none", "sa"])
def test_port_vjp_is_transpose_of_jvp(port_built, tmp_path, turb):
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "vjp_" + turb, 23, 15, turbulence=turb)
    p = PortCase(c)
    q = C.perturbed_state(c, 6)
    rng = np.random.default_rng(2)
    beta = 1.0 + 0.1 * rng.standard_normal(q.shape[:2])
    v = rng.standard_normal(q.shape)
    vb = rng.standard_normal(q.shape[:2])
    psi = rng.standard_normal(q.shape)
    oq, ob = p.vjp(q, psi, beta)
    lhs = float((psi * p.jvp(q, v, beta, vb)).sum())
    rhs = float((oq * v).sum() + (ob * vb).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_port_objective_gradient_matches_fd(port_built, tmp_path):
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "obj", 29, 15, turbulence="sa")
    p = PortCase(c)
    q = C.perturbed_state(c, 8)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1))
    g = p.objective_grad(q)
    h = 1e-6
    fd = (p.skin_friction(q + h * v)[1] - p.skin_friction(q - h * v)[1]) / (2 * h)
    assert abs((g * v).sum() - fd) <= 1e-7 * abs(fd)


@pytest.mark.parametrize("angle,mu", [(1.5, 0.0), (0.0, 3e-7)])
def test_uniform_flow_is_preserved(port_built, tmp_path, angle, mu):
    """Freestream with freestream boundaries: R = 0 up to round-off.  Viscous
    cases use a rectangular grid: the reference's boundary-face Green-Gauss
    gradient (src/utils/mesh.cpp:54-82) does not close on skewed boundary
    cells, so a constant field has a small non-zero gradient there."""
    from oracle.port import PortCase
    c = flat_plate(tmp_path, "uni", 33, 17, top_angle_deg=angle)
    c.mu_inf = mu
    c.boundaries = [C.Boundary("freestream", f, 0, -1) for f in ("bottom", "top", "left", "right")]
    p = PortCase(c)
    q = C.freestream_state(c)
    r = p.residual(q)
    assert rel_err(r, 0 * r, p.flux_scale(q)) < 1e-13


def test_stretching_rules():
    # first cell 1e-4 at 1.08 over 64 cells cannot reach 0.5: ratio is solved up
    y = C.stretched_spacing(64, 1e-4, 1.08, 0.5)
    assert abs(y[-1] - 0.5) < 1e-15 and abs(y[1] - 1e-4) < 1e-12
    d = np.diff(y)
    assert np.all(np.diff(d) > 0)
    # 256 cells at 1.08 overshoot: geometric, then uniform
    y = C.stretched_spacing(256, 1e-4, 1.08, 0.5)
    d = np.diff(y)
    assert abs(y[-1] - 0.5) < 1e-15 and abs(d[0] - 1e-4) < 1e-15
    assert np.all(np.diff(d) > -1e-12)
    r = d[1:40] / d[:39]
    assert np.allclose(r, 1.08)


def test_grid_and_inp_roundtrip(tmp_path):
    c = flat_plate(tmp_path, "rt", 17, 9, top_angle_deg=-2.0)
    xv, yv = C.load_grid(c)
    g = C.flat_plate_grid(17, 9, h1=1e-4, ratio=1.08, top_angle_deg=-2.0)
    np.testing.assert_array_equal(xv, g.xv)
    np.testing.assert_array_equal(yv, g.yv)
    c2 = C.read_inp(os.path.join(str(tmp_path), "rt.inp"))
    assert c2.ni == c.ni and c2.mu_inf == c.mu_inf and len(c2.boundaries) == len(c.boundaries)
    assert [b.type for b in c2.boundaries] == [b.type for b in c.boundaries]
    assert c2.boundaries[0].face == "bottom" and c2.i_le == c.i_le


@pytest.mark.parametrize("name", ["wake", "channel"])
def test_port_vjp_transposes_jvp_with_nonlocal_boundaries(port_built, name):
    """Wake and periodic boundaries couple distant cells; the oracle's
    transposed product must still satisfy psi . (J v) = (J^T psi) . v."""
    from oracle.port import PortCase
    c, g = load_golden(name)
    p = PortCase(c, g["xv"], g["yv"])
    rng = np.random.default_rng(5)
    v = rng.standard_normal(g["q"].shape)
    psi = rng.standard_normal(g["q"].shape)
    oq, _ = p.vjp(g["q"], psi)
    lhs = float((psi * p.jvp(g["q"], v)).sum())
    assert abs(lhs - float((oq * v).sum())) <= 1e-12 * abs(lhs)


def test_port_objective_gradient_with_wake_matches_fd(port_built):
    """dJ/dQ where the plate's first faces read wake-cut ghosts (a distant
    column) against central differences."""
    from oracle.port import PortCase
    c, g = load_golden("wake")
    c.i_le = 9  # the no-slip wall's first vertex in this fixture
    p = PortCase(c, g["xv"], g["yv"])
    q = g["q"]
    v = np.random.default_rng(2).standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1))
    h = 1e-6
    fd = (p.skin_friction(q + h * v)[1] - p.skin_friction(q - h * v)[1]) / (2 * h)
    assert abs(float((p.objective_grad(q) * v).sum()) - fd) <= 1e-8 * abs(fd)
