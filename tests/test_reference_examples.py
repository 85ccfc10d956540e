"""The reference's own example cases (examples/laminar/naca0012/config.inp with
its grid.unf2, examples/laminar/channel/{explicit,implicit}.inp with
channel_3x101.unf2), read by this package's .inp reader and grid loaders
(src/utils/config.cpp, src/utils/mesh.cpp:134-169): the oracle's metrics and
residual on them equal the compiled reference's own, the channel generator
reproduces the example grid, and the partner-block Jacobian layout reproduces
the oracle's JVP on the full 281 x 151 NACA 0012 example grid.  CPU only; the
reference's files are read where they lie and the tests skip without them."""
import os

import numpy as np
import pytest

import block_jacobian as BJ
from conftest import REF_ROOT
from structured_gb300 import case as C

EXAMPLES = os.path.join(REF_ROOT, "examples", "laminar")
CASES = [("naca0012", "config.inp"), ("channel", "implicit.inp"), ("channel", "explicit.inp")]


def example(name, inp):
    d = os.path.join(EXAMPLES, name)
    c = C.read_inp(os.path.join(d, inp))
    c.grid_path = os.path.join(d, os.path.basename(c.grid_path))
    return d, c, C.load_grid(c)


@pytest.mark.parametrize("name,inp", CASES)
def test_example_reads_and_matches_the_reference(ref_available, port_built, monkeypatch, name, inp):
    if not ref_available:
        pytest.skip("reference sources not mounted")
    from oracle.port import PortCase
    from oracle.refcase import RefCase
    d, c, (xv, yv) = example(name, inp)
    monkeypatch.chdir(d)  # the reference opens the grid relative to the working directory
    ref = RefCase(inp)
    assert (ref.ni, ref.nj) == xv.shape == (c.ni, c.nj)
    port = PortCase(c, xv, yv)
    for a, b in zip(ref.metrics(), port.metrics()[:3]):
        assert np.array_equal(a, b)
    q = C.perturbed_state(c, 5)
    assert np.array_equal(ref.residual(q), port.residual(q))
    assert np.array_equal(ref.residual(q, lhs=True), port.residual(q, lhs=True))


def test_channel_generator_reproduces_the_example_grid(ref_available, tmp_path):
    if not os.path.isdir(EXAMPLES):
        pytest.skip("reference examples not mounted")
    _, c, (xv, yv) = example("channel", "implicit.inp")
    g = C.channel_case(str(tmp_path), "ch", nj=101)
    xg, yg = C.load_grid(g)
    assert np.array_equal(xg, xv) and np.array_equal(yg, yv)
    assert [(b.type, b.face, b.start, b.end) for b in g.boundaries] == \
        [(b.type, b.face, b.start, b.end) for b in c.boundaries]


def test_partner_layout_on_the_naca_example_grid(port_built):
    if not os.path.isdir(EXAMPLES):
        pytest.skip("reference examples not mounted")
    from oracle.port import PortCase
    _, c, (xv, yv) = example("naca0012", "config.inp")
    port = PortCase(c, xv, yv)
    q = C.perturbed_state(c, 9)
    masks, on = BJ.partner_masks(c)
    assert on == [True, False, False] and masks[0].sum() == 2 * 40
    jac = BJ.assemble_regular(port, q, 2)
    W = BJ.assemble_partners(port, q, masks, on, 2)
    A = BJ.to_sparse(jac, W)
    x = np.random.default_rng(4).standard_normal(q.shape)
    jv = port.jvp(q, x)
    assert np.abs(A @ x.ravel() - jv.ravel()).max() < 1e-13 * np.abs(jv).max()
    # (transposed products against the oracle's VJP: tests/test_partner_jacobian.py,
    # on grids where the oracle's dense VJP path is affordable)


def test_surface_file_on_the_naca_example_matches_the_reference(ref_available, tmp_path):
    """IOManager::write_surface on the C-grid example (wall faces tail-1 ..
    ni-tail-1 of the j = 0 row, src/utils/io.cpp:182-255): this package's
    writer, given the reference's wall gradients, writes the same bytes."""
    if not ref_available:
        pytest.skip("reference sources not mounted")
    from oracle.refcase import RefCase
    from structured_gb300 import io
    d, c, (xv, yv) = example("naca0012", "config.inp")
    text = open(os.path.join(d, "config.inp")).read()
    text = text.replace('filename = "grid.unf2"', 'filename = "%s"' % c.grid_path)
    text = text.replace('label = "implicit"', 'label = "%s"' % str(tmp_path / "ref"))
    inp = tmp_path / "config.inp"
    inp.write_text(text)
    ref = RefCase(str(inp))
    q = C.perturbed_state(c, 21)
    ref.residual(q)  # fills the reference's face gradients of this state
    grad = np.ascontiguousarray(ref.eta_gradients()[:, 0, :])
    ref.write_outputs(q)
    forces = io.write_surface(str(tmp_path / "ours.surface"), c, xv, yv, q, grad)
    assert (tmp_path / "ours.surface").read_bytes() == (tmp_path / "ref.surface").read_bytes()
    assert all(np.isfinite(v) for v in forces.values())
