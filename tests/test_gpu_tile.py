"""The tiled residual sweeps (TMA-staged tiles, st_tile.cuh) against the
per-stage passes on the same inputs: the reference's residual fixtures
(flat plate orders 1/2, AUSM, channel with periodic and isothermal walls,
inviscid, the NACA0012 wake-cut pattern) and SA plates whose sizes are not
multiples of the tiles.  Both paths use the same face arithmetic, so they
agree to round-off (bound: 1e-13 of each cell's flux scale; the oracle parity
tests hold the default, per-stage, path at 1e-12; here the tiled path is
also checked against the oracle directly)."""
import numpy as np
import pytest

from helpers import flat_plate, golden_names, load_golden, rel_err
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu


def both_paths(eq, q, lhs=False):
    assert eq.set_residual_path(True)
    a = eq.calc_residual(q, lhs=lhs)
    assert not eq.set_residual_path(False)
    b = eq.calc_residual(q, lhs=lhs)
    return a, b


@pytest.mark.parametrize("name", golden_names())
def test_tiled_sweeps_match_per_stage_passes_on_fixtures(gpu_lib, name):
    from structured_gb300.solver import EulerEquation
    c, g = load_golden(name)
    eq = EulerEquation(c, g["xv"], g["yv"])
    for lhs, sc, ref in ((False, g["scale"], g["rhs"]), (True, g["scale_lhs"], g["rhs_lhs"])):
        a, b = both_paths(eq, g["q"], lhs)
        err = rel_err(a, b, sc)
        print("%s lhs=%d: tiled vs per-stage %.2e, tiled vs reference %.2e" % (name, lhs, err, rel_err(a, ref, sc)))
        assert err <= 1e-13
        assert rel_err(a, ref, sc) < 1e-12


@pytest.mark.parametrize("shape,order", [((37, 23), 2), ((70, 45), 2), ((70, 45), 1), ((131, 67), 2)])
def test_tiled_sweeps_match_on_sa_plates(gpu_lib, port_built, tmp_path, shape, order):
    from oracle.port import PortCase
    from structured_gb300.solver import EulerEquation
    c = flat_plate(tmp_path, "tile", shape[0], shape[1], turbulence="sa", reynolds=5e6, h1=1e-6, ratio=1.15,
                   order=order)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 31)
    beta = 1.0 + 0.2 * np.random.default_rng(32).standard_normal((c.nic, c.njc))
    eq = EulerEquation(c, xv, yv)
    eq.set_beta(beta)
    a, b = both_paths(eq, q)
    port = PortCase(c, xv, yv)
    sc = port.flux_scale(q, beta)
    err = rel_err(a, b, sc)
    print("SA %dx%d order %d: tiled vs per-stage %.2e, vs oracle %.2e"
          % (shape[0], shape[1], order, err, rel_err(a, port.residual(q, beta), sc)))
    assert err <= 1e-13
    assert rel_err(a, port.residual(q, beta), sc) < 1e-12
