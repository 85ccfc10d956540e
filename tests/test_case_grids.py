"""Generated grids (structured_gb300/case.py) on CPU: the NACA 0012 C-grid
reproduces the reference example's topology and boundary list, with positive
cell volumes under the oracle's metrics and a finite residual."""
import numpy as np

from structured_gb300 import case as C


def test_naca0012_cgrid_topology_and_metrics(port_built, tmp_path):
    from oracle.port import PortCase
    c = C.naca0012_case(str(tmp_path), "naca", ni=121, nj=41, tail=21)
    xv, yv = C.load_grid(c)
    assert xv.shape == (121, 41)
    # the wake cut: vertex i and ni-1-i coincide on j = 0 for the tail vertices
    np.testing.assert_array_equal(xv[:21, 0], xv[::-1][:21, 0])
    np.testing.assert_array_equal(yv[:21, 0], yv[::-1][:21, 0])
    # the section is closed at the trailing edge and passes through the leading edge
    assert xv[20, 0] == 1.0 and yv[20, 0] == 0.0 and abs(xv[60, 0]) < 1e-15
    kinds = [(b.type, b.face, b.start, b.end) for b in C.read_inp(str(tmp_path / "naca.inp")).boundaries]
    assert ("wake", "bottom", 1, 20) in kinds and ("wall", "bottom", 21, 100) in kinds
    p = PortCase(c, xv, yv)
    vol = p.metrics()[2]
    assert (vol > 0).all()
    assert np.isfinite(p.residual(C.freestream_state(c))).all()


def test_naca0012_thickness_is_twelve_percent():
    x = np.linspace(0.0, 1.0, 20001)
    t = 2 * C.naca0012_half_thickness(x)
    assert abs(t.max() - 0.12) < 2e-4 and abs(x[t.argmax()] - 0.30) < 0.01
    assert abs(C.naca0012_half_thickness(np.array([1.0]))[0]) < 1e-12  # closed trailing edge


def test_inp_round_trip_keeps_solver_and_boundary_keys(tmp_path):
    c = C.naca0012_case(str(tmp_path), "rt", ni=41, nj=11, tail=11, write_files=False)
    c.flux, c.scheme, c.cfl, c.cfl_ramp, c.iteration_max = "ausm", "forward_euler", 2.5, True, 77
    c.grid_path = str(tmp_path / "rt.p3d")
    C.write_p3d(c.grid_path, C.naca0012_cgrid(41, 11, 11))
    path = str(tmp_path / "rt.inp")
    C.write_inp(path, c)
    r = C.read_inp(path)
    for k in ("ni", "nj", "tail", "flux", "scheme", "cfl", "cfl_ramp", "iteration_max", "aoa", "u_inf", "v_inf",
              "mu_inf", "order", "lhs_order"):
        assert getattr(r, k) == getattr(c, k), k
    assert [(b.type, b.face, b.start, b.end) for b in r.boundaries] == \
        [(b.type, b.face, b.start, b.end) for b in c.boundaries]


def test_missing_flux_key_reads_as_the_reference_default(tmp_path):
    """config.cpp:54: solver.flux defaults to "ausm"."""
    c = C.channel_case(str(tmp_path), "ch", nj=11)
    path = str(tmp_path / "ch.inp")
    text = open(path).read().replace('flux = "roe"\n', "")
    open(path, "w").write(text)
    assert C.read_inp(path).flux == "ausm"
