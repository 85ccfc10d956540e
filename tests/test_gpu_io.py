"""Output path on the GPU: the wall-face gradients behind the surface file
against the reference's (golden io_fp.npz), the files written from a device
solution, and the command-line driver end to end."""
import os

import numpy as np
import pytest

from helpers import load_golden
from structured_gb300 import case as C
from structured_gb300 import io

pytestmark = pytest.mark.gpu


def eq_for(c, g):
    from structured_gb300.solver import EulerEquation
    eq = EulerEquation(c, g["xv"], g["yv"])
    eq.set_state(g["q"])
    return eq


def test_wall_gradients_match_reference(gpu_lib):
    c, g = load_golden("io_fp")
    wg = eq_for(c, g).wall_gradients()
    ref = g["wall_grad"]
    scale = np.abs(ref).max(axis=0) + 1e-300
    assert (np.abs(wg - ref).max(axis=0) / scale).max() < 1e-11


def test_outputs_from_device_solution_match_reference(gpu_lib, tmp_path):
    c, g = load_golden("io_fp")
    eq = eq_for(c, g)
    label = str(tmp_path / "gpu")
    forces = io.write_outputs(eq, label)
    assert np.array_equal(np.fromfile(label + ".out", dtype=np.uint8), g["out"])
    ours = np.loadtxt(label + ".surface")
    ref = np.array([[float(t) for t in line.split()] for line in str(g["surface"]).splitlines()])
    assert ours.shape == ref.shape
    # six significant digits either side; device gradients differ in the last bits
    np.testing.assert_allclose(ours, ref, rtol=2e-6, atol=1e-12)
    d = np.load(label + ".npz")
    for k in d.files:
        assert np.array_equal(d[k], g["npz_" + k]), k
    assert np.isfinite(forces["cd"])


@pytest.mark.parametrize("explicit", [False, True])
def test_driver_writes_the_reference_files(gpu_lib, tmp_path, explicit):
    from structured_gb300 import run
    if explicit:
        c = C.channel_case(str(tmp_path), "ch", nj=21)
        c.scheme, c.cfl, c.iteration_max = "rk4_jameson", 0.5, 30
    else:
        c = C.flat_plate_case(str(tmp_path), "fp", 33, 21, 0.3, 1e5, 1e-3, 1.1, lhs_order=1)
        c.cfl, c.cfl_ramp, c.cfl_ramp_iteration, c.cfl_ramp_exponent, c.iteration_max = 10.0, True, 2, 1.5, 6
    c.tail = 1
    inp = str(tmp_path / "case.inp")
    C.write_inp(inp, c)
    res = run.run(inp, explicit=explicit, log=lambda m: None)
    for ext in (".out", ".npz", ".tec", ".surface", ".history"):
        assert os.path.getsize(c.label + ext) > 0, ext
    with open(c.label + ".history") as f:
        lines = f.read().splitlines()
    assert len(lines) == res["steps"] == c.iteration_max
    norms = np.array([[float(t) for t in line.split()[4:]] for line in lines])
    assert np.isfinite(norms).all()
    if not explicit:
        assert norms[-1].max() < norms[0].max()  # the implicit steps reduce the residual
    q = io.read_restart(c.label + ".out", c.ni - 1, c.nj - 1, 4)
    assert np.isfinite(q).all()
