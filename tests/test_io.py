"""Output files against the reference's own (IOManager, src/utils/io.cpp),
from the golden fixture io_fp.npz that tests/golden/make_golden.py writes by
running the reference's IOManager::write on a seeded flat-plate state."""
import os

import numpy as np

from helpers import load_golden
from structured_gb300 import io


def golden():
    return load_golden("io_fp")


def test_restart_bytes_match_reference(tmp_path):
    c, g = golden()
    path = str(tmp_path / "r.out")
    io.write_restart(path, g["q"])
    assert np.array_equal(np.fromfile(path, dtype=np.uint8), g["out"])
    q = io.read_restart(path, c.ni - 1, c.nj - 1, 4)
    assert np.array_equal(q, g["q"])


def test_restart_size_is_checked(tmp_path):
    c, g = golden()
    path = str(tmp_path / "r.out")
    io.write_restart(path, g["q"][:, :-1])
    try:
        io.read_restart(path, c.ni - 1, c.nj - 1, 4)
    except ValueError:
        return
    raise AssertionError("a short restart file was accepted")


def test_npz_arrays_match_reference(tmp_path):
    c, g = golden()
    xc, yc = io.cell_centres(g["xv"], g["yv"])
    path = str(tmp_path / "s.npz")
    io.write_npz(path, xc, yc, g["q"], io.primitives(g["q"], c))
    d = np.load(path)
    assert sorted(d.files) == sorted(k[4:] for k in g if k.startswith("npz_"))
    for k in d.files:
        assert d[k].shape == g["npz_" + k].shape, k
        assert np.array_equal(d[k], g["npz_" + k]), k  # bit for bit


def test_surface_text_matches_reference(tmp_path):
    c, g = golden()
    path = str(tmp_path / "s.surface")
    forces = io.write_surface(path, c, g["xv"], g["yv"], g["q"], g["wall_grad"])
    with open(path) as f:
        assert f.read() == str(g["surface"])
    assert all(np.isfinite(v) for v in forces.values())
    assert abs(forces["cl"] - forces["cl_pressure"] - forces["cl_viscous"]) < 1e-15


def test_surface_of_tail_zero_is_empty(tmp_path):
    c, g = golden()
    c.tail = 0
    path = str(tmp_path / "s.surface")
    io.write_surface(path, c, g["xv"], g["yv"], g["q"], g["wall_grad"])
    assert os.path.getsize(path) == 0


def test_tecplot_matches_reference(tmp_path):
    c, g = golden()
    xc, yc = io.cell_centres(g["xv"], g["yv"])
    path = str(tmp_path / "s.tec")
    io.write_tecplot(path, xc, yc, g["q"])
    with open(path) as f:
        ours = f.read().splitlines()
    ref = str(g["tec"]).splitlines()
    assert len(ours) == len(ref)
    assert ours[:3] == ref[:3]
    for a, b in zip(ours[3:], ref[3:]):
        assert a.split()[:6] == b.split()[:6]  # x, y, q; the q_aux columns are unset in the reference


def test_history_line_format():
    line = io.history_line(12, 0.5, 1.25, 10.0, [1e-3, 2e-4, 3e-5, 4e-6, 5e-7])
    assert line == "00000012 5.00e-01 1.25e+00 1.00e+01 1.00e-03 2.00e-04 3.00e-05 4.00e-06"
