"""Generates the golden fixtures in this folder from the reference solver's own
residual code (anandpratap/structured src/, compiled out of tree by
oracle/Makefile into oracle/_ref/libref_serial.so).

Run from the repository root where the reference sources are mounted:
    make -C oracle ref port && python tests/golden/make_golden.py
Each fixture stores the grid, the case, a seeded state and the reference's
calc_residual (both reconstruction orders), calc_dt and ghost-padded
primitives, plus the per-cell flux scale used to state relative errors;
io_fp.npz holds the reference's output files for one state.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.port import PortCase  # noqa: E402
from oracle.refcase import RefCase  # noqa: E402
from structured_gb300 import case as C  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def cases(tmp: str):
    yield "fp_o2", C.flat_plate_case(tmp, "fp_o2", 41, 21, 0.3, 1e6, 1e-4, 1.08, lhs_order=1), 7
    yield "fp_o1", C.flat_plate_case(tmp, "fp_o1", 41, 21, 0.3, 1e6, 1e-4, 1.08, order=1, lhs_order=1), 7
    yield "fp_lowre", C.flat_plate_case(tmp, "fp_lowre", 33, 17, 0.2, 2e3, 2e-3, 1.1, lhs_order=1), 11
    yield "fp_incl", C.flat_plate_case(tmp, "fp_incl", 37, 19, 0.2, 1e5, 1e-3, 1.1, top_angle_deg=2.0, lhs_order=1), 13
    yield "channel", C.channel_case(tmp, "channel", nj=41), 17
    c = C.flat_plate_case(tmp, "inviscid", 33, 17, 0.5, 1e6, 1e-3, 1.1, lhs_order=1)
    c.mu_inf = 0.0
    c.boundaries = [C.Boundary("slipwall", "bottom", 1, -2), C.Boundary("freestream", "top", 0, -1),
                    C.Boundary("freestream", "left", 0, -1), C.Boundary("outflow", "right", 0, -1)]
    C.write_inp(os.path.join(tmp, "inviscid.inp"), c)
    yield "inviscid", c, 19
    # AUSM (the reference's default flux): subsonic viscous plate, and a supersonic
    # inviscid one whose i-face Mach numbers pass |M| > 1 (both split branches)
    c = C.flat_plate_case(tmp, "fp_ausm", 41, 21, 0.3, 1e6, 1e-4, 1.08, lhs_order=1)
    c.flux = "ausm"
    C.write_inp(os.path.join(tmp, "fp_ausm.inp"), c)
    yield "fp_ausm", c, 29
    c = C.flat_plate_case(tmp, "ausm_sup", 33, 17, 1.5, 1e6, 1e-3, 1.1, lhs_order=1)
    c.mu_inf = 0.0
    c.flux = "ausm"
    c.boundaries = [C.Boundary("slipwall", "bottom", 1, -2), C.Boundary("freestream", "top", 0, -1),
                    C.Boundary("freestream", "left", 0, -1), C.Boundary("outflow", "right", 0, -1)]
    C.write_inp(os.path.join(tmp, "ausm_sup.inp"), c)
    yield "ausm_sup", c, 31
    # the wake cut of the reference's NACA0012 C-grid example (bc.cpp:224-263): bottom
    # cells 1..tail exchange ghosts with cells nic+1-i..; no-slip wall between
    c = C.flat_plate_case(tmp, "wake", 41, 21, 0.5, 1e5, 1e-3, 1.1, lhs_order=1)
    tail = 8
    c.boundaries = [C.Boundary("freestream", "top", 0, -1), C.Boundary("freestream", "left", 0, -1),
                    C.Boundary("freestream", "right", 0, -1), C.Boundary("wake", "bottom", 1, tail),
                    C.Boundary("wall", "bottom", tail + 1, c.ni - 1 - tail)]
    C.write_inp(os.path.join(tmp, "wake.inp"), c)
    yield "wake", c, 37


def io_fixture(tmp: str):
    """The reference's own output files (IOManager::write, src/utils/io.cpp:41-255)
    for one flat-plate state: tecplot, npz, restart and surface text, with the
    wall-face gradients and primitives the surface file was computed from."""
    c = C.flat_plate_case(tmp, "io_fp", 41, 21, 0.3, 1e6, 1e-4, 1.08, lhs_order=1)
    c.tail = 1  # surface faces [tail-1, ni-tail): the whole bottom row
    C.write_inp(os.path.join(tmp, "io_fp.inp"), c)
    xv, yv = C.load_grid(c)
    q = C.perturbed_state(c, 23)
    ref = RefCase(os.path.join(tmp, "io_fp.inp"))
    ref.write_outputs(q)
    lab = c.label
    ref_npz = np.load(lab + ".npz")
    d = C.case_to_dict(c)
    d["grid_path"] = ""
    d["label"] = "io_fp"
    with open(lab + ".surface") as f:
        surface = f.read()
    with open(lab + ".tec") as f:
        tec = f.read()
    out = np.fromfile(lab + ".out", dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, "io_fp.npz"), case=json.dumps(d), xv=xv, yv=yv, q=q,
                        surface=surface, tec=tec, out=out, wall_grad=ref.eta_gradients()[:, 0, :],
                        **{"npz_" + k: ref_npz[k] for k in ref_npz.files})
    print("io_fp", q.shape, len(surface.splitlines()), "surface lines")


def main():
    with tempfile.TemporaryDirectory() as tmp:
        io_fixture(tmp)
        for name, c, seed in cases(tmp):
            xv, yv = C.load_grid(c)
            ref = RefCase(os.path.join(tmp, name + ".inp"))
            q = C.perturbed_state(c, seed)
            if name == "channel":
                q = C.perturbed_state(c, seed, amplitude=0.01)
            rhs = ref.residual(q)
            prim = ref.primitives()
            rhs_lhs = ref.residual(q, lhs=True)
            dt = ref.dt(q, 2.5)
            port = PortCase(c, xv, yv)
            scale = port.flux_scale(q)
            scale_lhs = port.flux_scale(q, lhs=True)
            d = C.case_to_dict(c)
            d["grid_path"] = ""
            d["label"] = name
            np.savez_compressed(os.path.join(OUT, name + ".npz"), case=json.dumps(d), xv=xv, yv=yv, q=q,
                                rhs=rhs, rhs_lhs=rhs_lhs, dt=dt, cfl=2.5, prim=prim, scale=scale,
                                scale_lhs=scale_lhs, seed=seed)
            print(name, q.shape, float(np.abs(rhs).max()))


if __name__ == "__main__":
    main()
