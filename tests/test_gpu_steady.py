"""Converged flat plates on the GPU against the oracle's steady states
(tests/golden/make_steady.py: Newton with exact sparse-LU steps on the
oracle's second-order Jacobian): the laminar plate of the plain-method
workload (129x65, M=0.2, Re_L=1e5) and an SA plate (69x49, first cell 1e-7,
Re_L=5e6).  Both solves start from the uniform freestream.  Wall skin friction
Cf per face (the reference's Cf, src/utils/io.cpp:217-226) and the drag
J = sum Cf dx over the plate agree to 1e-8: Cf per face relative to the
largest |Cf|, J relative to |J|."""
import json
import os

import numpy as np
import pytest

from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = C.case_from_dict(json.loads(str(d["case"])))
    return c, d


def compare(eq, d, label):
    cf, J = eq.skin_friction()
    cf_ref, J_ref = d["cf"], float(d["J"])
    q, q_ref = eq.get_state(), d["q"]
    cf_err = float(np.abs(cf - cf_ref).max() / np.abs(cf_ref).max())
    j_err = abs(J - J_ref) / abs(J_ref)
    q_err = float((np.abs(q - q_ref).max(axis=(0, 1)) / np.abs(q_ref).max(axis=(0, 1))).max())
    print("%s: Cf %.2e, J %.2e (J = %.12e), state %.2e" % (label, cf_err, j_err, J, q_err))
    assert cf_err <= 1e-8
    assert j_err <= 1e-8


def test_laminar_plate_matches_oracle_steady_state(gpu_lib):
    from structured_gb300.solver import EulerEquation, Solver
    c, d = load("steady_laminar_129x65")
    eq = EulerEquation(c, d["xv"], d["yv"])
    eq.set_state(C.freestream_state(c))
    # run into the residual's round-off floor: the tolerance sits below it
    ok, hist = Solver(eq, max_steps=120, cfl=5.0, cfl_ramp=1, cfl_ramp_iteration=3, cfl_ramp_exponent=1.3,
                      rel_tolerance=1e-15, krylov_rtol=1e-6).solve(raise_on_noconv=False)
    assert hist[-1, 3:].max() <= 1e-11 * hist[0, 3:].max(), hist[-5:]
    compare(eq, d, "laminar 129x65 (%d steps, residual %.1e)" % (len(hist), hist[-1, 3:].max()))


def test_sa_plate_matches_oracle_steady_state(gpu_lib):
    from structured_gb300.solver import EulerEquation, Solver
    c, d = load("steady_sa_69x49")
    eq = EulerEquation(c, d["xv"], d["yv"])
    eq.set_state(C.freestream_state(c))
    ok, hist = Solver(eq, max_steps=120, cfl=5.0, cfl_growth=2.0, rel_tolerance=1e-15,
                      krylov_rtol=1e-6).solve(raise_on_noconv=False)
    assert hist[-1, 3:].max() <= 1e-11 * hist[0, 3:].max(), hist[-5:]
    compare(eq, d, "SA 69x49 (%d steps, residual %.1e)" % (len(hist), hist[-1, 3:].max()))
