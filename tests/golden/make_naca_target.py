"""Target for the full-size NACA 0012 implicit run on the GPU: the oracle's
steady state of the laminar example's flow on this package's generated
281 x 151 C-grid (case.naca0012_case), by Newton with exact sparse LU steps on
the partner-block Jacobian (tests/block_jacobian.py), and its Cl/Cd from the
compiled reference's wall gradients through structured_gb300.io.write_surface.
Writes tests/golden/naca0012_281x151_target.json.  CPU, about an hour:

    python tests/golden/make_naca_target.py [workdir]
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import block_jacobian as BJ  # noqa: E402
from oracle.port import PortCase  # noqa: E402
from oracle.refcase import RefCase  # noqa: E402
from structured_gb300 import case as C  # noqa: E402
from structured_gb300 import io  # noqa: E402


def main(work):
    c = C.naca0012_case(work, "naca", ni=281, nj=151, tail=41)
    c.lhs_order = 2
    C.write_inp(os.path.join(work, "naca.inp"), c)
    xv, yv = C.load_grid(c)
    port = PortCase(c, xv, yv)
    q, hist = BJ.steady_newton(port, c, C.freestream_state(c), tol=1e-9, max_steps=80)
    print("Newton:", len(hist), "steps, last residuals", hist[-4:], flush=True)
    ref = RefCase(os.path.join(work, "naca.inp"))
    rr = ref.residual(q)  # fills the reference's face gradients of this state
    assert np.sqrt((rr ** 2).sum(axis=(0, 1))).max() < 1e-8
    grad = np.ascontiguousarray(ref.eta_gradients()[:, 0, :])
    forces = io.write_surface(os.path.join(work, "naca.surface"), c, xv, yv, q, grad)
    out = {"grid": "case.naca0012_case(ni=281, nj=151, tail=41)", "lhs_order": 2, "newton_steps": len(hist) - 1,
           "residual": [float(h) for h in hist], "forces": forces}
    with open(os.path.join(HERE, "naca0012_281x151_target.json"), "w") as f:
        json.dump(out, f, indent=1)
    np.save(os.path.join(work, "q.npy"), q)
    print(json.dumps(forces, indent=1))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else tempfile.mkdtemp())
