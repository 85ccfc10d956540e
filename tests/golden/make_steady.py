"""Converged flat-plate states from the oracle, the targets of the GPU
steady-state tests (tests/test_gpu_steady.py):

  steady_laminar_129x65.npz  the laminar plate (129x65, M=0.2, Re_L=1e5,
                             Sutherland, Pr=0.72) from a uniform freestream
  steady_sa_69x49.npz        the SA plate (69x49, first cell 1e-7 at ratio 1.05,
                             M=0.2, Re_L=5e6, beta = 1)

Each holds the case, the oracle's Newton steady state (exact sparse-LU steps
on the second-order Jacobian assembled from the oracle's dual-number JVPs,
tests/block_jacobian.py), its residual history, and the oracle's wall skin
friction Cf per face and drag J = sum Cf dx over the plate (the reference's
Cf of IOManager::write_surface, src/utils/io.cpp:217-226).  CPU, a few minutes:

    python tests/golden/make_steady.py
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
from structured_gb300 import case as C  # noqa: E402
from structured_gb300 import workloads  # noqa: E402

CASES = {
    "steady_laminar_129x65": lambda w: workloads.laminar_plate(w),
    "steady_sa_69x49": lambda w: workloads.turbulent_plate(w, 69, 49),
}


def make(name, work, tol, max_steps=120):
    c = CASES[name](work)
    xv, yv = C.load_grid(c)
    port = PortCase(c, xv, yv)
    q, hist = BJ.steady_newton(port, c, C.freestream_state(c), tol=tol, max_steps=max_steps)
    cf, J = port.skin_friction(q)
    print(name, len(hist), "steps; residuals", " ".join("%.2e" % h for h in hist), "J %.15e" % J, flush=True)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), case=json.dumps(C.case_to_dict(c)), xv=xv, yv=yv, q=q,
                        hist=hist, cf=cf, J=J)


def main(work):
    # tolerances at the residuals' round-off floors (about 4e-11 laminar, 1e-7 SA)
    make("steady_laminar_129x65", work, tol=1e-10, max_steps=60)
    make("steady_sa_69x49", work, tol=5e-7, max_steps=60)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else tempfile.mkdtemp())
