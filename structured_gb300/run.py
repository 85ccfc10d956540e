"""Command-line driver of a GB300 run, in the place of the reference's
main.cpp + Solver::solve (src/main.cpp:8-42, src/solver/solver.cpp:198-236):

    python -m structured_gb300.run -c config.inp [--explicit] [--steps N]

Reads the same .inp and grid, starts from freestream or from <label>.out when
[io] restart = true, marches on the GPU and leaves the reference's files:
<label>.out, .npz, .tec, .surface and <label>.history.  The implicit
pseudo-time Newton solve is the default (the reference's ADOL-C build); with
--explicit the [solver] scheme (forward_euler | rk4_jameson) marches
explicitly.  Steps run in chunks of [io] stdout_frequency so every history
line carries its wall time; the implicit CFL ramp (CFL <- CFL^e once the step
count passes cfl_ramp_iteration, capped at 1e12) continues across chunks.
"""
from __future__ import annotations

import argparse
import math
import sys
import time
import tomllib

import numpy as np

from . import case as C
from . import io
from .solver import EulerEquation, Solver


def _io_keys(path: str) -> dict:
    with open(path, "rb") as f:
        t = tomllib.load(f)
    s = t.get("io", {})
    return {"restart": bool(s.get("restart", False)), "stdout_frequency": max(1, int(s.get("stdout_frequency", 1)))}


def run(config: str, explicit: bool = False, steps: int | None = None, log=print) -> dict:
    c = C.read_inp(config)
    keys = _io_keys(config)
    eq = EulerEquation(c)
    label = c.label
    if keys["restart"]:
        eq.set_state(io.read_restart(label + ".out", eq.nic, eq.njc, eq.nq))
    else:
        eq.set_state(C.freestream_state(c))
    total = c.iteration_max if steps is None else steps
    chunk = keys["stdout_frequency"]
    tol = c.tolerance if c.tolerance < 1e9 else 0.0
    rows, done, cfl = [], 0, c.cfl
    t0 = time.time()
    log("Welcome to structured (GB300)!")
    while done < total:
        n = min(chunk, total - done)
        if explicit:
            k, hist = eq.explicit_solve(c.scheme, cfl=c.cfl, steps=n, tolerance=tol, check_every=n,
                                        raise_on_noconv=False)
            norms = hist[-1, 1:] if len(hist) else np.zeros(eq.nq)
            stop = k < n or (tol > 0 and norms.max() <= tol)
        else:
            ramp_left = max(0, c.cfl_ramp_iteration - done)
            ok, hist = Solver(eq, cfl=cfl, max_steps=n, cfl_ramp_iteration=ramp_left,
                              tolerance=tol).solve(raise_on_noconv=False)
            k = int(hist[-1, 0])
            norms = hist[-1, 3:]
            cfl = float(hist[-1, 1])
            if c.cfl_ramp and done + k > c.cfl_ramp_iteration:
                cfl = min(math.pow(cfl, c.cfl_ramp_exponent), 1e12)
            stop = ok or k == 0
        done += k
        rows.append((done, 0.0, time.time() - t0, c.cfl if explicit else cfl, list(norms)))
        log("Step: %08d Wall Time: %.2e Density Norm: %.2e" % (done, rows[-1][2], norms[0]))
        if stop:
            break
    io.write_history(label + ".history", rows)
    forces = io.write_outputs(eq, label)
    log("Pressure Cl: %s Cd: %s" % (forces["cl_pressure"], forces["cd_pressure"]))
    log("Viscous Cl: %s Cd: %s" % (forces["cl_viscous"], forces["cd_viscous"]))
    log("Total Cl: %s Cd: %s" % (forces["cl"], forces["cd"]))
    return {"steps": done, "wall_s": time.time() - t0, "forces": forces, "history": rows}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("-c", "--config", default="config.inp")
    ap.add_argument("--explicit", action="store_true", help="march with the [solver] scheme")
    ap.add_argument("--steps", type=int, default=None, help="override [solver] iteration_max")
    a = ap.parse_args(argv)
    run(a.config, explicit=a.explicit, steps=a.steps)
    return 0


if __name__ == "__main__":
    sys.exit(main())
