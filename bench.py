#!/usr/bin/env python
"""Residual + discrete-adjoint throughput of the structured-grid solver path.

Workload: the residual-throughput sweep's largest grid (4097x2049 vertices,
8,388,608 cells, flat plate, first cell 1e-4 growing at 1.08 then uniform to
y=0.5), Spalart-Allmaras (nq=5, beta=1, i.e. plain SA), freestream M=0.3,
Re=1e6 with seeded 1 % Gaussian perturbations on rho, u, p, nu_tilde (v: 1 % of
u_inf).  One step = one full residual evaluation (+ one adjoint VJP
(dR/dQ)^T psi and (dR/dbeta)^T psi when built) on inputs resident in HBM.
Inputs (q 336 MB, primitives 537 MB) are larger than the 129 MB L2, so no
flush between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 (torchrun) runs independent replicas, one per GPU: the residual of one
block is not split across GPUs.  --impl reference times the CPU restatement of
the reference's residual (oracle/port, bit-exact with the reference's
calc_residual on the laminar fixtures) on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20261203
MACH, REYNOLDS = 0.3, 1e6
GRIDS = {"4097x2049": (4097, 2049), "2049x1025": (2049, 1025), "513x257": (513, 257)}
# algorithmic (compulsory) FP64 bytes per cell: q + metrics (+ wall distance,
# beta) read, rhs written; adjoint also reads psi and writes both products.
ALG_BYTES = {("none", "res"): 104, ("sa", "res"): 136, ("sa", "adj"): 184, ("none", "adj"): 136}


def build_case(grid: str, turbulence: str):
    from structured_gb300 import case as C
    ni, nj = GRIDS[grid]
    c = C.flat_plate_case(tempfile.gettempdir(), "bench", ni, nj, MACH, REYNOLDS, 1e-4, 1.08,
                          turbulence=turbulence, write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-4, ratio=1.08)
    q = C.perturbed_state(c, SEED)
    return c, g.xv, g.yv, q


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_figure(name: str, key: str):
    """Reads `key: value` from a committed ncu summary under profiles/."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            m = re.match(r"\s*[-*]?\s*%s\s*:\s*([0-9.eE+-]+)" % re.escape(key), line)
            if m:
                return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.gpus != world and world > 1:
        raise SystemExit("--gpus %d but WORLD_SIZE %d" % (args.gpus, world))
    return world, rank, local


def ensure_port():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)


def time_port(port, q, psi, with_adj, budget_s=None, steps=None):
    """Seconds per step of the CPU restatement: one residual, plus (with_adj)
    one forward-mode dual-number pass (dR/dQ) v of the same Jacobian, the
    operation-count class of a taped reverse sweep."""
    port.residual(q)
    if with_adj:
        port.jvp(q, psi)
    n, t0 = 0, time.perf_counter()
    while True:
        port.residual(q)
        if with_adj:
            port.jvp(q, psi)
        n += 1
        el = time.perf_counter() - t0
        if (steps is not None and n >= steps) or (budget_s is not None and el > budget_s):
            break
    return el / n, n


def cpu_baseline_sample(turbulence: str, budget_s: float, threads: int, with_adj: bool):
    """Times the CPU restatement (oracle/port) on the 513x257 grid of the
    same workload for about budget_s seconds."""
    ensure_port()
    from oracle.port import PortCase
    c, xv, yv, q = build_case("513x257", turbulence)
    port = PortCase(c, xv, yv)
    used = port.set_threads(threads)
    psi = np.random.default_rng(SEED + 1).standard_normal(q.shape)
    dt, n = time_port(port, q, psi, with_adj, budget_s=budget_s)
    what = "residual + dual-number JVP (adjoint-class pass)" if with_adj else "residual"
    return {"value": c.nic * c.njc / dt / 1e6, "unit": "Mcells/s", "cores": used, "kind": "port",
            "sample": "%d steps (%s) of the 513x257 grid of the same workload (%s), %.1f s"
                      % (n, what, turbulence, n * dt)}


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's figure (every rank gets it): replicas are timed
    independently, and the job is as slow as its slowest replica."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, cells: int, steps: int, seconds: float) -> float:
    """Whole-job Mcells/s: every replica processes `cells` per step."""
    return world * cells * steps / seconds / 1e6


def rate_breakdown(cells: int, res_ms: float, fused_ms: float | None) -> dict:
    """Per-evaluation rates from the per-launch event times of one residual
    pipeline and one fused residual+adjoint pipeline: residual alone, the
    adjoint's share (fused minus residual) and the fused step."""
    out = {"unit": "Mcells/s", "residual": cells / (res_ms * 1e-3) / 1e6, "residual_ms": res_ms}
    if fused_ms:
        out["fused_residual_adjoint"] = cells / (fused_ms * 1e-3) / 1e6
        out["fused_ms"] = fused_ms
        if fused_ms > res_ms:
            out["adjoint_increment"] = cells / ((fused_ms - res_ms) * 1e-3) / 1e6
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ensure_port()
    from oracle.port import PortCase
    with_adj = not args.residual_only
    # per step: one residual (+ adjoint-class pass) of the largest grid of this
    # workload that fits the time budget
    budget = 150.0 / max(1, args.steps + args.warmup)
    grid = "513x257"
    c, xv, yv, q = build_case(grid, args.turbulence)
    port = PortCase(c, xv, yv)
    port.set_threads(threads)
    psi = np.random.default_rng(SEED + 1).standard_normal(q.shape)
    t1, _ = time_port(port, q, psi, with_adj, steps=1)
    for g in ("2049x1025", "4097x2049"):
        ni, nj = GRIDS[g]
        if t1 * (ni - 1) * (nj - 1) / (c.nic * c.njc) < budget:
            grid = g
    if grid != "513x257":
        c, xv, yv, q = build_case(grid, args.turbulence)
        port = PortCase(c, xv, yv)
        port.set_threads(threads)
        psi = np.random.default_rng(SEED + 1).standard_normal(q.shape)
    for _ in range(args.warmup):
        port.residual(q)
        if with_adj:
            port.jvp(q, psi)
    dt, _ = time_port(port, q, psi, with_adj, steps=args.steps)
    cells = c.nic * c.njc
    v = cells / dt / 1e6
    what = "residual + dual-number JVP pass" if with_adj else "residual"
    line = {"impl": "reference", "metric": metric_name(with_adj), "value": v, "unit": "Mcells/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args, args.grid),
            "cpu_baseline": {"value": v, "unit": "Mcells/s", "cores": threads, "kind": "port",
                             "sample": "%s of the %s grid of the workload per step, %d steps" % (what, grid, args.steps)},
            "e2e": {"value": v, "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def metric_name(with_adjoint: bool) -> str:
    return "Mcells/s residual+adjoint" if with_adjoint else "Mcells/s residual"


def workload_config(args, grid):
    return {"workload": "flat-plate residual throughput, %s vertices, %s, M=%.1f Re=%.0e, seeded 1%% perturbations"
                        % (grid, "SA" if args.turbulence == "sa" else "laminar", MACH, REYNOLDS),
            "grid": grid, "turbulence": args.turbulence, "order": 2, "seed": SEED,
            "l2": "inputs larger than L2 (q 336 MB, primitives 537 MB); no flush", "parallelism": "replicas"}


CLOSURE = os.path.join(ROOT, "results", "closure_273x193")


def closure_leg():
    """The metric's second clause, on the learned-correction workload's
    held-out case (Re_L 3e6, top inclined at -2 deg; 273x193, the grid of the
    committed inversion study): a solve from freestream with the committed
    network (trained on the other cases' inversions) fused into the SA source,
    timed here, with its plate Cf error against the held-out case's
    inverted-beta solution; beside it the field inversion's own wall time on
    the same GPU type and plain SA's error, from the study's results file
    (python -m structured_gb300.validate closure)."""
    if not os.path.exists(CLOSURE + ".json"):
        return None
    import torch
    from structured_gb300 import case as C
    from structured_gb300 import inversion as inv
    from structured_gb300 import mlp, workloads
    from structured_gb300.solver import EulerEquation
    study = json.load(open(CLOSURE + ".json"))
    res = study["training"]["all"]
    held = np.load(CLOSURE + "_heldout.npz")
    params = np.load(CLOSURE + "_all_params.npy")
    c = workloads.turbulent_plate(tempfile.gettempdir(), 273, 193, 3e6, -2.0, write_files=False)
    g = C.flat_plate_grid(273, 193, h1=1e-7, ratio=1.05, top_angle_deg=-2.0)
    eq = EulerEquation(c, g.xv, g.yv)
    eq.mlp_init(0)
    eq.mlp_set_params(params.astype(np.float32))
    eq.mlp_set_normalization(np.array(res["feature_mean"], np.float32), np.array(res["feature_std"], np.float32))
    eq.mlp_enable(True)
    eq.set_state(C.freestream_state(c))
    mask = inv.plate_mask(c, g.xv)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ok, hist = inv.converge(eq)
    wall = time.perf_counter() - t0
    cf, _ = eq.skin_friction()
    eq.mlp_enable(False)
    err = float(np.abs((cf - held["cf_inv"])[mask] / held["cf_inv"][mask]).max())
    fi = res.get("field_inversion", {})
    other = {m: {"train_cases": len(r["train_cases"]), "learned_cf_err_vs_inverted": r["learned"]["cf_err_vs_inverted"],
                 "learned_solve_s": r["learned"]["wall_s"]}
             for m, r in study["training"].items() if m != "all"}
    return {"case": "turbulent plate 273x193, Re_L 3e6, top -2 deg (held out)",
            "network": "trained on the eight other cases' inversions (results/closure_273x193_all_params.npy)",
            "learned_solve_s": wall, "learned_steps": int(hist.shape[0] - 1) if hist is not None else None,
            "learned_converged": bool(ok), "learned_cf_err_vs_inverted": err,
            "plain_sa_cf_err_vs_inverted": res["plain_sa"]["cf_err_vs_inverted"],
            "field_inversion_s": fi.get("wall_s"), "field_inversion_s_to_cf_err_1pct": fi.get("wall_s_to_cf_err_1pct"),
            "other_training_sets": other,
            "source": "learned solve timed here; inversion, plain-SA and other training sets from "
                      "results/closure_273x193.json (python -m structured_gb300.validate closure)"}


def run_ours(args, world, rank, local):
    import torch
    from structured_gb300 import build
    from structured_gb300.solver import EulerEquation, StructuredError

    build.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    c, xv, yv, q = build_case(args.grid, args.turbulence)
    eq = EulerEquation(c, xv, yv, device=local)
    eq.set_state(q)
    qd, rd, sp = eq.device_state()
    stream = torch.cuda.ExternalStream(sp, device=torch.device("cuda", local))
    cells = c.nic * c.njc
    rng = np.random.default_rng(SEED + 1)
    psi = torch.tensor(rng.standard_normal(q.shape), device="cuda")
    outq = torch.empty_like(psi)
    outb = torch.empty((c.nic, c.njc), dtype=torch.float64, device="cuda")
    with_adj = not args.residual_only
    try:
        eq.vjp_device(psi.data_ptr(), outq.data_ptr(), outb.data_ptr())
        torch.cuda.synchronize()
    except StructuredError:
        with_adj = False
    n_res, n_vjp = eq.launch_counts()
    kernels_per_step = eq.fused_launch_count() if with_adj else n_res

    def step():
        if with_adj:
            eq.residual_vjp_device(psi.data_ptr(), rd, outq.data_ptr(), outb.data_ptr())
        else:
            eq.residual_device(qd, rd)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    el_ms = max_over_ranks(ev0.elapsed_time(ev1), world, "cuda")
    ms_step = el_ms / args.steps
    value = job_rate(world, cells, args.steps, el_ms * 1e-3)

    # per-launch attribution (outside the timed region): the residual by the
    # default per-stage passes and, for comparison, by the tiled (TMA-staged) sweeps
    kern_res = eq.profile("residual")
    res_ms = float(sum(kern_res.values()))
    kern_res_tiled = None
    try:
        eq.set_residual_path(True)
        kern_res_tiled = eq.profile("residual")
        eq.set_residual_path(False)
    except StructuredError:
        pass
    kern_adj = eq.profile("fused") if with_adj else {}
    adj_ms = float(sum(kern_adj.values()))
    fp64_peak = eq.probe_fp64_tflops()

    # end to end through the host-buffer C ABI: pinned q in, rhs (+ adjoint) out
    qh = torch.tensor(q).pin_memory()
    rh = torch.empty_like(qh).pin_memory()
    psih = torch.tensor(psi.cpu().numpy()).pin_memory()
    oqh = torch.empty_like(psih).pin_memory()
    obh = torch.empty((c.nic, c.njc), dtype=torch.float64).pin_memory()
    lib = eq.lib
    P = ctypes.POINTER(ctypes.c_double)

    def hp(t):
        return ctypes.cast(t.data_ptr(), P)

    def e2e_step():
        if lib.st_set_state(eq.h, hp(qh)):
            raise RuntimeError(lib.st_last_error())
        rc = lib.st_residual_vjp(eq.h, hp(psih), hp(rh), hp(oqh), hp(obh), 0) if with_adj \
            else lib.st_residual(eq.h, 0, hp(rh))
        if rc:
            raise RuntimeError(lib.st_last_error())

    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, args.steps // 4)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    nq = c.nq
    h2d = cells * nq * 8 * (2 if with_adj else 1)
    d2h = cells * nq * 8 * (2 if with_adj else 1) + (cells * 8 if with_adj else 0)
    e2e = {"value": job_rate(world, cells, e2e_steps, e2e_s), "unit": "Mcells/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    peak, peak_kind = measured_peaks()
    tb = args.turbulence
    alg = ALG_BYTES[(tb, "res")] + (ALG_BYTES[(tb, "adj")] if with_adj else 0)
    t_path = adj_ms if with_adj else res_ms
    achieved = alg * cells / (t_path * 1e-3) / 1e9
    prof = ("residual_adjoint_%s_%s.md" if with_adj else "residual_%s_%s.md") % (tb, args.grid)
    traffic_cell = profile_figure(prof, "dram_bytes_per_cell")
    flops_cell = profile_figure(prof, "fp64_flops_per_cell")
    pipe_pct = profile_figure(prof, "fp64_pipe_active_pct")
    kern = kern_adj if with_adj else kern_res
    top = max(kern, key=kern.get) if kern else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "traffic": traffic_cell * cells if traffic_cell else None,
            "scope": "whole %s evaluation (%d launches), %d algorithmic B/cell"
                     % ("fused residual+adjoint" if with_adj else "residual", kernels_per_step, alg),
            "kernels_ms": {"residual": kern_res, "residual_tiled": kern_res_tiled, "adjoint": kern_adj}}
    if top:
        roof["dominant_kernel"] = {"name": top, "ms": kern[top], "share": kern[top] / max(sum(kern.values()), 1e-30)}
    if flops_cell:
        fp64_ach = flops_cell * cells / (t_path * 1e-3) / 1e12
        roof["fp64"] = {"scope": "%s pipeline (ncu-counted flops / event time)"
                                 % ("fused residual+adjoint" if with_adj else "residual"),
                        "achieved_tflops": fp64_ach, "peak_tflops": fp64_peak, "frac": fp64_ach / fp64_peak,
                        "flops_per_cell": flops_cell, "peak_source": "live DFMA probe (st_probe_fp64)",
                        "pipe_active_frac": pipe_pct / 100.0 if pipe_pct else None,
                        "pipe_source": "ncu sm__pipe_fp64_cycles_active, time-weighted over the step (profiles/)"}
    else:
        roof["fp64"] = {"peak_tflops": fp64_peak, "peak_source": "live DFMA probe (st_probe_fp64)"}
    line = {"metric": metric_name(with_adj), "value": value, "unit": "Mcells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, args.grid), "roofline": roof, "e2e": e2e,
            "clocks": clk.summary(), "gpu_launches": kernels_per_step * args.steps,
            "breakdown": rate_breakdown(cells, res_ms, adj_ms if with_adj else None)}
    if kern_res_tiled:
        t_ms = float(sum(kern_res_tiled.values()))
        line["breakdown"]["residual_tiled"] = cells / (t_ms * 1e-3) / 1e6
        line["breakdown"]["residual_tiled_ms"] = t_ms
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(tb, 12.0, os.cpu_count() or 1, with_adj)
    if world == 1 and tb == "sa" and not args.no_closure:
        eq.close()
        line["closure"] = closure_leg()
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", choices=sorted(GRIDS), default="4097x2049")
    ap.add_argument("--turbulence", choices=["sa", "none"], default="sa")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-closure", action="store_true", help="skip the learned-correction solve")
    ap.add_argument("--residual-only", action="store_true", help="time the residual without the adjoint")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
