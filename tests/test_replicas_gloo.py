"""The multi-GPU path of bench.py runs independent replicas (no data-path
collective); its host logic is the barrier plus the max-over-ranks time and
the whole-job rate.  Exercised here with two CPU processes over gloo."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    slowest = bench.max_over_ranks(1.0 + rank, world, device="cpu")  # rank r took 1 + r seconds
    out[rank] = (slowest, bench.job_rate(world, 1_000_000, 10, slowest))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    with mp.Manager() as m:
        out = m.dict()
        procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    assert res[0] == res[1]
    slowest, rate = res[0]
    assert slowest == 2.0
    assert rate == pytest.approx(2 * 1_000_000 * 10 / 2.0 / 1e6)


def test_rate_breakdown():
    import importlib
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    b = bench.rate_breakdown(8_000_000, 16.0, 40.0)
    assert b["residual"] == pytest.approx(500.0)
    assert b["fused_residual_adjoint"] == pytest.approx(200.0)
    assert b["adjoint_increment"] == pytest.approx(8e6 / 24e-3 / 1e6)
    assert "fused_residual_adjoint" not in bench.rate_breakdown(8_000_000, 16.0, None)
