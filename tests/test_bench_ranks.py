"""The multi-rank reduction of bench.py (replicas, one per GPU) on two gloo
ranks on the CPU: the job time is the slowest rank's and the rate counts the
site updates of every rank."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, mlups = bench.over_ranks(1.0 + rank, 2_000_000, world, dist, "cpu")
    out.put((rank, ms, mlups))
    dist.barrier()
    dist.destroy_process_group()


def test_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, mlups in res:
        # slowest rank: 2 ms; two ranks of 2e6 updates each
        assert ms == 2.0
        assert mlups == pytest.approx(2 * 2_000_000 / 2e-3 / 1e6)


def test_over_ranks_single_rank():
    sys.path.insert(0, ROOT)
    import bench

    ms, mlups = bench.over_ranks(0.5, 1_000_000, 1)
    assert ms == 0.5 and mlups == pytest.approx(2000.0)
