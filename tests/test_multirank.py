"""The replica aggregation of bench.py across ranks (gloo, two processes on
the CPU): the slowest rank's time, all ranks' work."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    secs, value = bench.aggregate_ranks(1.0 + rank, 1000, dist, "cpu")
    out[rank] = (secs, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        secs, value = res[r]
        assert secs == 2.0 and value == 2 * 1000 / 2.0


def test_single_process_aggregation():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.aggregate_ranks(0.5, 100) == (0.5, 200.0)
