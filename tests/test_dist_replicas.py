"""Multi-rank bench aggregation on CPU: two gloo ranks, each timing its own
replica; the job's rate is the summed work over the slowest rank's time."""
from __future__ import annotations

import os
import socket

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import sys

    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank                     # rank 1 is the slower replica
    out[rank] = (bench.reduce_max(ms, world), bench.whole_job_rate(1e6, ms, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_bench():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        slowest, rate = res[r]
        assert slowest == 150.0
        assert rate == pytest.approx(2 * 1e6 / 0.150 * 1e-6)
