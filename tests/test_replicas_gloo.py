"""The N > 1 path of bench.py on CPU: world_size-2 gloo ranks agree on the
slowest rank's time and on the whole-job throughput (replicas: every rank
answers its own query batch, no data-path collective)."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    worst = bench._max_over_ranks(torch, world, local_ms, device="cpu")
    out[rank] = (worst, bench.aggregate_qps(world, 10000, 5, worst))
    torch.distributed.destroy_process_group()


def test_two_rank_max_and_throughput():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    port = _free_port()
    ctx = tmp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1]
    assert res[0][0] == 150.0
    assert res[0][1] == pytest.approx(2 * 10000 * 5 / 0.150)
