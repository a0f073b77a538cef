"""The multi-GPU path is replicas only; its cross-rank arithmetic (sum of
units, max of time) is checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from colo import replicas  # noqa: E402


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = 1000.0 * (rank + 1)          # rank r processed 1000 (r+1) candidates
        ms = 10.0 + 5.0 * rank               # in 10 + 5 r ms
        dist.barrier()
        total, slowest = replicas.aggregate(dist, units, ms)
        value = replicas.throughput(dist, units, ms)
        out.put((rank, total, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_sum_units_and_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, slowest, value in res:
        assert total == 3000.0 and slowest == 15.0
        assert value == pytest.approx(3000.0 / 0.015)


def test_single_process_is_the_identity():
    assert replicas.aggregate(None, 5.0, 2.0) == (5.0, 2.0)
    assert replicas.throughput(None, 5.0, 2.0) == pytest.approx(2500.0)
