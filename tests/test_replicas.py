"""Replica aggregation of bench.py on CPU: two gloo ranks.

The path does not shard (one GPU holds the whole domain), so `bench.py
--gpus N` runs N independent replicas: the whole-job time is the slowest
rank's, and the rate counts every rank's steps.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, e2e = bench.max_over_ranks([100.0 + 10 * rank, 200.0 - 10 * rank])
        out[rank] = (ms, e2e, bench.whole_job_rate(world, 20, ms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        ms, e2e, rate = res[r]
        assert ms == 110.0 and e2e == 200.0
        assert rate == pytest.approx(2 * 20 / 0.110)


def test_single_process_is_identity():
    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    assert bench.whole_job_rate(1, 10, 500.0) == pytest.approx(20.0)
