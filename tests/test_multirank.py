"""The N>1 path of bench.py on CPU: two gloo ranks run as replicas (each its
own batch, no data-path collective); the reported time is the slowest rank's
and the value counts every rank's elements."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [4.0, 7.5][rank]  # rank 1 is slower
        slowest = bench.max_over_ranks(ms, world, dist)
        value = bench.whole_job_value(1000, 10, world, slowest)
        dist.barrier()
        q.put((rank, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, slowest, value in got:
        assert slowest == 7.5
        assert value == pytest.approx(2 * 1000 * 10 / 7.5e-3)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.whole_job_value(1 << 20, 50, 1, 5.0) == pytest.approx((1 << 20) * 50 / 5e-3)
