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


def _replica_rank(rank, world, port, q, n):
    """One replica: price this rank's own seeded shard (the oracle's NT2
    Black-Scholes on the host cores), time it, and report the checksum; the
    only cross-rank traffic is the timing max and the test's gather."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      OMP_NUM_THREADS="2")
    import time

    import numpy as np
    import torch

    import bench
    from oracle import oracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(1000 + rank)
        S = rng.uniform(5, 30, n).astype(np.float32)
        K = rng.uniform(1, 100, n).astype(np.float32)
        T = rng.uniform(0.25, 10, n).astype(np.float32)
        dist.barrier()
        t0 = time.perf_counter()
        c, p = oracle.blackscholes(S, K, T, 0.02, 0.30, nthreads=2)
        ms = 1e3 * (time.perf_counter() - t0)
        slowest = bench.max_over_ranks(ms, world, dist)
        value = bench.whole_job_value(n, 1, world, slowest)
        sums = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(sums, torch.tensor([float(np.sum(c, dtype=np.float64)), float(np.sum(p, dtype=np.float64))],
                                           dtype=torch.float64))
        q.put((rank, ms, slowest, value, [s.tolist() for s in sums]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_run_their_own_shards():
    """Two gloo ranks each price their own batch (seeded by rank) as the bench's
    replicas do: every shard's result equals the single-process evaluation of
    the same shard, the reported time is the slowest rank's, and the value
    counts both ranks' options."""
    import numpy as np

    from oracle import oracle
    n = 1 << 16
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_rank, args=(r, 2, port, q, n)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    times = [g[1] for g in got]
    for rank, ms, slowest, value, sums in got:
        assert slowest == max(times)
        assert value == pytest.approx(2 * n / (slowest * 1e-3))
        for r in range(2):  # each shard as one process computes it
            rng = np.random.default_rng(1000 + r)
            S = rng.uniform(5, 30, n).astype(np.float32)
            K = rng.uniform(1, 100, n).astype(np.float32)
            T = rng.uniform(0.25, 10, n).astype(np.float32)
            c, p = oracle.blackscholes(S, K, T, 0.02, 0.30, nthreads=1)
            assert sums[r] == [float(np.sum(c, dtype=np.float64)), float(np.sum(p, dtype=np.float64))]


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference launched by torch.distributed.run on two
    ranks (127.0.0.1 rendezvous): rank 0 times NT2's CPU path and prints one
    JSON line; rank 1 exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "3", "--config", "bs"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run(cmd, cwd=root, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
