"""The multi-rank side of bench.py on CPU: two gloo ranks (one process each, as
torchrun starts them) agree on the slowest rank's step time, the whole-job
throughput counts every rank's points, and the reference arm does its work on
rank 0 only."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(2.0 + 3.0 * rank, dist, "cpu")
        q.put((rank, ms, bench.job_mpoints_s(world, 4_000_000, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [5.0, 5.0]
    # 2 ranks x 4M points in 5 ms
    assert all(abs(g[2] - 1600.0) < 1e-9 for g in got)


def test_single_process_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_mpoints_s(1, 4_000_000, 5.0) == 800.0


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, no_extras = 1, 3, True

    assert bench.run_reference(Args(), world=2, rank=1) is None
