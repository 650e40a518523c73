"""bench.py's multi-rank timing on the CPU: two gloo ranks on 127.0.0.1.  Each rank runs its own
replica of the workload (the path shards by solve, with no collective in the data path); the step
time is the slowest rank's and the whole-job value counts every rank's solves."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")      # rank 1 is the slower one
    v = bench.whole_job_rate(world, 60, t)
    dist.barrier()
    q.put((rank, t, v))
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_step_and_all_solves():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in out:
        assert t == 15.0
        assert v == pytest.approx(2 * 60 / 0.015)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.whole_job_rate(1, 60, 1000.0) == pytest.approx(60.0)
