"""The N > 1 path of the bench: independent replicas, max-over-ranks timing and whole-job throughput,
as world-size-2 gloo process groups on the CPU (127.0.0.1 rendezvous)."""

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, times: list, out):
    import torch.distributed as dist
    from sphexa_gb300 import replicas as R
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        R.barrier(world)
        job = R.max_over_ranks(times[rank], world, "cpu")
        out.put((rank, job, R.job_throughput(1000, 4, world, job)))
        R.barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [12.5, 20.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, job, thr in res:
        assert job == 20.0  # both ranks report the slowest rank's time
        assert thr == pytest.approx(1000 * 4 * 2 / 0.020)


def test_single_rank_needs_no_process_group():
    from sphexa_gb300 import replicas as R
    R.barrier(1)
    assert R.max_over_ranks(7.0, 1) == 7.0
    assert R.job_throughput(10, 2, 1, 1000.0) == pytest.approx(20.0)
