"""Replica bookkeeping over 2 ranks with the gloo backend on CPU: the timing reduction takes
the slowest rank and the whole-job rate counts every rank's units."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE=str(world))
    from opensubdiv_gb300 import replicas
    dist = replicas.init("gloo")
    assert replicas.world() == (rank, rank, world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    worst = replicas.max_over_ranks(dist, ms)
    rate = replicas.job_rate(1000, world, worst / 1e3)
    dist.barrier()
    q.put((rank, worst, rate))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, worst, rate in res:
        assert worst == 15.0
        assert rate == pytest.approx(2 * 1000 / 0.015)


def test_single_process_needs_no_group():
    from opensubdiv_gb300 import replicas
    assert replicas.init("gloo") is None or replicas.world()[2] > 1
    assert replicas.max_over_ranks(None, 3.5) == 3.5
    assert replicas.job_rate(10, 1, 2.0) == 5.0
