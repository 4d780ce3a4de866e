"""Replica bookkeeping of multi-GPU runs on CPU: two gloo ranks agree on the
slowest rank's time and on the job throughput (no GPU involved)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    from lehrfempp_gb300.replicas import Replicas, dist_env
    r, w, lr = dist_env()
    reps = Replicas(w)
    reps.barrier()
    ms_here = 10.0 + 5.0 * r  # rank 1 is the slow one
    value, ms = reps.throughput(1000, ms_here)
    reps.barrier()
    reps.close()
    q.put((r, w, lr, value, ms))


def test_two_gloo_ranks_take_the_slowest_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, lr, value, ms) in enumerate(out):
        assert (rank, w, lr) == (r, 2, r)
        assert ms == 15.0                         # max over ranks
        assert value == pytest.approx(2 * 1000 / 15e-3)  # all ranks' units / slowest time


def test_single_rank_is_a_no_op():
    from lehrfempp_gb300.replicas import Replicas
    reps = Replicas(1)
    reps.barrier()
    assert reps.throughput(500, 2.0) == (500 / 2e-3, 2.0)
    reps.close()
