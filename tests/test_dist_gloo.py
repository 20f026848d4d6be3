"""Multi-rank host logic of bench.py on CPU: two gloo ranks.

With N GPUs the benchmark runs N independent replicas (the multigrid path
has no exchange between independent solves). What needs checking is the
host side: every rank reaches the barrier, the per-rank time is reduced
with a max over ranks, and rank 0 alone reports.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, w, local = bench.dist_init()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    mine = 10.0 + 5.0 * rank  # rank 1 is the slow one
    got = bench.max_over_ranks(mine, w)
    q.put((rank, got))
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    out = dict(q.get(timeout=5) for _ in range(world))
    assert out == {0: 15.0, 1: 15.0}


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
