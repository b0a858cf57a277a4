"""The multi-GPU path of bench.py on CPU: replicas only (each rank renders its
own copy of the workload, no data-path collective), timed as the slowest rank.
Two gloo ranks check the rank bookkeeping and the max-over-ranks timing."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_init(world)
    bench.barrier(w)
    slowest = bench.max_over_ranks(1.0 + rank, w)  # rank 1 is the slower replica
    out.put((r, w, local, slowest))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[:3] for r in results] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == 2.0 for r in results)
