"""The bench's multi-rank host logic (replicas, barrier, max-over-ranks
timing) on two gloo ranks on CPU; the GPU data path has no collective."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    w, r, local, pg = bench.dist_setup(backend="gloo")
    ms = 10.0 + 5.0 * r  # rank 1 is slower
    pg.barrier()
    m = bench.barrier_max(pg, ms, "cpu")
    v = bench.aggregate_value(1000, w, m)
    q.put((r, w, m, v))
    pg.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert [x[1] for x in res] == [2, 2]
    assert all(x[2] == 15.0 for x in res)  # max over ranks
    assert all(abs(x[3] - 2000 / 0.015) < 1e-6 for x in res)  # whole-job pairs/s
