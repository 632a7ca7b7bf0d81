"""The bench's multi-process path on CPU: with one process per GPU (replicas),
rank 0 reports the slowest rank's time and the sum of all ranks' work.  Run
here as two gloo ranks over 127.0.0.1, no GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    class A:
        pass

    w, r, local, dist = bench.init_dist(A())
    try:
        t = bench.gather_max(dist, 1.0 + r)          # per-rank times 1 s and 2 s
        n = bench.gather_sum(dist, 100.0 * (r + 1))  # per-rank work 100 and 200
        out.put((r, w, t, n))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_sum_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[1] for x in res] == [2, 2]
    assert all(x[2] == 2.0 for x in res)
    assert all(x[3] == 300.0 for x in res)
