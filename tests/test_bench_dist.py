"""Multi-process host logic of bench.py on CPU: world_size 2 with gloo --
barrier and max-over-ranks of the step time (replicas, no data exchange)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      BENCH_BACKEND="gloo", LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w = bench.dist_init()
    bench.dist_barrier(dist)
    m = bench.dist_max(dist, float(rank + 1) * 0.5)
    q.put((r, w, m))
    dist.destroy_process_group()


def test_two_rank_max_reduction():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert [r[:2] for r in res] == [(0, 2), (1, 2)]
    assert all(abs(r[2] - 1.0) < 1e-15 for r in res)
