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


def test_roofline_classes_and_arithmetic():
    """bench.roofline_live on a synthetic launch list: outer-block launches
    (K = 256) form the tensor-bound entry, inner ones (K <= 64) the nested
    HBM-bound entry; achieved = algorithmic work / device time."""
    sys.path.insert(0, ROOT)
    import bench
    M = N = 4096
    klist = [(2.0, M, N, 256), (1.0, M, N, 256), (0.5, M, 128, 64), (0.5, 200, N, 64)]
    r = bench.roofline_live(klist, step_seconds=0.1, steps=1)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    flops = 2 * 8.0 * M * N * 256
    assert abs(r["achieved"] - flops / 3.0e-3 / 1e12) < 1e-9 * r["achieved"]
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert r["launches_per_step"] == 2 and abs(r["kernel_share_of_timed_steps"] - 0.03) < 1e-12
    inner = r["inner_launches"]
    assert inner["bound"] == "hbm" and inner["unit"] == "GB/s" and inner["launches_per_step"] == 2
    Kp = 128
    sp = 8.0 if bench.gb_tc_passes() == 3 else 4.0  # bytes per operand element: two split planes or one
    nbytes = (16.0 * M * 128 + sp * (M + 256) * Kp) + (16.0 * 200 * N + sp * (200 + 2 * N) * Kp)
    assert abs(inner["achieved"] - nbytes / 1.0e-3 / 1e9) < 1e-9 * inner["achieved"]
    assert bench.roofline_live([], 0.1, 1) is None


def test_roofline_assembly_arithmetic():
    """bench.roofline_assembly on synthetic timings: pairs per second from the
    recorded launches, issue and FP32-pipe fractions from the committed
    per-pair instruction counts at the sampled SM clock."""
    import ctypes
    import json
    sys.path.insert(0, ROOT)
    import bench
    rec = (ctypes.c_double(500.0), ctypes.c_double(1.0e8), ctypes.c_long(1))
    r = bench.roofline_assembly(rec, {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0})
    assert r["bound"] == "fp32-issue" and r["launches_per_step"] == 1
    assert abs(r["pairs_per_s"] - 2.0e8) < 1e-6
    iss = json.load(open(bench.ASM_ISSUE_FILE))
    slots = 152 * 4 * 2000.0e6
    assert abs(r["issue_frac"] - iss["inst_per_pair"] * 2.0e8 / slots) < 1e-12
    assert abs(r["frac"] - iss["fma_pipe_inst_per_pair"] * 2.0e8 / slots) < 1e-12
    assert 0.0 < r["frac"] < r["issue_frac"] < 1.0
    assert bench.roofline_assembly((ctypes.c_double(0.0), ctypes.c_double(0.0), ctypes.c_long(0)), {}) is None
