"""The multi-process timing logic of bench.py (replicas: one independent instance per
rank, barrier + MAX of the elapsed time), exercised with world size 2 over gloo on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    dist, r, w, lr = bench.dist_init()
    bench.barrier(dist)
    elapsed = 1.0 + rank  # each replica reports its own time
    m = bench.reduce_max(dist, elapsed, lr)
    dist.destroy_process_group()
    q.put((r, w, m))


def test_two_replicas_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r for r, _, _ in res] == [0, 1]
    assert all(w == 2 and m == 2.0 for _, w, m in res)
