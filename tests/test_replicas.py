"""Multi-GPU path of bench.py on the CPU: replicas, two gloo ranks.

The path has no exchange step: each rank propagates its own batch with its
own ASE seeds, and only the timing is combined (the slowest rank's time, the
summed work).  Two processes over gloo (127.0.0.1) check the reduction and
that the replicas draw different noise.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, w = bench.reduce_over_ranks(dist, "cpu", 10.0 + rank, 1000 * (rank + 1))
        q.put((rank, t, w, bench.replica_seed(rank, 2000)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replica_reduction():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, w, _ in results:
        assert t == 11.0 and w == 3000.0  # max of 10 / 11 ms, sum of 1000 + 2000
    assert results[0][3] != results[1][3]


def test_single_process_reduction_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(None, "cpu", 4.5, 7) == (4.5, 7.0)
    assert bench.replica_seed(0, 2000) == 2000
