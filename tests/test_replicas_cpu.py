"""The multi-GPU arrangement of this path is replicas: every rank runs its own solves (or its
share of the batched configuration's independent instances) and no collective touches the
data; the benchmark only combines timings (max over ranks) and work (sum over ranks).  This
exercises that host logic with two gloo ranks on the CPU.
"""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        out = {
            "max": bench.reduce_max(rank + 1.5, dist, "cpu"),
            "sum": bench.reduce_sum(rank + 1, dist, "cpu"),
            # rank r processed 10 (r + 1) units in r + 1 seconds
            "rate": bench.replica_rate(10.0 * (rank + 1), rank + 1.0, dist, "cpu"),
            "part": bench.partition(256, rank, world),
        }
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert res[r]["max"] == 2.5
        assert res[r]["sum"] == 3.0
        assert res[r]["rate"] == pytest.approx(30.0 / 2.0)
    parts = res[0]["part"] + res[1]["part"]
    assert sorted(parts) == list(range(256)) and not set(res[0]["part"]) & set(res[1]["part"])


def test_single_process_helpers_need_no_group():
    import bench
    assert bench.reduce_max(3.0) == 3.0
    assert bench.replica_rate(100.0, 4.0) == 25.0
    assert bench.partition(5, 0, 1) == [0, 1, 2, 3, 4]
