"""Multi-GPU runs of bench.py are N independent replicas (the tessellation
path does not shard): the job's time is the slowest rank's and its triangle
count the sum over ranks. Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        seconds, tris = bench.replica_totals(0.5 + rank, 1000.0 * (rank + 1), "cpu")
        q.put((rank, seconds, tris))
    finally:
        dist.destroy_process_group()


def test_replica_totals_with_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, seconds, tris in got:
        assert seconds == 1.5  # the slowest rank
        assert tris == 3000.0  # both ranks' triangles


def test_replica_totals_single_process_is_identity():
    import bench
    assert bench.replica_totals(0.25, 7.0, "cpu") == (0.25, 7.0)
