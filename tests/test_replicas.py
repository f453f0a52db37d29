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


_RANK_SCRIPT = """
import json, os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank, world, local = bench.dist_env()
dist.init_process_group("gloo")
seconds, tris = bench.replica_totals(0.5 + rank, 1000.0 * (rank + 1), "cpu")
dist.barrier()
if rank == 0:
    print(json.dumps({{"n_gpus": world, "local_rank": local, "seconds": seconds, "tris": tris}}))
dist.destroy_process_group()
"""


def test_spawn_path_runs_two_gloo_replicas(tmp_path, capfd):
    """bench.py --gpus N without torchrun spawns N ranks with torchrun's
    environment; here two gloo ranks on the CPU run the replica reduction and
    rank 0 alone prints."""
    import json

    import bench
    script = tmp_path / "rank.py"
    script.write_text(_RANK_SCRIPT.format(root=os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    import sys
    assert bench.spawn_replicas([sys.executable, str(script)], 2) == 0
    out = [line for line in capfd.readouterr().out.splitlines() if line.startswith("{")]
    assert len(out) == 1
    got = json.loads(out[0])
    assert got == {"n_gpus": 2, "local_rank": 0, "seconds": 1.5, "tris": 3000.0}
