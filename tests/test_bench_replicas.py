"""bench.py's multi-rank bookkeeping (CPU, gloo, world size 2): the chains
shard into independent replicas, so ranks exchange only the timing (max over
ranks) and the mutation counts (sum); the reference arm runs on rank 0 only."""
from __future__ import annotations

import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, done = bench.replica_totals(10.0 + 5.0 * rank, 1000 * (rank + 1), world)
        ref = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0})(), world, rank) if rank == 1 else "skip"
        q.put((rank, ms, done, ref))
    finally:
        dist.destroy_process_group()


def test_replica_totals_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, ms, done) for r, ms, done, _ in out] == [(0, 15.0, 3000), (1, 15.0, 3000)]
    assert out[1][3] is None  # the reference arm is rank 0's alone


def test_single_rank_passthrough():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replica_totals(3.5, 7, 1) == (3.5, 7)


def test_gpus_flag_must_match_world_size():
    """--gpus N without a torchrun world of N ranks is refused, not silently run on one rank."""
    import subprocess
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--gpus", "2", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0
    assert "world size is 1" in r.stderr
