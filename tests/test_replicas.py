"""The multi-GPU form of the frame loop: independent replicas, one per rank, each drawing its own
frames of the spin with no exchange between them; the job's time is the slowest rank's.

Run here as two `gloo` ranks on the CPU: the frame partition the benchmark uses and its
max-over-ranks reduction."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_partition_single_rank():
    assert [bench.rank_frame(0, 1, k, 60) for k in range(62)] == list(range(60)) + [0, 1]


@pytest.mark.parametrize("world", [2, 3, 4, 8])
def test_partition_disjoint_and_complete(world):
    n = bench.SPIN_FRAMES
    steps = n // world
    seen = [bench.rank_frame(r, world, k, n) for r in range(world) for k in range(steps)]
    assert len(set(seen)) == len(seen) == steps * world       # no frame drawn twice in a pass
    assert set(seen) == set(range(steps * world))             # consecutive frames of the spin


def test_max_over_ranks_without_group():
    assert bench.max_over_ranks(None, 1.25, "cpu") == 1.25


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, steps, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        frames = [bench.rank_frame(rank, world, k, bench.SPIN_FRAMES) for k in range(steps)]
        seconds = 0.5 + rank  # rank 1 is the slow one
        job = bench.max_over_ranks(dist, seconds, "cpu")
        got = [None] * world
        dist.all_gather_object(got, frames)
        q.put((rank, job, got))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world, steps = 2, 40
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, job, got in out:
        assert job == 1.5                       # every rank sees the slowest rank's time
        a, b = got
        assert a[:30] == list(range(0, 60, 2)) and b[:30] == list(range(1, 60, 2))
        assert set(a[:30]) | set(b[:30]) == set(range(60))
