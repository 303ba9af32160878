"""The bench's multi-rank path ("replicas only"): barrier and max-over-ranks
timing with world_size 2 on the gloo backend, on CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    r, w, local = bench.dist_setup()
    assert (r, w, local) == (rank, world, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank reports its own "time"; every rank must see the maximum
    got = bench.max_over_ranks(10.0 + rank, w)
    q.put((rank, got))
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 11.0, 1: 11.0}


def test_step_accounting():
    sys.path.insert(0, str(ROOT))
    import bench
    calls = bench.step_calls()
    assert len(calls) == 14  # 5 pass counts x {gather, scatter} + 4 STREAM ops
    n = 1 << 28
    step = sum(bench.call_bytes(c, n) for c, _ in calls)
    assert step == n * (10 * 12 + 8 + 8 + 12 + 12)
    assert sum(bench.call_launches(c, p, "sweep") for c, p in calls) == 2 * 31 + 4
    assert sum(bench.call_launches(c, p, "partition") for c, p in calls) == 2 + 4 * 5 + 4 * 4 + 4
    assert sum(bench.call_launches(c, p, "tiled") for c, p in calls) == 5 * 7 + 5 * 5 + 4
