"""The replicas path of bench.py (N > 1): each rank steps its own scene and
the whole-job numbers are the slowest rank's time and the sum of all ranks'
Newton iterations. Checked with two gloo ranks on the CPU."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, n = bench.aggregate(dist, "cpu", 10.0 + 5.0 * rank, 3 + 4 * rank)
    q.put((rank, t, n))
    dist.destroy_process_group()


def test_replicas_aggregate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    out = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t, n in out:
        assert t == pytest.approx(15.0)  # slowest rank
        assert n == 3 + 7                 # all ranks' Newton iterations
