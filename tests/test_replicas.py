"""The multi-GPU path of the benchmark is replicas only: every rank runs its
own simulation, the timed region is bracketed by barriers and the whole-job
value uses the slowest rank's time.  This checks that host logic with two
gloo ranks on CPU (no GPU, no collective on the data path)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_init()
    bench.barrier(w)
    ms = bench.reduce_max(10.0 + r, w)  # rank r "took" 10 + r ms
    out.put((r, w, ms))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 11.0), (1, 2, 11.0)]
