"""Multi-GPU runs shard stations across ranks with no data-path collective: each rank takes its
own stations.  Checked with two gloo ranks on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    _, _, sts = bench.workload(rank, 4)
    names = [s["name"] for s in sts]
    out = [None] * world
    dist.all_gather_object(out, names)
    if rank == 0:
        q.put(out)
    dist.destroy_process_group()


def test_two_ranks_take_disjoint_stations():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = q.get(timeout=120)
    for p in ps:
        p.join(timeout=60)
    a, b = out
    assert len(a) == 4 and len(b) == 4 and not set(a) & set(b)
    assert sorted(a + b) == [f"S{i:04d}" for i in range(8)]
