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


def _ray_worker(rank, world, port, seed, d, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import ray_cases as RC
    from oracle_util import oracle_trace
    from fdtomoc_gb300 import rayderv as R
    spec = RC.write_inputs(RC.make_case(seed), os.path.join(d, str(rank)))
    traced = []

    def counting(grid, fields, obs, nobs, cap):
        traced.append(nobs)
        return oracle_trace(1)(grid, fields, obs, nobs, cap)

    out = R.run(spec, R.sharded(counting))
    gold = RC.load_golden(seed)
    q.put((rank, traced, all(out[k] == gold[k] for k in RC.OUT_FILES)))
    dist.destroy_process_group()


def test_two_ranks_share_the_rays(tmp_path):
    """sphrayderv's observations split over two ranks, results all-gathered: each rank writes the
    reference's files, and each traced only its own share"""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30600 + os.getpid() % 1000
    ps = [ctx.Process(target=_ray_worker, args=(r, 2, port, 2, str(tmp_path), q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=180) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
    (r0, t0, ok0), (r1, t1, ok1) = got
    assert ok0 and ok1
    assert len(t0) == 1 and len(t1) == 1 and t0[0] > 0 and t1[0] > 0 and abs(t0[0] - t1[0]) <= 1
