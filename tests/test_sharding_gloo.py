"""Multi-GPU runs shard independent work across ranks with no data-path collective: par files
(sphfd's driver) and observations (sphrayderv's rays), gathered once at the end.  Checked with two
gloo ranks on the CPU, with the oracles as the solvers."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _sphfd_worker(rank, world, port, d, q, write):
    """One rank of the sharded sphfd driver, with the oracle as its solver."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle_util import run_oracle
    from fdtomoc_gb300 import driver
    solved = []

    def oracle_solver(entries, outdir):
        for e in entries:
            run_oracle(e[len("par="):], outdir)
        solved.extend(entries)
        return [0] * len(entries)

    st = driver.run_spec(os.path.join(d, "spec"), oracle_solver, write=write)
    q.put((rank, st, solved))
    dist.destroy_process_group()


@pytest.mark.parametrize("write", ["each", "rank0"])
def test_two_ranks_solve_a_parlist(tmp_path, write):
    """sphfd's driver over two ranks: each solves every other par file (P and S of four stations);
    the time files in the timedir, written by each rank for its own stations or sent to rank 0 and
    written there, are the reference binary's files byte for byte (tests/golden/reference_outputs.json)."""
    import hashlib
    import json
    from cases import ps_station_case
    from fdtomoc_gb300 import parfiles
    paths, _, _ = ps_station_case(str(tmp_path / "in"))
    out = tmp_path / "out"
    parfiles.write_parlist(paths, str(tmp_path / "parlist"), str(out), str(tmp_path / "spec"))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    port += 0 if write == "each" else 7
    ps = [ctx.Process(target=_sphfd_worker, args=(r, 2, port, str(tmp_path), q, write)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=300) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
    (r0, st0, s0), (r1, st1, s1) = got
    assert st0 == st1 == [0] * len(paths)
    assert s0 == ["par=" + p for p in paths[0::2]] and s1 == ["par=" + p for p in paths[1::2]]
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_outputs.json")))["ps_stations"]
    files = {f: hashlib.sha256((out / f).read_bytes()).hexdigest() for f in sorted(os.listdir(out))}
    assert files == gold


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


def _ray_shared_worker(rank, world, port, seed, d, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import ray_cases as RC
    from oracle_util import oracle_trace
    from fdtomoc_gb300 import rayderv as R
    if rank == 0:
        RC.write_inputs(RC.make_case(seed), d)   # one rank writes the shared inputs
    dist.barrier()
    spec = os.path.join(d, "spec")
    tr = R.sharded(oracle_trace(1))
    out = R.run(spec, tr)
    gold = RC.load_golden(seed)
    q.put((rank, all(out[k] == gold[k] for k in RC.OUT_FILES), tr.writes()))
    dist.destroy_process_group()


def test_two_ranks_share_one_output_directory(tmp_path):
    """Both ranks run sphrayderv on the same spec and directory: only rank 0 writes the six files,
    which equal the reference's; both ranks return them."""
    import ray_cases as RC
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 31700 + os.getpid() % 1000
    ps = [ctx.Process(target=_ray_shared_worker, args=(r, 2, port, 3, str(tmp_path), q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=180) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
    assert got == [(0, True, True), (1, True, False)]   # rank 1 returns the files, rank 0 alone writes
    gold = RC.load_golden(3)
    from fdtomoc_gb300 import rayderv as R
    sp = R.read_spec(str(tmp_path / "spec"))
    for k in RC.OUT_FILES:
        assert open(sp[k], "rb").read() == gold[k], k
