"""A station solved by a cluster of 1, 2, 4 or 8 CTAs gives the same field, bit for bit, and the
field equals the oracle's: the CTAs share one dependency walk, so their number changes only who
evaluates a node, never what it reads."""
import numpy as np
import pytest

from cases import random_case, write_random_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [4, 13, 21, 33])
def test_cluster_sizes_agree(gpu_lib, seed, tmp_path):
    from oracle_util import run_oracle
    lib = gpu_lib
    c = random_case(seed)
    pf = write_random_case(c, str(tmp_path / "c"))
    st, _, _ = lib.station_from_par("par=" + pf)
    run_oracle(pf, str(tmp_path / "o"))
    ref = np.fromfile(tmp_path / "o" / "case.ptimes", dtype="<f4", offset=232)
    fields = {}
    with lib.Context(0) as ctx:
        for cs in (1, 2, 4, 8):
            ctx.set_cluster(cs)
            (t,), (stats,) = ctx.solve_host([st], c["vel"])
            assert stats["status"] == 0, (cs, stats)
            fields[cs] = t
    for cs, t in fields.items():
        assert np.array_equal(t.reshape(-1).view(np.uint32), ref.reshape(-1).view(np.uint32)), f"{cs} CTAs differ"


def test_cluster_batch(gpu_lib, tmp_path):
    """Eight stations in one launch with two CTAs each equal the same stations with one CTA each."""
    lib = gpu_lib
    c = random_case(101)
    pf = write_random_case(c, str(tmp_path / "c"))
    st0, _, _ = lib.station_from_par("par=" + pf)
    rng = np.random.default_rng(5)
    sts = []
    for _ in range(8):
        w = lib.Station.from_buffer_copy(st0)
        w.xs = int(rng.integers(0, w.nx))
        w.ys = int(rng.integers(0, w.ny))
        w.zs = int(rng.integers(0, min(3, w.nz)))
        sts.append(w)
    with lib.Context(0) as ctx:
        ctx.set_cluster(1)
        one, _ = ctx.solve_host(sts, c["vel"])
        ctx.set_cluster(2)
        two, stats = ctx.solve_host(sts, c["vel"])
    assert all(s["status"] == 0 for s in stats)
    for a, b in zip(one, two):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
