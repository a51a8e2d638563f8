"""Batched solves equal solo solves: stations of different sizes and sources solved in one batch
(packed back to back in one device buffer by the host entry point) give the same fields, bit for
bit, as each station solved alone."""
import numpy as np
import pytest

from cases import random_case, write_random_case

pytestmark = pytest.mark.gpu


def test_batch_equals_alone(gpu_lib, tmp_path):
    lib = gpu_lib
    # windows of one model: different sizes (odd lengths), origins and sources
    model = random_case(101)["vel"]
    nz, ny, nx = model.shape
    stations, solo = [], []
    for k, seed in enumerate([3, 8, 11, 21]):
        c = random_case(seed)
        pf = write_random_case(c, str(tmp_path / f"c{k}"))
        st, _, _ = lib.station_from_par("par=" + pf)
        stations.append((st, c["vel"]))
    with lib.Context(0) as ctx:
        for st, vel in stations:
            (t,), _ = ctx.solve_host([st], vel)
            solo.append(t)
        # the same stations in one batch: each reads its own model, so batch those sharing a model
        # layout by stacking them into one model grid along z is not possible; instead batch the
        # first station's model with windows of itself
        st0, vel0 = stations[0]
        wins = []
        for (ox, oy, oz) in [(0, 0, 0), (1, 0, 0), (0, 1, 1)]:
            w = lib.Station.from_buffer_copy(st0)
            w.nx, w.ny, w.nz = st0.nx - ox, st0.ny - oy, st0.nz - oz
            w.ox, w.oy, w.oz = ox, oy, oz
            w.xs = min(w.xs, w.nx - 1)
            w.ys = min(w.ys, w.ny - 1)
            w.zs = min(w.zs, w.nz - 1)
            wins.append(w)
        batch, stats = ctx.solve_host(wins, vel0)
        for w, b in zip(wins, batch):
            v = np.ascontiguousarray(vel0[w.oz:w.oz + w.nz, w.oy:w.oy + w.ny, w.ox:w.ox + w.nx])
            w2 = lib.Station.from_buffer_copy(w)
            w2.ox = w2.oy = w2.oz = 0
            (alone,), _ = ctx.solve_host([w2], v)
            assert np.array_equal(alone.view(np.uint32), b.view(np.uint32))
    assert all(s["status"] == 0 for s in stats)


def test_multi_station_dropin(gpu_lib, tmp_path):
    """Four par files sharing one velocity file run as one GPU batch through the drop-in parlist
    entry point; each time file equals the oracle's."""
    import os
    from fdtomoc_gb300.formats import read_par, write_par
    from oracle_util import run_oracle
    c = random_case(4)
    base = write_random_case(c, str(tmp_path / "m"))
    par = read_par(base)
    nx, ny, nz = int(par["nx"]), int(par["ny"]), int(par["nz"])
    rng = np.random.default_rng(9)
    pfs = []
    for k in range(4):
        q = dict(par)
        q.pop("floatsrc", None)
        for key in ("xs", "ys", "zs"):
            q.pop(key, None)
        q["floatsrc"] = 0
        q["xs"], q["ys"], q["zs"] = int(rng.integers(0, nx)), int(rng.integers(0, ny)), int(rng.integers(0, nz))
        q["timefile"] = f"s{k}.ptimes"
        pf = str(tmp_path / f"s{k}.par")
        write_par(pf, q)
        pfs.append(pf)
    os.makedirs(tmp_path / "gpu")
    st = gpu_lib.sphfd_parlist(["par=" + p for p in pfs], str(tmp_path / "gpu"))
    assert st == [0, 0, 0, 0]
    for k, pf in enumerate(pfs):
        run_oracle(pf, str(tmp_path / "orc"))
        a = open(tmp_path / "orc" / f"s{k}.ptimes", "rb").read()
        b = open(tmp_path / "gpu" / f"s{k}.ptimes", "rb").read()
        assert a == b, f"station {k} differs"
