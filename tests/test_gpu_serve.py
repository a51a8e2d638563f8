"""The serving session: requests of mixed window sizes arrive while others run, are admitted as
request slots and session memory free up, and each result is bit-identical to the same station
solved alone by the batch entry point (itself bit-identical to the oracle, see test_gpu_parity).
Model updates are versioned: requests keep the model they were submitted against."""
import time

import numpy as np
import pytest

from fdtomoc_gb300 import formats
from fdtomoc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def base_station(lib, tmp_path, cfg=1):
    g, v, sts = W.config(cfg)
    par = tmp_path / "base.par"
    formats.write_par(par, W.par_for(g, sts[0], str(tmp_path / "vp.mod"), "s.ptimes"))
    st, _, _ = lib.station_from_par("par=" + str(par))
    return st, v


def window(lib, st0, nx, ny, nz, ox, oy, oz, xs, ys, zs):
    """A sub-grid of the base station's grid: its own origin (so its own geometry tables) and an
    integer-node source inside it."""
    w = lib.Station.from_buffer_copy(st0)
    w.nx, w.ny, w.nz = nx, ny, nz
    w.ox, w.oy, w.oz = ox, oy, oz
    w.x0 = st0.x0 + st0.df * ox
    w.y0 = st0.y0 + st0.dq * oy
    w.z0r = st0.z0r - st0.h * oz
    w.xs, w.ys, w.zs = xs, ys, zs
    w.src_geo[0] = w.x0 + w.df * xs
    w.src_geo[1] = w.y0 + w.dq * ys
    w.src_geo[2] = w.z0r - w.h * zs
    return w


def random_windows(lib, st0, n, seed, lo=(12, 12, 8)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(lo[0], st0.nx + 1))
        ny = int(rng.integers(lo[1], st0.ny + 1))
        nz = int(rng.integers(lo[2], st0.nz + 1))
        ox, oy, oz = (int(rng.integers(0, m - k + 1)) for m, k in ((st0.nx, nx), (st0.ny, ny), (st0.nz, nz)))
        xs, ys = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        zs = int(rng.integers(0, min(nz, 4)))
        out.append(window(lib, st0, nx, ny, nz, ox, oy, oz, xs, ys, zs))
    return out


def solve_alone(ctx, st, vel):
    (t,), (s,) = ctx.solve_host([st], vel)
    assert s["status"] == 0
    return t


def work_bytes(st):
    """Device bytes one request holds: field, face scratch and sweep-graph arrays, geometry tables
    (the accounting of fdgpu_station.h, rounded up)."""
    nn = st.nx * st.ny * st.nz
    mf = max(st.nx * st.ny, st.nx * st.nz, st.ny * st.nz)
    return 4 * nn + 34 * (mf + 16) + 17 * nn + (st.nx + st.ny + st.nz + 8) * 48 + (8 + 8) * 65536 + 4 * 262144 \
        + 8 * (st.ny + 3 * st.nz + 9 * st.nz * st.ny + 72 * st.nz * st.ny) + 8 * 256


def test_served_equals_alone_under_memory_pressure(gpu_lib, tmp_path):
    import torch
    lib = gpu_lib
    st0, vel = base_station(lib, tmp_path)
    wins = random_windows(lib, st0, 24, seed=5)
    with lib.Context(0) as ctx:
        alone = [solve_alone(ctx, w, vel) for w in wins]
    # room for about three of the largest requests beside the model: admission must queue
    budget = 4 * vel.size + 3 * max(work_bytes(w) for w in wins)
    outs = []
    with lib.Server(0, hbm_bytes=budget, max_inflight=8) as sv:
        sv.set_model(0, vel)
        ids = {}
        for k, w in enumerate(wins):
            kind = k % 3
            if kind == 0:
                out = np.full(w.shape, -1.0, dtype=np.float32)          # pageable host memory
            elif kind == 1:
                out = torch.full(w.shape, -1.0, dtype=torch.float32).pin_memory()
            else:
                out = torch.full(w.shape, -1.0, dtype=torch.float32, device="cuda")
            outs.append(out)
            ids[sv.submit(w, 0, out, tag=k)] = k
            if k % 5 == 4:
                time.sleep(0.01)   # arrivals spread over the running work
        sv.drain(120000)
        res = sv.poll(256)
        m = sv.metrics()
    assert len(res) == len(wins)
    for r in res:
        assert r["status"] == 0, r
        k = ids[r["id"]]
        assert r["tag"] == k and r["model_version"] == 1
        o = outs[k]
        got = o.cpu().numpy() if hasattr(o, "cpu") else o
        assert np.array_equal(got.view(np.uint32), alone[k].view(np.uint32)), k
    assert m["completed"] == len(wins) and m["failed"] == 0
    assert m["hbm_peak"] <= budget
    assert m["p99_ms"] >= m["p50_ms"] > 0
    assert sum(m["hist"]) == len(wins)


def test_model_update_keeps_submitted_version(gpu_lib, tmp_path):
    lib = gpu_lib
    st0, vel = base_station(lib, tmp_path)
    vel2 = (vel * (1.0 + 0.01 * W.smooth_noise(vel.shape, (1.0, 1.1, 1.0), 5.0, 77))).astype(np.float32)
    wins = random_windows(lib, st0, 8, seed=9)
    with lib.Context(0) as ctx:
        a1 = [solve_alone(ctx, w, vel) for w in wins]
        a2 = [solve_alone(ctx, w, vel2) for w in wins]
    o1 = [np.empty(w.shape, np.float32) for w in wins]
    o2 = [np.empty(w.shape, np.float32) for w in wins]
    with lib.Server(0, hbm_bytes=1 << 30) as sv:
        assert sv.set_model(0, vel) == 1
        i1 = [sv.submit(w, 0, o) for w, o in zip(wins, o1)]
        assert sv.set_model(0, vel2) == 2          # while the first requests run
        i2 = [sv.submit(w, 0, o) for w, o in zip(wins, o2)]
        sv.drain(120000)
        res = {r["id"]: r for r in sv.poll(64)}
    for k in range(len(wins)):
        assert res[i1[k]]["model_version"] == 1 and res[i2[k]]["model_version"] == 2
        assert np.array_equal(o1[k].view(np.uint32), a1[k].view(np.uint32))
        assert np.array_equal(o2[k].view(np.uint32), a2[k].view(np.uint32))
    assert not all(np.array_equal(x, y) for x, y in zip(a1, a2))


def test_restart_from_supplied_field(gpu_lib, tmp_path):
    """srctype 3: the starting field comes with the request (host or device memory)."""
    import torch
    lib = gpu_lib
    st0, vel = base_station(lib, tmp_path)
    w = random_windows(lib, st0, 1, seed=13)[0]
    with lib.Context(0) as ctx:
        first = solve_alone(ctx, w, vel)
        r = lib.Station.from_buffer_copy(w)
        r.srctype, r.srcwall = 3, 5
        init = first.copy()
        init[1:] = 1.0e10            # only the top wall holds times
        (want,), (s,) = ctx.solve_host([r], vel, init_times=[init])
        assert s["status"] == 0
    with lib.Server(0, hbm_bytes=1 << 30) as sv:
        sv.set_model(0, vel)
        out_h = np.empty(w.shape, np.float32)
        out_d = torch.empty(w.shape, dtype=torch.float32, device="cuda")
        sv.submit(r, 0, out_h, init=init)
        sv.submit(r, 0, out_d, init=torch.from_numpy(init).cuda())
        sv.drain(120000)
        res = sv.poll(8)
    assert [x["status"] for x in res] == [0, 0]
    assert np.array_equal(out_h.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(out_d.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_grid_stops_when_idle_and_comes_back(gpu_lib, tmp_path):
    lib = gpu_lib
    st0, vel = base_station(lib, tmp_path)
    wins = random_windows(lib, st0, 2, seed=21)
    with lib.Context(0) as ctx:
        alone = [solve_alone(ctx, w, vel) for w in wins]
    with lib.Server(0, hbm_bytes=1 << 30, idle_stop_us=500) as sv:
        sv.set_model(0, vel)
        outs = [np.empty(w.shape, np.float32) for w in wins]
        sv.submit(wins[0], 0, outs[0])
        sv.drain(120000)
        time.sleep(0.05)
        sv.submit(wins[1], 0, outs[1])
        sv.drain(120000)
        res = sv.poll(8)
        m = sv.metrics()
    assert [x["status"] for x in res] == [0, 0]
    assert m["grid_launches"] >= 2
    for o, a in zip(outs, alone):
        assert np.array_equal(o.view(np.uint32), a.view(np.uint32))


def test_rejects_what_cannot_fit(gpu_lib, tmp_path):
    lib = gpu_lib
    st0, vel = base_station(lib, tmp_path)
    with lib.Server(0, hbm_bytes=4 * vel.size + (1 << 20)) as sv:
        sv.set_model(0, vel)
        with pytest.raises(lib.FdgpuError, match="ETOOBIG"):
            sv.submit(st0, 0, np.empty(st0.shape, np.float32))
        w = lib.Station.from_buffer_copy(st0)
        w.nx = st0.nx + 1      # window outside the model
        with pytest.raises(lib.FdgpuError, match="EINVAL"):
            sv.submit(w, 0, np.empty(w.shape, np.float32))
        with pytest.raises(lib.FdgpuError, match="EINVAL"):
            sv.submit(st0, 1, np.empty(st0.shape, np.float32))    # model slot 1 never set
