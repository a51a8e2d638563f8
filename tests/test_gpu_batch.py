"""fdgpu_batch_*: stations prepared once (checks, geometry, records, stats slots), then launched as
often as the caller wants, each launch a single kernel on the caller's stream.  A launch queues no
host work, so it can be captured in a CUDA graph; every replay must give the fields that
fdgpu_solve_device gives for the same stations, bit for bit.
"""
import numpy as np
import pytest

from cases import random_case, write_random_case

pytestmark = pytest.mark.gpu


def _cases(lib, tmp_path, seeds):
    out = []
    for s in seeds:
        c = random_case(s)
        pf = write_random_case(c, str(tmp_path / f"c{s}"))
        st, _, _ = lib.station_from_par("par=" + pf)
        if st.srctype == 1:
            out.append((st, c["vel"]))
    return out


def _slowness(ctx, vel):
    import torch
    v = torch.from_numpy(np.ascontiguousarray(vel).reshape(-1)).cuda()
    slow = torch.empty_like(v)
    ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel())
    return slow


def test_batch_replayed_from_a_cuda_graph(gpu_lib, tmp_path):
    import torch
    lib = gpu_lib
    cases = _cases(lib, tmp_path, range(1, 40))[:6]
    assert len(cases) >= 3
    with lib.Context(0) as ctx:
        for st, vel in cases:
            nz, ny, nx = vel.shape
            slow = _slowness(ctx, vel)
            ref = torch.empty((st.nz, st.ny, st.nx), dtype=torch.float32, device="cuda")
            ref_stats = ctx.solve_device([st], slow.data_ptr(), nx, nx * ny, [ref.data_ptr()])
            torch.cuda.synchronize()

            # the same station twice in one batch, each with its own field
            outs = [torch.full_like(ref, -1.0) for _ in range(2)]
            b = lib.Batch(ctx, [st, st], slow.data_ptr(), nx, nx * ny, [o.data_ptr() for o in outs])
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                b.run(s.cuda_stream)                      # eager launch first
            s.synchronize()
            for o in outs:
                assert torch.equal(o.view(torch.int32), ref.view(torch.int32))

            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    b.run(s.cuda_stream)
            for rep in range(2):
                for o in outs:
                    o.fill_(-1.0)
                torch.cuda.synchronize()
                g.replay()
                torch.cuda.synchronize()
                for k, o in enumerate(outs):
                    assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), f"replay {rep} field {k}"
            stats = b.stats()
            for x in stats:
                assert x["status"] == 0
                assert x["sweeps"] == ref_stats[0]["sweeps"]
            b.close()
            del g


def test_graph_follows_a_model_updated_in_place(gpu_lib, tmp_path):
    """The inversion loop: velocity -> slowness -> solve captured once; each iteration writes a new
    velocity model into the same buffer and replays the graph."""
    import torch
    lib = gpu_lib
    st, vel = _cases(lib, tmp_path, range(1, 40))[0]
    nz, ny, nx = vel.shape
    with lib.Context(0) as ctx:
        v = torch.from_numpy(np.ascontiguousarray(vel).reshape(-1)).cuda()
        slow = torch.empty_like(v)
        out = torch.empty((st.nz, st.ny, st.nx), dtype=torch.float32, device="cuda")
        ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel())
        b = lib.Batch(ctx, [st], slow.data_ptr(), nx, nx * ny, [out.data_ptr()])
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel(), s.cuda_stream)
                b.run(s.cuda_stream)
        rng = np.random.default_rng(7)
        for it in range(3):
            model = (vel * rng.uniform(0.9, 1.1, size=vel.shape)).astype(np.float32)
            v.copy_(torch.from_numpy(model.reshape(-1)))
            torch.cuda.synchronize()
            g.replay()
            torch.cuda.synchronize()
            got = out.clone()
            ref = torch.empty_like(out)
            slow2 = torch.empty_like(v)
            ctx.velocity_to_slowness(v.data_ptr(), slow2.data_ptr(), v.numel())
            ctx.solve_device([st], slow2.data_ptr(), nx, nx * ny, [ref.data_ptr()])
            torch.cuda.synchronize()
            assert torch.equal(got.view(torch.int32), ref.view(torch.int32)), f"iteration {it}"
        assert b.stats()[0]["status"] == 0
        b.close()
        del g


def test_batch_rejects_bad_station(gpu_lib, tmp_path):
    import torch
    lib = gpu_lib
    st, vel = _cases(lib, tmp_path, range(1, 40))[0]
    with lib.Context(0) as ctx:
        slow = _slowness(ctx, vel)
        nz, ny, nx = vel.shape
        bad = lib.Station.from_buffer_copy(st)
        bad.nx = 0
        out = torch.empty(16, dtype=torch.float32, device="cuda")
        with pytest.raises(lib.FdgpuError):
            lib.Batch(ctx, [bad], slow.data_ptr(), nx, nx * ny, [out.data_ptr()])


def test_launch_order_tuned_by_measured_times(gpu_lib, tmp_path):
    """fdgpu_batch_tune_order puts the longest solves of the last run first; any order gives the same
    fields, bit for bit."""
    import torch
    lib = gpu_lib
    cases = _cases(lib, tmp_path, range(1, 60))[:8]
    st0, vel = cases[0]
    nz, ny, nx = vel.shape
    # windows of the first case's model with different sizes and sources
    wins = []
    for k in range(6):
        w = lib.Station.from_buffer_copy(st0)
        w.ox, w.oy, w.oz = k % 2, (k // 2) % 2, 0
        w.nx, w.ny, w.nz = nx - w.ox - (k % 3), ny - w.oy, nz - (k % 2)
        w.xs, w.ys, w.zs = min(st0.xs, w.nx - 1), min(st0.ys, w.ny - 1), min(st0.zs, w.nz - 1)
        wins.append(w)
    with lib.Context(0) as ctx:
        slow = _slowness(ctx, vel)
        outs = [torch.empty((w.nz, w.ny, w.nx), dtype=torch.float32, device="cuda") for w in wins]
        b = lib.Batch(ctx, wins, slow.data_ptr(), nx, nx * ny, [o.data_ptr() for o in outs])
        b.run()
        torch.cuda.synchronize()
        first = [o.clone() for o in outs]
        stats = b.stats()
        dur = [s["t_end_ns"] - s["t_start_ns"] for s in stats]
        b.tune_order()
        order = b.order()
        assert sorted(order) == list(range(len(wins)))
        assert [dur[k] for k in order] == sorted(dur, reverse=True)
        for o in outs:
            o.fill_(-1.0)
        b.run()
        torch.cuda.synchronize()
        for a, o in zip(first, outs):
            assert torch.equal(a.view(torch.int32), o.view(torch.int32))
        b.set_order(list(reversed(order)))
        assert b.order() == list(reversed(order))
        for o in outs:
            o.fill_(-1.0)
        b.run()
        torch.cuda.synchronize()
        for a, o in zip(first, outs):
            assert torch.equal(a.view(torch.int32), o.view(torch.int32))
        with pytest.raises(lib.FdgpuError):
            b.set_order([0] * len(wins))
        b.close()


def test_order_table_saved_and_loaded(gpu_lib, tmp_path):
    """A context records each solve's measured time; saved and loaded into a new context, the table
    orders a new batch of the same stations longest first; the fields are unchanged."""
    import torch
    lib = gpu_lib
    st0, vel = _cases(lib, tmp_path, range(1, 60))[0]
    nz, ny, nx = vel.shape
    wins = []
    for k in range(5):
        w = lib.Station.from_buffer_copy(st0)
        w.ox, w.oy = k % 2, (k // 2) % 2
        w.nx, w.ny, w.nz = nx - w.ox - (k % 3), ny - w.oy, nz - (k % 2)
        w.xs, w.ys, w.zs = min(st0.xs, w.nx - 1), min(st0.ys, w.ny - 1), min(st0.zs, w.nz - 1)
        wins.append(w)
    table = str(tmp_path / "order.bin")
    with lib.Context(0) as ctx:
        slow = _slowness(ctx, vel)
        outs = [torch.empty((w.nz, w.ny, w.nx), dtype=torch.float32, device="cuda") for w in wins]
        stats = ctx.solve_device(wins, slow.data_ptr(), nx, nx * ny, [o.data_ptr() for o in outs])
        torch.cuda.synchronize()
        first = [o.clone() for o in outs]
        ctx.save_order(table)
    dur = [s["t_end_ns"] - s["t_start_ns"] for s in stats]
    with lib.Context(0) as ctx:
        ctx.load_order(table)
        slow = _slowness(ctx, vel)
        b = lib.Batch(ctx, wins, slow.data_ptr(), nx, nx * ny, [o.data_ptr() for o in outs])
        assert [dur[k] for k in b.order()] == sorted(dur, reverse=True)
        for o in outs:
            o.fill_(-1.0)
        b.run()
        torch.cuda.synchronize()
        for a, o in zip(first, outs):
            assert torch.equal(a.view(torch.int32), o.view(torch.int32))
        b.close()
        with pytest.raises(lib.FdgpuError):
            ctx.load_order(str(tmp_path / "missing.bin"))


def test_batch_run_recorded_once(gpu_lib, tmp_path):
    """A batch run's times enter the order table once: reading the statistics again, or tuning the
    order after reading them, leaves the table as the first read left it."""
    import torch
    lib = gpu_lib
    st0, vel = _cases(lib, tmp_path, range(1, 60))[0]
    nz, ny, nx = vel.shape
    wins = []
    for k in range(4):
        w = lib.Station.from_buffer_copy(st0)
        w.ox, w.oy = k % 2, k // 2
        w.nx, w.ny = nx - w.ox - (k % 3), ny - w.oy
        w.xs, w.ys = min(st0.xs, w.nx - 1), min(st0.ys, w.ny - 1)
        wins.append(w)
    with lib.Context(0) as ctx:
        slow = _slowness(ctx, vel)
        outs = [torch.empty((w.nz, w.ny, w.nx), dtype=torch.float32, device="cuda") for w in wins]
        b = lib.Batch(ctx, wins, slow.data_ptr(), nx, nx * ny, [o.data_ptr() for o in outs])
        tables = []
        for run in range(2):
            b.run()
            b.stats()
            ctx.save_order(str(tmp_path / f"run{run}.bin"))
            tables.append((tmp_path / f"run{run}.bin").read_bytes())
        b.stats()
        ctx.save_order(str(tmp_path / "again.bin"))
        b.tune_order()
        ctx.save_order(str(tmp_path / "tuned.bin"))
        b.close()
    assert (tmp_path / "again.bin").read_bytes() == tables[1]
    assert (tmp_path / "tuned.bin").read_bytes() == tables[1]
