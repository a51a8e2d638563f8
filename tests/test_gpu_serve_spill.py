"""Fields of many stations kept on the device up to a budget and spilled to pinned host memory
beyond it (fdtomoc_gb300.fieldstore), solved by a serving session: with a budget of three fields for
ten stations, some fields stay on the device, the oldest finished ones are spilled, later ones go
straight to host memory, and every field equals the same station solved in one batch, bit for
bit.  P and S requests share the session (S = P/1.73)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_spill_keeps_every_field_exact(gpu_lib, tmp_path):
    import torch
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.fieldstore import FieldStore
    lib = gpu_lib
    g, v, _ = W.config(1)
    sts = W.stations(g, 5, 11)
    W.write_case(str(tmp_path), g, v, sts)
    stations = [lib.station_from_par("par=" + str(tmp_path / (s["name"] + ".par")))[0] for s in sts]
    vs = (v / np.float32(1.73)).astype(np.float32)
    field_bytes = 4 * g.nx * g.ny * g.nz
    with lib.Context(0) as ctx:
        want = {}
        for ph, model in ((0, v), (1, vs)):
            (fields, stats) = ctx.solve_host(stations, model)
            assert all(s["status"] == 0 for s in stats)
            for k, f in enumerate(fields):
                want[(k, ph)] = f
    with lib.Server(0, hbm_bytes=1 << 30, max_inflight=4) as sv:
        sv.set_model(0, v)
        sv.set_model(1, vs)
        store = FieldStore(sv, 3 * field_bytes)
        for k, st in enumerate(stations):
            for ph in (0, 1):
                store.submit((k, ph), st, ph)
                # each request finished before the next one: the fields are placed deterministically
                # (the first three on the device, then each new one spills the oldest)
                while (k, ph) not in store.results:
                    store.poll(16, 1000)
        store.drain(60000)
        assert all(r["status"] == 0 for r in store.results.values())
        places = {key: store.where(key) for key in want}
        assert sum(p == "device" for p in places.values()) == 3
        assert store.spilled == len(want) - 3 and store.direct_to_host == 0
        assert all(places[key] == "device" for key in [(3, 1), (4, 0), (4, 1)])
        for key, f in want.items():
            got = store.get(key)
            got = got.cpu().numpy() if got.is_cuda else got.numpy()
            assert np.array_equal(got.view(np.uint32), f.view(np.uint32)), key
