"""The benchmark workloads against the reference binary, every field: the 64 stations of the
201x201x81 workload (config 2) in one launch, and the 500 uneven windows over the 401x401x161 model
(config 3) as one prepared batch.  Each field's SHA-256 and each sweep count must equal the
reference's (tests/golden/headline_reference.json, made by make_headline_golden.py, which also found
the oracle equal to the reference on all 564 solves).  The models are regenerated from their seeds;
their own SHA-256 is checked first, so a generator that produced different bits is reported as such."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def pins():
    return json.load(open(os.path.join(HERE, "golden", "headline_reference.json")))


def _sha(t):
    return hashlib.sha256(t.cpu().numpy().tobytes()).hexdigest()


def test_config2_all_stations(gpu_lib, pins, tmp_path):
    import torch
    from fdtomoc_gb300 import workloads as W
    lib = gpu_lib
    g, v, sts = W.config(2)
    assert hashlib.sha256(np.ascontiguousarray(v, dtype="<f4").tobytes()).hexdigest() == pins["models"]["config2"]
    W.write_case(str(tmp_path), g, v, sts)
    stations = [lib.station_from_par("par=" + str(tmp_path / (s["name"] + ".par")))[0] for s in sts]
    with lib.Context(0) as ctx:
        vd = torch.from_numpy(v.reshape(-1)).cuda()
        slow = torch.empty_like(vd)
        ctx.velocity_to_slowness(vd.data_ptr(), slow.data_ptr(), v.size)
        fields = [torch.empty(s.shape, dtype=torch.float32, device="cuda") for s in stations]
        stats = ctx.solve_device(stations, slow.data_ptr(), g.nx, g.nx * g.ny, [f.data_ptr() for f in fields])
        torch.cuda.synchronize()
    bad = [s["name"] for s, f in zip(sts, fields) if _sha(f) != pins["config2"][s["name"]]["data_sha256"]]
    assert not bad, f"{len(bad)} stations differ from the reference: {bad[:8]}"
    assert [x["sweeps"] for x in stats] == [pins["config2"][s["name"]]["sweeps"] for s in sts]


def test_config3_all_windows(gpu_lib, pins, tmp_path):
    import torch
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_par
    lib = gpu_lib
    g, v, _ = W.config(3)
    assert hashlib.sha256(np.ascontiguousarray(v, dtype="<f4").tobytes()).hexdigest() == pins["models"]["config3"]
    wins = W.config3_windows()
    stations = []
    for w in wins:
        pf = str(tmp_path / (w["name"] + ".par"))
        write_par(pf, W.window_par(g, w, str(tmp_path / "vp.mod"), w["name"] + ".ptimes"))
        st = lib.station_from_par("par=" + pf)[0]
        st.ox, st.oy, st.oz = w["ox"], w["oy"], 0
        stations.append(st)
    with lib.Context(0) as ctx:
        vd = torch.from_numpy(v.reshape(-1)).cuda()
        slow = torch.empty_like(vd)
        ctx.velocity_to_slowness(vd.data_ptr(), slow.data_ptr(), v.size)
        del vd
        fields = [torch.empty(s.shape, dtype=torch.float32, device="cuda") for s in stations]
        b = lib.Batch(ctx, stations, slow.data_ptr(), g.nx, g.nx * g.ny, [f.data_ptr() for f in fields])
        b.run()
        stats = b.stats()
        b.close()
    bad = [w["name"] for w, f in zip(wins, fields) if _sha(f) != pins["config3"][w["name"]]["data_sha256"]]
    assert not bad, f"{len(bad)} windows differ from the reference: {bad[:8]}"
    assert [x["sweeps"] for x in stats] == [pins["config3"][w["name"]]["sweeps"] for w in wins]
