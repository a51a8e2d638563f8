"""The drop-in boundary on the GPU, against the reference binary's own outputs
(tests/golden/reference_outputs.json, made by make_golden.py):

- one inversion iteration's P and S par files, in make_par_file's dialect and sharing VP.mod and
  VS.mod, through the parlist entry point, the drop-in executable (spec on stdin, as run.sh runs
  sphfd) and the per-station sphfd() replacement;
- byte-swapped models and time files (swab 1, 2, 3);
- windows of one model at odd offsets, so that fields and model windows start at addresses that
  are not 16-byte aligned: each equals the same window solved alone (the regression test of the
  misaligned-address fault that an early field initialisation had);
- a velocity file without the "HEAD" header, against the oracle (the reference itself aborts
  there under _FORTIFY_SOURCE).
"""
import ctypes as C
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from cases import SWAB_SEEDS, ps_station_case, random_case, write_random_case, write_swab_case

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "reference_outputs.json")))


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def test_ps_stations_through_the_parlist_entry_point(gpu_lib, tmp_path):
    paths, _, _ = ps_station_case(str(tmp_path / "in"))
    out = tmp_path / "out"
    os.makedirs(out)
    st = gpu_lib.sphfd_parlist(["par=" + p for p in paths], str(out))
    assert st == [0] * len(paths)
    got = {f: _sha(out / f) for f in sorted(os.listdir(out))}
    assert got == GOLD["ps_stations"]


def test_ps_stations_through_the_drop_in_executable(gpu_lib, tmp_path):
    from fdtomoc_gb300 import build, parfiles
    paths, _, _ = ps_station_case(str(tmp_path / "in"))
    out = tmp_path / "out"
    os.makedirs(out)
    spec = parfiles.write_parlist(paths, str(tmp_path / "parlist"), str(out), str(tmp_path / "spec"))
    r = subprocess.run([build.EXE], input=spec + "\n", capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got = {f: _sha(out / f) for f in sorted(os.listdir(out))}
    assert got == GOLD["ps_stations"]


def test_per_station_sphfd_replacement(gpu_lib, tmp_path):
    """fdgpu_sphfd(ac, av, output_path), called as the reference's main calls sphfd()."""
    paths, _, _ = ps_station_case(str(tmp_path / "in"))
    lib = C.CDLL(gpu_lib.LIB_PATH)
    lib.fdgpu_sphfd.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p]
    out = tmp_path / "out"
    os.makedirs(out)
    for p in paths[:3]:
        av = (C.c_char_p * 2)(b"sphfd", ("par=" + p).encode())
        assert lib.fdgpu_sphfd(2, av, str(out).encode()) == 0
    got = {f: _sha(out / f) for f in sorted(os.listdir(out))}
    assert got == {k: v for k, v in GOLD["ps_stations"].items() if k in got} and len(got) == 3


@pytest.mark.parametrize("seed", SWAB_SEEDS)
@pytest.mark.parametrize("swab", [1, 2, 3])
def test_swab(gpu_lib, tmp_path, seed, swab):
    pf = write_swab_case(random_case(seed), str(tmp_path / "in"), swab)
    out = tmp_path / "out"
    os.makedirs(out)
    assert gpu_lib.sphfd_parlist(["par=" + pf], str(out)) == [0]
    assert _sha(out / "case.ptimes") == GOLD["swab_cases"][f"{seed}_{swab}"]["sha256"]


def test_velocity_file_without_header(gpu_lib, tmp_path):
    from oracle_util import run_oracle
    c = random_case(8)
    pf = write_random_case(c, str(tmp_path / "in"))
    (tmp_path / "in" / "vp.mod").write_bytes(np.ascontiguousarray(c["vel"], dtype="<f4").tobytes())
    run_oracle(pf, str(tmp_path / "orc"))
    out = tmp_path / "out"
    os.makedirs(out)
    assert gpu_lib.sphfd_parlist(["par=" + pf], str(out)) == [0]
    assert (out / "case.ptimes").read_bytes() == (tmp_path / "orc" / "case.ptimes").read_bytes()


def _window(lib, st0, ox, oy, oz, dx, dy, dz):
    w = lib.Station.from_buffer_copy(st0)
    w.nx, w.ny, w.nz = st0.nx - ox - dx, st0.ny - oy - dy, st0.nz - oz - dz
    w.ox, w.oy, w.oz = ox, oy, oz
    w.xs = min(max(w.xs - ox, 0), w.nx - 1)
    w.ys = min(max(w.ys - oy, 0), w.ny - 1)
    w.zs = min(max(w.zs - oz, 0), w.nz - 1)
    return w


def test_batch_equals_alone(gpu_lib, tmp_path):
    """Windows at odd offsets of one model, solved in one batch (host buffers: the fields are packed
    back to back, so most start off a 16-byte boundary; device buffers: each field one float past
    an aligned address), equal each window solved alone on its own cut of the model."""
    import torch
    lib = gpu_lib
    c = random_case(101)
    vel = c["vel"]
    nz, ny, nx = vel.shape
    pf = write_random_case(c, str(tmp_path / "m"))
    st0, _, _ = lib.station_from_par("par=" + pf)
    if st0.srctype != 1 or min(nx, ny, nz) < 8:
        pytest.skip("case 101 is not a point source on a large enough grid")
    wins = [_window(lib, st0, *o) for o in [(0, 0, 0, 0, 0, 0), (1, 0, 0, 0, 1, 0), (0, 1, 1, 1, 0, 0),
                                            (1, 2, 1, 2, 1, 1), (3, 1, 2, 0, 0, 1)]]
    with lib.Context(0) as ctx:
        batch, stats = ctx.solve_host(wins, vel)
        assert all(s["status"] == 0 for s in stats)
        alone = []
        for w in wins:
            v = np.ascontiguousarray(vel[w.oz:w.oz + w.nz, w.oy:w.oy + w.ny, w.ox:w.ox + w.nx])
            w2 = lib.Station.from_buffer_copy(w)
            w2.ox = w2.oy = w2.oz = 0
            (t,), (s,) = ctx.solve_host([w2], v)
            assert s["status"] == 0
            alone.append(t)
        for k, (a, b) in enumerate(zip(alone, batch)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"window {k} (host buffers)"
        # device buffers: the model in place, each field one float past an aligned address
        v = torch.from_numpy(np.ascontiguousarray(vel).reshape(-1)).cuda()
        slow = torch.empty_like(v)
        ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel())
        bufs = [torch.empty(w.nx * w.ny * w.nz + 4, dtype=torch.float32, device="cuda") for w in wins]
        ptrs = [b.data_ptr() + 4 for b in bufs]
        stats = ctx.solve_device(wins, slow.data_ptr(), nx, nx * ny, ptrs)
        torch.cuda.synchronize()
        assert all(s["status"] == 0 for s in stats)
        for k, (a, b, w) in enumerate(zip(alone, bufs, wins)):
            got = b[1:1 + w.nx * w.ny * w.nz].cpu().numpy()
            assert np.array_equal(a.reshape(-1).view(np.uint32), got.view(np.uint32)), f"window {k} (device)"


def test_ps_stations_over_a_device_list(gpu_lib, tmp_path):
    """fdgpu_sphfd_parlist_devices with device 0 listed twice: two worker threads, each with its own
    context on the one GPU, share the stations of each velocity file; the files are the reference's."""
    paths, _, _ = ps_station_case(str(tmp_path / "in"))
    out = tmp_path / "out"
    os.makedirs(out)
    st = gpu_lib.sphfd_parlist(["par=" + p for p in paths], str(out), devices=[0, 0])
    assert st == [0] * len(paths)
    got = {f: _sha(out / f) for f in sorted(os.listdir(out))}
    assert got == GOLD["ps_stations"]
    with pytest.raises(gpu_lib.FdgpuError):
        gpu_lib.sphfd_parlist(["par=" + paths[0]], str(out), devices=[0, 4096])
