"""sphrayderv's rays on the GPU (fdgpu_raytrace) against the oracle (oracle/fd_ray.c) with the same
double-double trig functions: every observation's status, segment count, residual, hypocentre
derivatives and coarse derivatives bit for bit, and the six output files the host side writes from
them.  The oracle's files equal the reference sphrayderv's (tests/test_oracle_ray.py), so the GPU
files are compared with the committed reference files too.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

import ray_cases as RC  # noqa: E402
from oracle_util import oracle_trace  # noqa: E402

from fdtomoc_gb300 import rayderv as R  # noqa: E402

pytestmark = pytest.mark.gpu


def _setup(seed, d):
    p = RC.make_case(seed)
    spec = RC.write_inputs(p, d)
    sp = R.read_spec(spec)
    g, keep = R.grid_from_spec(sp)
    obs, nobs, plan, fields = R.build_observations(sp, g, R.read_stations(sp["stafile"]), R.read_events(sp["locdfil"]))
    return spec, sp, g, keep, obs, nobs, plan, R.load_fields(sp, g, fields)


def _same_rays(a, b, nobs):
    ra, oa, ia, da = a
    rb, ob, ib, db = b
    for o in range(nobs):
        x, y = ra[o], rb[o]
        assert (x.status, x.nseg, x.nnz) == (y.status, y.nseg, y.nnz), f"observation {o}"
        if x.status in (R.RAY_NOTIME, R.RAY_OUTSIDE) and x.nseg == 0:
            continue
        assert np.float64(x.dt).tobytes() == np.float64(y.dt).tobytes(), f"observation {o} dt"
        assert bytes(x.am) == bytes(y.am) and np.float32(x.wet) == np.float32(y.wet), f"observation {o} am"
    assert np.array_equal(oa, ob)
    assert np.array_equal(ia, ib)
    assert np.array_equal(da.view(np.int32), db.view(np.int32))


@pytest.mark.parametrize("seed", RC.SEEDS + RC.EXTRA_SEEDS)
def test_rays_equal_oracle_and_files_equal_reference(gpu_lib, seed, tmp_path):
    spec, sp, g, keep, obs, nobs, plan, fields = _setup(seed, str(tmp_path))
    cap = R.default_cap(g)
    want = oracle_trace(1)(g, fields, obs, nobs, cap)
    with gpu_lib.Context(0) as ctx:
        got = R.gpu_trace(ctx)(g, fields, obs, nobs, cap)
        _same_rays(got, want, nobs)
        out = R.run(spec, R.gpu_trace(ctx))
    gold = RC.load_golden(seed)
    for name in RC.OUT_FILES:
        assert out[name] == gold[name], f"{name} differs"


def test_many_rays_equal_oracle(gpu_lib, tmp_path):
    """every (event, station, phase) of a case, each event repeated at jittered depths: a few
    thousand rays in one launch"""
    spec, sp, g, keep, obs, nobs, plan, fields = _setup(2, str(tmp_path))
    rng = np.random.default_rng(5)
    many = []
    for rep in range(40):
        for o in range(nobs):
            x = R.RayObs.from_buffer_copy(obs[o])
            x.ez = float(np.clip(x.ez + rng.uniform(-1.0, 1.0), g.z0 + 0.1, g.z0 + (g.nz - 2) * g.h))
            many.append(x)
    arr = (R.RayObs * len(many))(*many)
    cap = R.default_cap(g)
    want = oracle_trace(1)(g, fields, arr, len(many), cap)
    with gpu_lib.Context(0) as ctx:
        got = R.gpu_trace(ctx)(g, fields, arr, len(many), cap)
    _same_rays(got, want, len(many))
    assert sum(1 for o in range(len(many)) if got[0][o].status == R.RAY_OK) > len(many) // 2


def test_small_cap_reports_steps(gpu_lib, tmp_path):
    spec, sp, g, keep, obs, nobs, plan, fields = _setup(1, str(tmp_path))
    want = oracle_trace(1)(g, fields, obs, nobs, 4)
    with gpu_lib.Context(0) as ctx:
        got = R.gpu_trace(ctx)(g, fields, obs, nobs, 4)
    _same_rays(got, want, nobs)
    assert any(got[0][o].status == R.RAY_STEPS for o in range(nobs))


def test_cxx_drop_in_on_the_gpu(gpu_lib, tmp_path):
    """fdgpu_sphrayderv with its default tracer (fields to the device, fdgpu_raytrace): the six files
    equal the reference's."""
    import ctypes as C
    lib = gpu_lib.load()
    lib.fdgpu_sphrayderv.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p]
    lib.fdgpu_sphrayderv.restype = C.c_int
    for seed in (2, 3):
        d = tmp_path / str(seed)
        spec = RC.write_inputs(RC.make_case(seed), str(d))
        assert lib.fdgpu_sphrayderv(spec.encode(), 1, None, None) == 0
        sp = R.read_spec(spec)
        gold = RC.load_golden(seed)
        for name in RC.OUT_FILES:
            with open(sp[name], "rb") as fh:
                assert fh.read() == gold[name], f"seed {seed}: {name} differs"
