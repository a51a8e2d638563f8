"""The C++ sphrayderv drop-in (fdgpu_sphrayderv, fdtomoc_gb300/csrc/fdgpu_rayderv.cpp) without a GPU:
its spec, station and event reading, its bookkeeping and its six files, with the ray oracle plugged
in as the tracer.  On every golden case the files must equal the reference sphrayderv's byte for byte
(the rays themselves are compared with the GPU's in tests/test_gpu_ray.py).
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

import ray_cases as RC  # noqa: E402
from oracle_util import ray_lib  # noqa: E402

from fdtomoc_gb300 import lib as L  # noqa: E402
from fdtomoc_gb300 import rayderv as R  # noqa: E402

TRACER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(R.RayGrid), C.POINTER(C.POINTER(C.c_float)), C.c_int, C.c_int,
                     C.POINTER(R.RayObs), C.POINTER(R.RayResult), C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                     C.POINTER(C.c_float), C.c_longlong)


def _oracle_tracer(mode, calls):
    def trace(user, g, fields, nfields, nobs, obs, res, off, idx, du, total_cap):
        calls.append(nobs)
        olib = ray_lib()
        grid = g.contents
        cap = R.default_cap(grid)
        rr = (R.RayResult * max(1, nobs))()
        ti = np.zeros(max(1, nobs) * cap, dtype=np.int32)
        tv = np.zeros(max(1, nobs) * cap, dtype=np.float32)
        rc = olib.fdr_trace(g, fields, nobs, obs, mode, R.default_max_seg(grid), cap, rr,
                            ti.ctypes.data_as(C.POINTER(C.c_int)), tv.ctypes.data_as(C.POINTER(C.c_float)))
        if rc:
            return -1
        off[0] = 0
        for o in range(nobs):
            res[o] = rr[o]
            off[o + 1] = off[o] + rr[o].nnz
        if off[nobs] > total_cap:
            return L.FDGPU_ETOOBIG
        for o in range(nobs):
            for q in range(rr[o].nnz):
                idx[off[o] + q] = int(ti[o * cap + q])
                du[off[o] + q] = float(tv[o * cap + q])
        return 0
    return TRACER(trace)


def _bind():
    lib = L.load()
    lib.fdgpu_sphrayderv.argtypes = [C.c_char_p, C.c_int, TRACER, C.c_void_p]
    lib.fdgpu_sphrayderv.restype = C.c_int
    return lib


@pytest.mark.parametrize("seed", RC.SEEDS + RC.EXTRA_SEEDS)
@pytest.mark.parametrize("trig", [0, 1])
def test_drop_in_files_equal_reference(seed, trig, tmp_path):
    lib = _bind()
    spec = RC.write_inputs(RC.make_case(seed), str(tmp_path))
    calls = []
    cb = _oracle_tracer(trig, calls)
    assert lib.fdgpu_sphrayderv(spec.encode(), 1, cb, None) == 0
    assert calls, "the tracer was not called"
    gold = RC.load_golden(seed)
    sp = R.read_spec(spec)
    for name in RC.OUT_FILES:
        with open(sp[name], "rb") as fh:
            assert fh.read() == gold[name], f"{name} differs"


def test_drop_in_refuses_teleseisms(tmp_path):
    lib = _bind()
    spec = RC.write_inputs(RC.make_case(1), str(tmp_path))
    with open(spec) as fh:
        text = fh.read()
    with open(spec, "w") as fh:
        fh.write("dotel 1\n" + text)
    assert lib.fdgpu_sphrayderv(spec.encode(), 1, _oracle_tracer(0, []), None) == -1


def test_drop_in_missing_spec_entry(tmp_path):
    lib = _bind()
    p = tmp_path / "spec"
    p.write_text("nxc 5\nnyc 5\n")
    assert lib.fdgpu_sphrayderv(str(p).encode(), 1, _oracle_tracer(0, []), None) == -5


def test_default_tracer_without_a_device_is_an_error(tmp_path):
    """no CPU fallback: with no GPU, the drop-in's default tracer reports it"""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = L.load()
    lib.fdgpu_sphrayderv.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p]
    spec = RC.write_inputs(RC.make_case(1), str(tmp_path))
    rc = lib.fdgpu_sphrayderv(spec.encode(), 1, None, None)
    assert rc in (-8, -3), rc
