"""The C++ sphfdloc drop-in (fdgpu_sphfdloc, fdtomoc_gb300/csrc/fdgpu_sphfdloc.cpp) without a GPU:
its spec and event reading, its time-file loading and its four report files, with the location
oracle plugged in as the locator.  On every golden location case the reports must equal the
reference sphfdloc's byte for byte (the search itself is compared with the GPU's in
tests/test_gpu_locate.py).
"""
import ctypes as C
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

import loc_cases as LC  # noqa: E402
from oracle_util import LocObs, LocResult, loc_lib  # noqa: E402

from fdtomoc_gb300 import lib as L  # noqa: E402


class ProdObs(C.Structure):
    _fields_ = [("field", C.c_int32), ("obstime", C.c_float), ("pwt", C.c_float), ("phase", C.c_char),
                ("good", C.c_char), ("pad", C.c_char * 2)]


LOCATOR = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.POINTER(C.c_float)), C.c_int, C.c_int,
                      C.POINTER(C.c_int), C.POINTER(ProdObs), C.POINTER(C.c_float), C.POINTER(C.c_float),
                      C.POINTER(LocResult))


def _oracle_locator(calls):
    def locate(user, grid, fields, nfields, nev, off, obs, resmin, tps, results):
        olib = loc_lib()
        calls.append(nev)
        for e in range(nev):
            a, b = off[e], off[e + 1]
            arr = (LocObs * (b - a))(*[LocObs(obs[i].field, obs[i].obstime, obs[i].pwt, obs[i].phase,
                                              1 if obs[i].good != b"\x00" else 0) for i in range(a, b)])
            rm = (C.c_float * (b - a))()
            tp = (C.c_float * (b - a))()
            r = LocResult()
            if olib.fdo_locate(C.cast(grid, C.c_void_p), fields, b - a, arr, rm, tp, C.byref(r)) != 0:
                return -1
            results[e] = r
            for i in range(a, b):
                obs[i].good = b"\x01" if arr[i - a].good else b"\x00"
                resmin[i] = rm[i - a]
                tps[i] = tp[i - a]
        return 0
    return LOCATOR(locate)


def _bind():
    lib = L.load()
    lib.fdgpu_sphfdloc.argtypes = [C.c_char_p, LOCATOR, C.c_void_p]
    lib.fdgpu_sphfdloc.restype = C.c_int
    olib = loc_lib()
    olib.fdo_locate.argtypes = [C.c_void_p, C.POINTER(C.POINTER(C.c_float)), C.c_int, C.POINTER(LocObs),
                                C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(LocResult)]
    return lib


@pytest.mark.parametrize("seed", LC.SEEDS)
def test_drop_in_reports_equal_reference(seed, tmp_path):
    lib = _bind()
    p, gold = LC.load_golden(seed)
    spec = LC.write_reference_inputs(p, str(tmp_path))
    calls = []
    assert lib.fdgpu_sphfdloc(spec.encode(), _oracle_locator(calls), None) == 0
    assert calls == [len(p["events"])]
    for k, name in (("fhd", "fhd.txt"), ("dat", "dat.txt"), ("sum", "sum.txt"), ("out", "out.txt")):
        with open(os.path.join(str(tmp_path), "out", name)) as fh:
            assert fh.read() == gold[k], f"{name} differs"


def test_drop_in_missing_time_file(tmp_path):
    lib = _bind()
    p, _ = LC.load_golden(1)
    spec = LC.write_reference_inputs(p, str(tmp_path))
    os.remove(os.path.join(str(tmp_path), "ttimes", p["stations"][0]["name"] + ".ptimes"))
    assert lib.fdgpu_sphfdloc(spec.encode(), _oracle_locator([]), None) == -4


def test_drop_in_refuses_a_marked_input_phase(tmp_path):
    """an input phase marked '*' leaves the reference's parser a blank phase code, and it aborts
    (src/sphfdloc.c:643-650); the drop-in returns FDGPU_EPAR"""
    lib = _bind()
    p, _ = LC.load_golden(1)
    spec = LC.write_reference_inputs(p, str(tmp_path))
    ev = os.path.join(str(tmp_path), "events.txt")
    lines = open(ev).read().split("\n")
    lines[1] = lines[1].replace(" P ", "*P ").replace(" S ", "*S ")
    with open(ev, "w") as fh:
        fh.write("\n".join(lines))
    assert lib.fdgpu_sphfdloc(spec.encode(), _oracle_locator([]), None) == -5
