"""The C++ sphfdloc drop-in (fdgpu_sphfdloc) with its default locator: the golden cases' fields go to
the device and fdgpu_locate searches them; the four reports must equal the reference sphfdloc's.

This file sorts after every other test, so that a run stopping at the first failure has run the
rest first.
"""
import ctypes as C

import pytest

import loc_cases as LC

pytestmark = pytest.mark.gpu


def test_cxx_sphfdloc_drop_in_on_the_gpu(gpu_lib, tmp_path):
    lib = gpu_lib.load()
    lib.fdgpu_sphfdloc.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    lib.fdgpu_sphfdloc.restype = C.c_int
    for seed in (1, 5):
        p, gold = LC.load_golden(seed)
        d = tmp_path / str(seed)
        spec = LC.write_reference_inputs(p, str(d))
        assert lib.fdgpu_sphfdloc(spec.encode(), None, None) == 0
        for k, name in (("fhd", "fhd.txt"), ("dat", "dat.txt"), ("sum", "sum.txt"), ("out", "out.txt")):
            assert (d / "out" / name).read_text() == gold[k], f"seed {seed}: {name} differs"
