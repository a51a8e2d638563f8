"""sphfdloc then sphrayderv, as run.sh runs them, with the two C++ drop-ins (fdgpu_sphfdloc,
fdgpu_sphrayderv) and the oracles plugged in as locator and tracer: the located-event report the
first writes is the event file the second reads, and all ten output files must equal the reference
programs' run in the same order (tests/golden/chain_cases.py).
"""
import ctypes as C
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
sys.path.insert(0, os.path.dirname(__file__))

import chain_cases as CC  # noqa: E402
from test_rayderv_driver import TRACER, _oracle_tracer  # noqa: E402
from test_sphfdloc_driver import LOCATOR, _oracle_locator  # noqa: E402
from test_sphfdloc_driver import _bind as _bind_loc  # noqa: E402



@pytest.mark.parametrize("seed", CC.SEEDS)
@pytest.mark.parametrize("trig", [0, 1])
def test_chain_equals_reference(seed, trig, tmp_path):
    lib = _bind_loc()
    lib.fdgpu_sphrayderv.argtypes = [C.c_char_p, C.c_int, TRACER, C.c_void_p]
    lib.fdgpu_sphrayderv.restype = C.c_int
    p, gold = CC.load_golden(seed)
    d = str(tmp_path)
    spec = CC.write_inputs(p, d)
    assert lib.fdgpu_sphfdloc(spec.encode(), _oracle_locator([]), None) == 0
    assert lib.fdgpu_sphrayderv(spec.encode(), 1, _oracle_tracer(trig, []), None) == 0
    for k, name in CC.LOC_FILES.items():
        with open(os.path.join(d, "out", name), "rb") as fh:
            assert fh.read() == gold[k], f"{name} differs"
    for k, name in CC.RAY_FILES.items():
        with open(os.path.join(d, "ray", name), "rb") as fh:
            assert fh.read() == gold[k], f"{name} differs"
