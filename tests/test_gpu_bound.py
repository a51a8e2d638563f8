"""The single-precision lower bound that lets the solver skip 2-D stencil evaluations must never
exceed the FP64 value it bounds.  Random and near-degenerate stencils (equal times, gradients far
above the slowness, so negative discriminants) over the geometry of configs 1 and 2."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

from fdtomoc_gb300 import build as B
from fdtomoc_gb300 import formats
from fdtomoc_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness():
    out = os.path.join(tempfile.mkdtemp(prefix="fdbound_"), "libbound.so")
    cmd = [B._nvcc()] + B.ARCH + B.NVFLAGS + ["-I" + B.CSRC, "-shared", "-cudart", "static",
                                             os.path.join(HERE, "bound_check.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.bound_check.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    return lib


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [1, 2])
def test_bound_never_exceeds_value(harness, gpu_lib, cfg, tmp_path):
    g, v, sts = W.config(cfg)
    par = tmp_path / "s.par"
    formats.write_par(par, W.par_for(g, sts[0], str(tmp_path / "vp.mod"), "s.ptimes"))
    st, _, _ = gpu_lib.station_from_par("par=" + str(par))
    counts = (C.c_ulonglong * 3)()
    rc = harness.bound_check(st.nx, st.ny, st.nz, st.h, st.dq, st.df, st.z0r, st.y0, 8_000_000, 12345 + cfg, counts)
    assert rc == 0
    viol, tight, usable = counts[0], counts[1], counts[2]
    assert usable > 1_000_000
    assert viol == 0, f"{viol} bounds above the FP64 value"
    # the bound is not vacuous (these random gradients are harsher than a travel-time field's)
    print(f"config {cfg}: {usable} accepted values, {tight} bounded within 1e-4")
    assert tight > 0.05 * usable, (tight, usable)
