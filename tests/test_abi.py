"""The C ABI without a GPU: the library loads, exports every function include/fdgpu.h declares,
parses par files as sphfd() does, and reports the missing device instead of falling back."""
import ctypes as C
import math
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fdgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fdgpu_\w+)\s*\(", src)))


def test_exports_every_declared_function(gpu_lib):
    lib = C.CDLL(gpu_lib.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n


def test_every_status_has_a_name_and_a_text(gpu_lib):
    """Each FDGPU_* status of include/fdgpu.h has its own fdgpu_strerror text and a name in the
    Python binding's table."""
    src = open(os.path.join(ROOT, "include", "fdgpu.h")).read()
    codes = {int(v): n for n, v in re.findall(r"\b(FDGPU_E\w+)\s*=\s*(-?\d+)", src)}
    assert len(codes) >= 10
    lib = C.CDLL(gpu_lib.LIB_PATH)
    lib.fdgpu_strerror.restype = C.c_char_p
    texts = {lib.fdgpu_strerror(v).decode() for v in codes}
    assert "unknown status" not in texts and len(texts) == len(codes)
    for v, n in codes.items():
        assert gpu_lib.ERRORS[v] == n[len("FDGPU_"):]


def test_no_device_is_an_error_not_a_fallback(gpu_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gpu_lib.FdgpuError, match="ENODEV"):
        gpu_lib.Context(0)


def test_serving_without_device_is_an_error(gpu_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(gpu_lib.FdgpuError, match="ENODEV"):
        gpu_lib.Server(0)


def test_station_from_par_matches_sphfd_setup(gpu_lib, tmp_path):
    """Geocentric set-up of src/sphfd.c:415-509 for the M001 par file."""
    from fdtomoc_gb300.formats import write_par
    pf = tmp_path / "M001.par"
    write_par(pf, dict(fxs="121.37915", fys="23.12651", fzs="-0.198", nx="41.000000", ny="41", nz="31", x0="120.9",
                       y0="23.8", z0="-4.0", h="2.0", timefile="M001.ptimes", velfile="/nonexistent", reverse="50"))
    st, vf, tf = gpu_lib.station_from_par(f"par={pf}")
    assert (st.nx, st.ny, st.nz) == (41, 41, 31) and vf == "/nonexistent" and tf == "M001.ptimes"
    degrad = 3.141592654 / 180.0
    assert st.x0 == 120.9 * degrad
    # dq, df default to h/rearth and h/(rearth sin y0)
    assert st.dq == 2.0 / 6371.0
    assert st.df == abs(2.0 / (6371.0 * math.sin(st.y0)))
    assert 0 <= st.xs < 41 and 0 <= st.ys < 41 and 0 <= st.zs < 31
    assert st.reverse == 50 and st.ncube == 2 and st.maxrad == 99999999


def test_missing_required_parameter(gpu_lib, tmp_path):
    from fdtomoc_gb300.formats import write_par
    pf = tmp_path / "bad.par"
    write_par(pf, dict(nx=10, ny=10, h=1.0, timefile="t", velfile="v"))   # nz missing
    with pytest.raises(gpu_lib.FdgpuError, match="EPAR"):
        gpu_lib.station_from_par(f"par={pf}")


def test_source_outside_grid(gpu_lib, tmp_path):
    from fdtomoc_gb300.formats import write_par
    pf = tmp_path / "out.par"
    write_par(pf, dict(nx=10, ny=10, nz=10, h=1.0, x0=120.5, y0=23.5, z0=0.0, fxs=150.0, fys=23.4, fzs=1.0,
                       timefile="t", velfile="v"))
    with pytest.raises(gpu_lib.FdgpuError, match="ESOURCE"):
        gpu_lib.station_from_par(f"par={pf}")
