"""The c2f oracle against the reference's own c2f: for the seeded coarse models of
tests/golden/c2f_cases.py the oracle's fine model has the SHA-256 the reference's three output files'
data had (tests/golden/c2f_reference.json, made by make_c2f_golden.py)."""
import pytest

import c2f_cases as CC
from oracle_util import oracle_c2f

GOLD = CC.load_golden()


@pytest.mark.parametrize("seed", CC.SEEDS)
def test_oracle_reproduces_reference_c2f(seed):
    g = GOLD[str(seed)]
    p = g["case"]
    fine = oracle_c2f(p, CC.coarse_model(p))
    d = CC.digests(fine)
    assert d == {"fine": g["fine"], "pvel": g["pvel"], "svel": g["svel"]}


def test_library_c2f_dims_and_argument_checks(gpu_lib):
    """fdgpu_c2f_dims (host code, no GPU) gives the oracle's fine dimensions and rejects bad grids."""
    import ctypes as C
    lib = gpu_lib.load()
    for seed in CC.SEEDS:
        p = GOLD[str(seed)]["case"]
        ix = (C.c_int * len(p["igridx"]))(*p["igridx"])
        iy = (C.c_int * len(p["igridy"]))(*p["igridy"])
        iz = (C.c_int * len(p["igridz"]))(*p["igridz"])
        g = gpu_lib.C2fGrid(p["nxc"], p["nyc"], p["nzc"], ix, iy, iz, p["x0"], p["y0"], p["z0"], p["h"])
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        assert lib.fdgpu_c2f_dims(C.byref(g), C.byref(nx), C.byref(ny), C.byref(nz)) == 0
        assert [nx.value, ny.value, nz.value] == GOLD[str(seed)]["dims"]
    bad = (C.c_int * 2)(3, 0)            # a zero step
    g = gpu_lib.C2fGrid(3, 3, 3, bad, bad, bad, 0.0, 0.0, 0.0, 1.0)
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    assert lib.fdgpu_c2f_dims(C.byref(g), C.byref(nx), C.byref(ny), C.byref(nz)) == -1
    g = gpu_lib.C2fGrid(1, 3, 3, bad, bad, bad, 0.0, 0.0, 0.0, 1.0)   # one node on an axis
    assert lib.fdgpu_c2f_dims(C.byref(g), C.byref(nx), C.byref(ny), C.byref(nz)) == -1
