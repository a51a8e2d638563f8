"""Test-side access to the CPU oracle (oracle/): build it and run it on par files."""
import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_lib = None


class OracleStats(C.Structure):
    _fields_ = [("node_updates", C.c_int64), ("calls", C.c_int64 * 5), ("skipped", C.c_int64 * 5),
                ("inherit_points", C.c_int64), ("faces", C.c_int64), ("sweeps", C.c_int),
                ("restarts", C.c_int * 7), ("changed_per_sweep", C.c_int64 * 64),
                ("depth_per_sweep", C.c_int64 * 64), ("updates_per_sweep", C.c_int64 * 64)]


def load_oracle():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so", "sphfd_oracle"], check=True)
        lib = C.CDLL(os.path.join(ORACLE_DIR, "liboracle.so"))
        lib.fdo_sphfd.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p, C.c_int, C.POINTER(OracleStats)]
        _lib = lib
    return _lib


def run_oracle(parfile: str, timedir: str, fast: bool = False):
    """Run the oracle's whole-station driver; returns its statistics."""
    lib = load_oracle()
    os.makedirs(timedir, exist_ok=True)
    argv = (C.c_char_p * 2)(b"sphfd", ("par=" + parfile).encode())
    st = OracleStats()
    rc = lib.fdo_sphfd(2, argv, timedir.encode(), 1 if fast else 0, C.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle failed on {parfile}: {rc}")
    return st


# ---- location oracle (oracle/fd_locate.c) ----------------------------------------------------

class LocGrid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x0", C.c_double), ("y0", C.c_double),
                ("z0", C.c_double), ("h", C.c_double), ("dq", C.c_double), ("df", C.c_double),
                ("xmax", C.c_float), ("ymax", C.c_float), ("zmax", C.c_float), ("z0r", C.c_double),
                ("kmin", C.c_int), ("ndiv", C.c_int), ("ndiv2", C.c_int), ("ivs", C.c_int), ("vpvs", C.c_float),
                ("nthres", C.c_int), ("resthres", C.c_float), ("resthrep", C.c_float), ("stdmax", C.c_float)]


class LocObs(C.Structure):
    _fields_ = [("field", C.c_int), ("obstime", C.c_float), ("pwt", C.c_float), ("phase", C.c_char),
                ("good", C.c_int)]


class LocResult(C.Structure):
    _fields_ = [("status", C.c_int), ("ngood", C.c_int), ("nxx", C.c_int), ("nyy", C.c_int), ("nzz", C.c_int),
                ("passes", C.c_int), ("exm", C.c_double), ("eym", C.c_double), ("ezm", C.c_double),
                ("stdmin", C.c_float), ("avrmin", C.c_float)]


def loc_lib():
    lib = load_oracle()
    if not getattr(lib, "_loc_bound", False):
        lib.fdo_loc_grid_from_spec.argtypes = [C.POINTER(LocGrid), C.c_int, C.c_int, C.c_int, C.c_double,
                                               C.c_double, C.c_double, C.c_double]
        lib.fdo_locate.argtypes = [C.POINTER(LocGrid), C.POINTER(C.POINTER(C.c_float)), C.c_int,
                                   C.POINTER(LocObs), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(LocResult)]
        lib.fdo_htoe.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
        lib.fdo_htoe.restype = C.c_double
        lib.fdo_etoh.argtypes = [C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int), C.POINTER(C.c_double)]
        lib.fdo_glathinv.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double)]
        lib.fdo_glathinv.restype = C.c_double
        lib.fdo_loc_hpi.restype = C.c_double
        lib.fdo_loc_degrad.restype = C.c_double
        lib._loc_bound = True
    return lib


def loc_helpers(grid):
    """htoe / etoh / glathinv of the oracle, and the grid's constants, for loc_cases.format_outputs"""
    lib = loc_lib()

    def etoh(e):
        y, d, h, m, s = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_double()
        lib.fdo_etoh(e, C.byref(y), C.byref(d), C.byref(h), C.byref(m), C.byref(s))
        return y.value, d.value, h.value, m.value, s.value

    def glathinv(x, r):
        hh = C.c_double()
        lat = lib.fdo_glathinv(x, r, C.byref(hh))
        return lat, hh.value

    return dict(htoe=lib.fdo_htoe, etoh=etoh, glathinv=glathinv, hpi=lib.fdo_loc_hpi(),
                degrad=lib.fdo_loc_degrad(), z0r=grid.z0r)


def loc_grid(p):
    lib = loc_lib()
    g = LocGrid()
    lib.fdo_loc_grid_from_spec(C.byref(g), p["nx"], p["ny"], p["nz"], p["x0"], p["y0"], p["z0"], p["h"])
    g.kmin, g.ndiv, g.ndiv2 = p["kmin"], p["ndiv"], p["ndiv2"]
    g.nthres, g.resthres, g.resthrep, g.stdmax = p["nthres"], p["resthres"], p["resthrep"], p["stdmax"]
    if "ivs" in p:
        g.ivs, g.vpvs = p["ivs"], p["vpvs"]
    return g


def oracle_locate(grid, field_list, obs):
    """obs: list of (field index, obstime, pwt, phase, good); returns a result dict as
    loc_cases.format_outputs reads it."""
    lib = loc_lib()
    n = len(obs)
    arr = (LocObs * n)(*[LocObs(f, t, w, ph.encode(), g) for f, t, w, ph, g in obs])
    fp = (C.POINTER(C.c_float) * len(field_list))(*[f.ctypes.data_as(C.POINTER(C.c_float)) for f in field_list])
    resmin = (C.c_float * n)()
    tps = (C.c_float * n)()
    r = LocResult()
    rc = lib.fdo_locate(C.byref(grid), fp, n, arr, resmin, tps, C.byref(r))
    assert rc == 0
    return dict(status=r.status, ngood=r.ngood, nxx=r.nxx, nyy=r.nyy, nzz=r.nzz, passes=r.passes, exm=r.exm,
                eym=r.eym, ezm=r.ezm, stdmin=r.stdmin, avrmin=r.avrmin, good=[a.good for a in arr],
                resmin=list(resmin), tps=list(tps))


# ---- c2f oracle (oracle/fd_c2f.c) ------------------------------------------------------------

class C2fGrid(C.Structure):
    _fields_ = [("nxc", C.c_int), ("nyc", C.c_int), ("nzc", C.c_int), ("igridx", C.POINTER(C.c_int)),
                ("igridy", C.POINTER(C.c_int)), ("igridz", C.POINTER(C.c_int)), ("x0", C.c_double),
                ("y0", C.c_double), ("z0", C.c_double), ("h", C.c_double)]


def oracle_c2f(p, coarse):
    """coarse (2, nzc, nyc, nxc) float32 -> fine (2, nz, ny, nx) float32 by the oracle"""
    import numpy as np
    lib = load_oracle()
    lib.fdo_c2f.argtypes = [C.POINTER(C2fGrid), C.POINTER(C.c_float), C.POINTER(C.c_float)]
    ix = (C.c_int * len(p["igridx"]))(*p["igridx"])
    iy = (C.c_int * len(p["igridy"]))(*p["igridy"])
    iz = (C.c_int * len(p["igridz"]))(*p["igridz"])
    g = C2fGrid(p["nxc"], p["nyc"], p["nzc"], ix, iy, iz, p["x0"], p["y0"], p["z0"], p["h"])
    nx, ny, nz = 1 + sum(p["igridx"]), 1 + sum(p["igridy"]), 1 + sum(p["igridz"])
    fine = np.empty((2, nz, ny, nx), np.float32)
    src = np.ascontiguousarray(coarse, np.float32)
    rc = lib.fdo_c2f(C.byref(g), src.ctypes.data_as(C.POINTER(C.c_float)), fine.ctypes.data_as(C.POINTER(C.c_float)))
    assert rc == 0
    return fine


def ray_lib():
    """liboracle's ray tracer (oracle/fd_ray.c)."""
    lib = load_oracle()
    if not getattr(lib, "_ray_bound", False):
        from fdtomoc_gb300 import rayderv as R
        lib.fdr_trace.argtypes = [C.POINTER(R.RayGrid), C.POINTER(C.POINTER(C.c_float)), C.c_int,
                                  C.POINTER(R.RayObs), C.c_int, C.c_int, C.c_int, C.POINTER(R.RayResult),
                                  C.POINTER(C.c_int), C.POINTER(C.c_float)]
        lib.fdr_trace.restype = C.c_int
        lib.fdr_trig.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        lib.fdr_trig.restype = C.c_double
        lib._ray_bound = True
    return lib


def oracle_trace(trig_mode: int):
    """A tracer for fdtomoc_gb300.rayderv.run: the oracle with the C library's trig functions
    (trig_mode 0, as the reference) or the double-double ones the device uses (1)."""
    import numpy as np
    from fdtomoc_gb300 import rayderv as R

    def trace(grid, fields, obs, nobs, cap):
        lib = ray_lib()
        n = max(1, nobs)
        res = (R.RayResult * n)()
        idx = np.zeros(n * cap, dtype=np.int32)
        du = np.zeros(n * cap, dtype=np.float32)
        fl = [np.ascontiguousarray(f, dtype=np.float32) for f in fields]
        fp = (C.POINTER(C.c_float) * max(1, len(fl)))(*[f.ctypes.data_as(C.POINTER(C.c_float)) for f in fl])
        rc = lib.fdr_trace(C.byref(grid), fp, nobs, obs, trig_mode, R.default_max_seg(grid), cap, res,
                           idx.ctypes.data_as(C.POINTER(C.c_int)), du.ctypes.data_as(C.POINTER(C.c_float)))
        assert rc == 0
        nnz = np.array([res[o].nnz for o in range(nobs)], dtype=np.int64)
        off = np.zeros(nobs + 1, dtype=np.int64)
        np.cumsum(nnz, out=off[1:])
        take = np.concatenate([o * cap + np.arange(nnz[o]) for o in range(nobs)]) if nobs else np.zeros(0, int)
        return res, off, idx[take], du[take]

    return trace
