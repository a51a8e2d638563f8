"""ctypes binding of libfdgpu.so (include/fdgpu.h).

This is the Python face of the drop-in boundary: the same C ABI a C caller (the sphfd driver, a
batch or serving loop) links against.  There is no CPU fallback — if the library or a GPU is
missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("FDGPU_LIB") or os.path.join(HERE, "libfdgpu.so")

FDGPU_OK = 0
ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "EIO", -5: "EPAR", -6: "ESOURCE", -7: "ESCHED", -8: "ENODEV",
          -9: "ETOOBIG"}


class Station(C.Structure):
    """fdgpu_station: one sphfd() solve after its par-file set-up."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double), ("dq", C.c_double),
                ("df", C.c_double), ("x0", C.c_double), ("y0", C.c_double), ("z0r", C.c_double),
                ("srctype", C.c_int), ("xs", C.c_int), ("ys", C.c_int), ("zs", C.c_int),
                ("src_geo", C.c_double * 3), ("ncube", C.c_int), ("reverse", C.c_int), ("headpref", C.c_int),
                ("maxrad", C.c_int), ("kminus", C.c_int), ("kplus", C.c_int), ("iplus", C.c_int),
                ("iminus", C.c_int), ("jminus", C.c_int), ("jplus", C.c_int), ("srcwall", C.c_int),
                ("ox", C.c_int), ("oy", C.c_int), ("oz", C.c_int)]

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)


class Stats(C.Structure):
    _fields_ = [("status", C.c_int32), ("sweeps", C.c_int32), ("node_updates", C.c_int64), ("faces", C.c_int64),
                ("rounds", C.c_int64), ("deferred", C.c_int64), ("stencils", C.c_int64 * 5),
                ("restart_wall", C.c_int32 * 8), ("phase_cycles", C.c_int64 * 6), ("t_start_ns", C.c_int64),
                ("t_end_ns", C.c_int64), ("pipelined_sweeps", C.c_int32), ("detail", C.c_int32)]

    def as_dict(self):
        return dict(status=self.status, sweeps=self.sweeps, node_updates=self.node_updates, faces=self.faces,
                    rounds=self.rounds, deferred=self.deferred, stencils=list(self.stencils),
                    restart_wall=list(self.restart_wall), phase_cycles=list(self.phase_cycles),
                    t_start_ns=self.t_start_ns, t_end_ns=self.t_end_ns, pipelined_sweeps=self.pipelined_sweeps,
                    detail=self.detail)


class FdgpuError(RuntimeError):
    pass


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FdgpuError(f"{LIB_PATH} is missing: run fdtomoc_gb300.build.build() (the GPU path has no fallback)")
        lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        lib.fdgpu_create.argtypes = [C.c_int, C.POINTER(P)]
        lib.fdgpu_destroy.argtypes = [P]
        lib.fdgpu_destroy.restype = None
        lib.fdgpu_strerror.argtypes = [C.c_int]
        lib.fdgpu_strerror.restype = C.c_char_p
        lib.fdgpu_last_error.argtypes = [P]
        lib.fdgpu_last_error.restype = C.c_char_p
        lib.fdgpu_set_cluster.argtypes = [P, C.c_int]
        lib.fdgpu_station_from_par.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(Station), C.c_char_p,
                                               C.c_size_t, C.c_char_p, C.c_size_t]
        lib.fdgpu_solve_host.argtypes = [P, C.c_int, C.POINTER(Station), C.POINTER(C.c_float), C.c_int, C.c_int,
                                         C.c_int, C.POINTER(C.POINTER(C.c_float)),
                                         C.POINTER(C.POINTER(C.c_float)), C.POINTER(Stats)]
        lib.fdgpu_solve_device.argtypes = [P, C.c_int, C.POINTER(Station), C.c_void_p, C.c_longlong, C.c_longlong,
                                           C.POINTER(C.c_void_p), C.c_int, C.POINTER(Stats), C.c_void_p]
        lib.fdgpu_probe_fp64.argtypes = [P, C.POINTER(C.c_double)]
        lib.fdgpu_velocity_to_slowness.argtypes = [P, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]
        lib.fdgpu_sphfd.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p]
        lib.fdgpu_sphfd_parlist.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p, C.POINTER(C.c_int)]
        _lib = lib
    return _lib


def _check(rc, ctx=None):
    if rc != FDGPU_OK:
        lib = load()
        msg = lib.fdgpu_strerror(rc).decode()
        if ctx is not None:
            extra = lib.fdgpu_last_error(ctx).decode()
            if extra:
                msg += ": " + extra
        raise FdgpuError(f"fdgpu error {rc} ({ERRORS.get(rc, '?')}): {msg}")


def station_from_par(*args: str):
    """Par-file set-up as sphfd() does it; args like ("par=/path/sta.par",).  Returns
    (Station, velfile, timefile)."""
    lib = load()
    argv = (C.c_char_p * (len(args) + 1))(b"sphfd", *[a.encode() for a in args])
    st = Station()
    vf = C.create_string_buffer(1024)
    tf = C.create_string_buffer(1024)
    _check(lib.fdgpu_station_from_par(len(args) + 1, argv, C.byref(st), vf, 1024, tf, 1024))
    return st, vf.value.decode(), tf.value.decode()


class Context:
    """An fdgpu_ctx on one device: owns geometry tables, scratch and a stream."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.ptr = C.c_void_p()
        _check(self.lib.fdgpu_create(device, C.byref(self.ptr)))

    def set_cluster(self, ctas_per_station: int):
        """CTAs per station in later solves (0: automatic)."""
        _check(self.lib.fdgpu_set_cluster(self.ptr, ctas_per_station))

    def close(self):
        if self.ptr:
            self.lib.fdgpu_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_host(self, stations, velocity: np.ndarray, init_times=None):
        """Solve stations against a host velocity model (nz, ny, nx) float32; returns (times, stats)."""
        vel = np.ascontiguousarray(velocity, dtype=np.float32)
        mnz, mny, mnx = vel.shape
        n = len(stations)
        arr = (Station * n)(*stations)
        outs = [np.empty(s.shape, dtype=np.float32) for s in stations]
        outp = (C.POINTER(C.c_float) * n)(*[o.ctypes.data_as(C.POINTER(C.c_float)) for o in outs])
        initp = None
        if init_times is not None:
            inits = [np.ascontiguousarray(t, dtype=np.float32) for t in init_times]
            initp = (C.POINTER(C.c_float) * n)(*[t.ctypes.data_as(C.POINTER(C.c_float)) for t in inits])
        stats = (Stats * n)()
        rc = self.lib.fdgpu_solve_host(self.ptr, n, arr, vel.ctypes.data_as(C.POINTER(C.c_float)), mnx, mny, mnz,
                                       outp, initp, stats)
        _check(rc, self.ptr)
        return outs, [s.as_dict() for s in stats]

    def solve_device(self, stations, slowness_ptr: int, s_sy: int, s_sz: int, time_ptrs, initialised=False,
                     stream_ptr: int = 0):
        """Solve with device buffers (raw pointers, e.g. torch tensor data_ptr())."""
        n = len(stations)
        arr = (Station * n)(*stations)
        tp = (C.c_void_p * n)(*time_ptrs)
        stats = (Stats * n)()
        rc = self.lib.fdgpu_solve_device(self.ptr, n, arr, C.c_void_p(slowness_ptr), s_sy, s_sz, tp,
                                         1 if initialised else 0, stats, C.c_void_p(stream_ptr))
        _check(rc, self.ptr)
        return [s.as_dict() for s in stats]

    def probe_fp64_gops(self) -> float:
        """Measured FP64 instruction rate (G instructions/s) of this GPU."""
        g = C.c_double()
        _check(self.lib.fdgpu_probe_fp64(self.ptr, C.byref(g)), self.ptr)
        return g.value

    def velocity_to_slowness(self, vel_ptr: int, slow_ptr: int, n: int, stream_ptr: int = 0):
        _check(self.lib.fdgpu_velocity_to_slowness(self.ptr, C.c_void_p(vel_ptr), C.c_void_p(slow_ptr), n,
                                                   C.c_void_p(stream_ptr)), self.ptr)


def sphfd_parlist(entries, timedir: str):
    """Drop-in for the reference's main loop: entries like "par=/path/sta.par"; returns statuses."""
    lib = load()
    n = len(entries)
    argv = (C.c_char_p * n)(*[e.encode() for e in entries])
    status = (C.c_int * n)()
    lib.fdgpu_sphfd_parlist(n, argv, timedir.encode(), status)
    return list(status)
