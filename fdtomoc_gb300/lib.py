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
FDGPU_ETOOBIG = -9
ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "EIO", -5: "EPAR", -6: "ESOURCE", -7: "ESCHED", -8: "ENODEV",
          -9: "ETOOBIG", -10: "ETIMEDOUT"}


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
                ("t_end_ns", C.c_int64), ("pipelined_sweeps", C.c_int32), ("detail", C.c_int32),
                ("sm", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self):
        return dict(status=self.status, sweeps=self.sweeps, node_updates=self.node_updates, faces=self.faces,
                    rounds=self.rounds, deferred=self.deferred, stencils=list(self.stencils),
                    restart_wall=list(self.restart_wall), phase_cycles=list(self.phase_cycles),
                    t_start_ns=self.t_start_ns, t_end_ns=self.t_end_ns, pipelined_sweeps=self.pipelined_sweeps, sm=self.sm,
                    detail=self.detail)


class ServeOpts(C.Structure):
    """fdgpu_serve_opts."""

    _fields_ = [("hbm_bytes", C.c_longlong), ("max_inflight", C.c_int), ("reserve_sms", C.c_int),
                ("max_models", C.c_int), ("idle_stop_us", C.c_int)]


class ServeResult(C.Structure):
    """fdgpu_serve_result."""

    _fields_ = [("id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("model_version", C.c_int32),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double), ("solve_ms", C.c_double), ("stats", Stats)]

    def as_dict(self):
        return dict(id=self.id, tag=self.tag, status=self.status, model_version=self.model_version,
                    queue_ms=self.queue_ms, latency_ms=self.latency_ms, solve_ms=self.solve_ms,
                    stats=self.stats.as_dict())


class ServeMetrics(C.Structure):
    """fdgpu_serve_metrics."""

    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("inflight", C.c_int64), ("p50_ms", C.c_double), ("p90_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("mean_ms", C.c_double), ("solve_p50_ms", C.c_double),
                ("solve_p99_ms", C.c_double), ("fields_per_s", C.c_double), ("node_updates_per_s", C.c_double),
                ("node_updates", C.c_int64), ("hbm_bytes", C.c_int64), ("hbm_used", C.c_int64),
                ("hbm_peak", C.c_int64), ("solver_ctas", C.c_int32), ("grid_launches", C.c_int32),
                ("hist", C.c_int64 * 40)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "hist"}
        d["hist"] = list(self.hist)
        return d


class LocGrid(C.Structure):
    """fdgpu_loc_grid: the grid and search parameters of sphfdloc's event location."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x0", C.c_double), ("y0", C.c_double),
                ("z0", C.c_double), ("h", C.c_double), ("dq", C.c_double), ("df", C.c_double),
                ("xmax", C.c_float), ("ymax", C.c_float), ("zmax", C.c_float), ("z0r", C.c_double),
                ("kmin", C.c_int), ("ndiv", C.c_int), ("ndiv2", C.c_int), ("ivs", C.c_int), ("vpvs", C.c_float),
                ("nthres", C.c_int), ("resthres", C.c_float), ("resthrep", C.c_float), ("stdmax", C.c_float)]


class LocObs(C.Structure):
    """fdgpu_loc_obs: one phase of an event."""

    _fields_ = [("field", C.c_int32), ("obstime", C.c_float), ("pwt", C.c_float), ("phase", C.c_char),
                ("good", C.c_char), ("pad", C.c_char * 2)]


class LocResult(C.Structure):
    """fdgpu_loc_result."""

    _fields_ = [("status", C.c_int32), ("ngood", C.c_int32), ("nxx", C.c_int32), ("nyy", C.c_int32),
                ("nzz", C.c_int32), ("passes", C.c_int32), ("exm", C.c_double), ("eym", C.c_double),
                ("ezm", C.c_double), ("stdmin", C.c_float), ("avrmin", C.c_float)]


class C2fGrid(C.Structure):
    """fdgpu_c2f_grid."""

    _fields_ = [("nxc", C.c_int), ("nyc", C.c_int), ("nzc", C.c_int), ("igridx", C.POINTER(C.c_int)),
                ("igridy", C.POINTER(C.c_int)), ("igridz", C.POINTER(C.c_int)), ("x0", C.c_double),
                ("y0", C.c_double), ("z0", C.c_double), ("h", C.c_double)]


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
        lib.fdgpu_set_wait_limits.argtypes = [P, C.c_longlong, C.c_longlong]
        lib.fdgpu_station_from_par.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(Station), C.c_char_p,
                                               C.c_size_t, C.c_char_p, C.c_size_t]
        lib.fdgpu_solve_host.argtypes = [P, C.c_int, C.POINTER(Station), C.POINTER(C.c_float), C.c_int, C.c_int,
                                         C.c_int, C.POINTER(C.POINTER(C.c_float)),
                                         C.POINTER(C.POINTER(C.c_float)), C.POINTER(Stats)]
        lib.fdgpu_solve_device.argtypes = [P, C.c_int, C.POINTER(Station), C.c_void_p, C.c_longlong, C.c_longlong,
                                           C.POINTER(C.c_void_p), C.c_int, C.POINTER(Stats), C.c_void_p]
        lib.fdgpu_probe_fp64.argtypes = [P, C.POINTER(C.c_double)]
        from . import rayderv as _R
        lib.fdgpu_ray_default_limits.argtypes = [C.POINTER(_R.RayGrid), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.fdgpu_raytrace.argtypes = [P, C.POINTER(_R.RayGrid), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                       C.POINTER(_R.RayObs), C.c_int, C.c_int, C.POINTER(_R.RayResult),
                                       C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_float),
                                       C.c_longlong, C.c_void_p]
        lib.fdgpu_batch_create.argtypes = [P, C.c_int, C.POINTER(Station), C.c_void_p, C.c_longlong, C.c_longlong,
                                           C.POINTER(C.c_void_p), C.c_int, C.POINTER(P)]
        lib.fdgpu_batch_run.argtypes = [P, C.c_void_p]
        lib.fdgpu_batch_stats.argtypes = [P, C.POINTER(Stats), C.c_void_p]
        lib.fdgpu_batch_order.argtypes = [P, C.POINTER(C.c_int), C.c_void_p]
        lib.fdgpu_order_save.argtypes = [P, C.c_char_p]
        lib.fdgpu_order_load.argtypes = [P, C.c_char_p]
        lib.fdgpu_batch_set_order.argtypes = [P, C.POINTER(C.c_int), C.c_void_p]
        lib.fdgpu_batch_tune_order.argtypes = [P, C.c_void_p]
        lib.fdgpu_batch_destroy.argtypes = [P]
        lib.fdgpu_batch_destroy.restype = None
        lib.fdgpu_velocity_to_slowness.argtypes = [P, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]
        lib.fdgpu_sphfd.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p]
        lib.fdgpu_sphfd_parlist.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p, C.POINTER(C.c_int)]
        lib.fdgpu_loc_grid_from_spec.argtypes = [C.POINTER(LocGrid), C.c_int, C.c_int, C.c_int, C.c_double,
                                                 C.c_double, C.c_double, C.c_double]
        lib.fdgpu_loc_grid_from_spec.restype = None
        lib.fdgpu_locate.argtypes = [P, C.POINTER(LocGrid), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(LocObs), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float), C.POINTER(LocResult), C.c_void_p]
        lib.fdgpu_c2f_dims.argtypes = [C.POINTER(C2fGrid), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]
        lib.fdgpu_c2f.argtypes = [P, C.POINTER(C2fGrid), C.c_void_p, C.c_void_p, C.c_void_p]
        lib.fdgpu_c2f_plan_create.argtypes = [P, C.POINTER(C2fGrid), C.POINTER(P)]
        lib.fdgpu_c2f_run.argtypes = [P, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.fdgpu_c2f_plan_destroy.argtypes = [P]
        lib.fdgpu_c2f_plan_destroy.restype = None
        lib.fdgpu_serve_open.argtypes = [C.c_int, C.POINTER(ServeOpts), C.POINTER(P)]
        lib.fdgpu_serve_set_model.argtypes = [P, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                              C.POINTER(C.c_int)]
        lib.fdgpu_serve_submit.argtypes = [P, C.POINTER(Station), C.c_int, C.c_void_p, C.c_void_p, C.c_uint64,
                                           C.POINTER(C.c_uint64)]
        lib.fdgpu_serve_poll.argtypes = [P, C.POINTER(ServeResult), C.c_int, C.c_int, C.POINTER(C.c_int)]
        lib.fdgpu_serve_drain.argtypes = [P, C.c_int]
        lib.fdgpu_serve_metrics_get.argtypes = [P, C.POINTER(ServeMetrics)]
        lib.fdgpu_serve_last_error.argtypes = [P]
        lib.fdgpu_serve_last_error.restype = C.c_char_p
        lib.fdgpu_serve_close.argtypes = [P]
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
        import weakref
        self.lib = load()
        self.ptr = C.c_void_p()
        self._batches = weakref.WeakSet()
        self.device = device
        _check(self.lib.fdgpu_create(device, C.byref(self.ptr)))

    def set_cluster(self, ctas_per_station: int):
        """CTAs per station in later solves (0: automatic)."""
        _check(self.lib.fdgpu_set_cluster(self.ptr, ctas_per_station))

    def save_order(self, path: str):
        """Write the context's measured solve times (the launch-order table) to a file."""
        _check(self.lib.fdgpu_order_save(self.ptr, path.encode()), self.ptr)

    def load_order(self, path: str):
        """Merge a saved launch-order table into the context."""
        _check(self.lib.fdgpu_order_load(self.ptr, path.encode()), self.ptr)

    def set_wait_limits(self, wait_cycles: int = 0, walk_cycles: int = 0):
        """Bounds of the solver's waits in SM cycles (0: built-in); see fdgpu_set_wait_limits."""
        _check(self.lib.fdgpu_set_wait_limits(self.ptr, C.c_longlong(wait_cycles), C.c_longlong(walk_cycles)))

    def close(self):
        if self.ptr:
            for b in list(getattr(self, "_batches", ())):
                b.close()
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


def raytrace(ctx: "Context", grid, d_fields, obs, nobs: int, cap: int = 0, max_seg: int = 0, stream_ptr: int = 0,
             total_cap: int | None = None):
    """fdgpu_raytrace: returns (results, off, idx, du), observation o's derivatives at
    idx/du[off[o] .. off[o+1])."""
    from . import rayderv as R
    lib = load()
    n = max(1, nobs)
    res = (R.RayResult * n)()
    off = np.zeros(n + 1, dtype=np.int64)
    fp = (C.c_void_p * max(1, len(d_fields)))(*d_fields)
    if total_cap is None:
        total_cap = 192 * max(1, nobs)   # a long ray has a few hundred; a second run only beyond that
    while True:
        idx = np.zeros(max(1, total_cap), dtype=np.int32)
        du = np.zeros(max(1, total_cap), dtype=np.float32)
        rc = lib.fdgpu_raytrace(ctx.ptr, C.byref(grid), fp, len(d_fields), nobs, obs, max_seg, cap, res,
                                off.ctypes.data_as(C.POINTER(C.c_longlong)), idx.ctypes.data_as(C.POINTER(C.c_int)),
                                du.ctypes.data_as(C.POINTER(C.c_float)), total_cap, C.c_void_p(stream_ptr))
        if rc == FDGPU_ETOOBIG and off[nobs] > total_cap:
            total_cap = int(off[nobs])
            continue
        _check(rc, ctx.ptr)
        return res, off[: nobs + 1], idx[: off[nobs]], du[: off[nobs]]


class Batch:
    """fdgpu_batch: stations prepared once, launched many times (capturable in a CUDA graph)."""

    def __init__(self, ctx: "Context", stations, slowness_ptr: int, s_sy: int, s_sz: int, time_ptrs,
                 initialised=False):
        self.lib = load()
        self.ctx = ctx
        self.n = len(stations)
        arr = (Station * self.n)(*stations)
        tp = (C.c_void_p * self.n)(*time_ptrs)
        self.ptr = C.c_void_p()
        _check(self.lib.fdgpu_batch_create(ctx.ptr, self.n, arr, C.c_void_p(slowness_ptr), s_sy, s_sz, tp,
                                           1 if initialised else 0, C.byref(self.ptr)), ctx.ptr)
        ctx._batches.add(self)   # a batch is destroyed before its context

    def run(self, stream_ptr: int = 0):
        _check(self.lib.fdgpu_batch_run(self.ptr, C.c_void_p(stream_ptr)), self.ctx.ptr)

    def stats(self, stream_ptr: int = 0):
        st = (Stats * self.n)()
        _check(self.lib.fdgpu_batch_stats(self.ptr, st, C.c_void_p(stream_ptr)), self.ctx.ptr)
        return [s.as_dict() for s in st]

    def order(self, stream_ptr: int = 0):
        """Launch order: the stations' indices, first launched first."""
        o = (C.c_int * self.n)()
        _check(self.lib.fdgpu_batch_order(self.ptr, o, C.c_void_p(stream_ptr)), self.ctx.ptr)
        return list(o)

    def set_order(self, order, stream_ptr: int = 0):
        o = (C.c_int * self.n)(*order)
        _check(self.lib.fdgpu_batch_set_order(self.ptr, o, C.c_void_p(stream_ptr)), self.ctx.ptr)

    def tune_order(self, stream_ptr: int = 0):
        """Longest measured solve of the last run first."""
        _check(self.lib.fdgpu_batch_tune_order(self.ptr, C.c_void_p(stream_ptr)), self.ctx.ptr)

    def close(self):
        if self.ptr:
            self.lib.fdgpu_batch_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def loc_grid_from_spec(nx, ny, nz, x0_deg, y0_deg, z0_km, h_km) -> LocGrid:
    """sphfdloc's grid from its spec values, with the reference's default search parameters."""
    g = LocGrid()
    load().fdgpu_loc_grid_from_spec(C.byref(g), nx, ny, nz, x0_deg, y0_deg, z0_km, h_km)
    return g


def locate(ctx: "Context", grid: LocGrid, field_ptrs, events, stream_ptr: int = 0):
    """Locate events against device fields.  events: a list of phase lists, each phase
    (field index, obstime, pwt, phase 'P'/'S', good).  Returns one dict per event with the result,
    the final good flags, resmin and tps."""
    lib = load()
    offs = [0]
    flat = []
    for ev in events:
        flat.extend(ev)
        offs.append(len(flat))
    n = len(flat)
    obs = (LocObs * max(n, 1))(*[LocObs(f, t, w, ph.encode(), bytes([1 if g else 0])) for f, t, w, ph, g in flat])
    off = (C.c_int * len(offs))(*offs)
    fp = (C.c_void_p * max(len(field_ptrs), 1))(*field_ptrs)
    resmin = (C.c_float * max(n, 1))()
    tps = (C.c_float * max(n, 1))()
    res = (LocResult * max(len(events), 1))()
    _check(lib.fdgpu_locate(ctx.ptr, C.byref(grid), fp, len(field_ptrs), len(events), off, obs, resmin, tps, res,
                            C.c_void_p(stream_ptr)), ctx.ptr)
    out = []
    for e in range(len(events)):
        r = res[e]
        a, b = offs[e], offs[e + 1]
        out.append(dict(status=r.status, ngood=r.ngood, nxx=r.nxx, nyy=r.nyy, nzz=r.nzz, passes=r.passes,
                        exm=r.exm, eym=r.eym, ezm=r.ezm, stdmin=r.stdmin, avrmin=r.avrmin,
                        good=[obs[k].good[0] for k in range(a, b)], resmin=list(resmin[a:b]), tps=list(tps[a:b])))
    return out


def c2f(ctx: "Context", nxc, nyc, nzc, igridx, igridy, igridz, x0, y0, z0, h, coarse, fine=None,
        stream_ptr: int = 0):
    """Coarse P/S velocities -> fine P/S velocities (c2f).  coarse: (2, nzc, nyc, nxc) float32 numpy
    array or device tensor; fine: a (2, nz, ny, nx) buffer (numpy array or device tensor) or None for
    a new numpy array.  Returns fine."""
    import numpy as np
    lib = load()
    ix = (C.c_int * max(1, len(igridx)))(*igridx)
    iy = (C.c_int * max(1, len(igridy)))(*igridy)
    iz = (C.c_int * max(1, len(igridz)))(*igridz)
    g = C2fGrid(nxc, nyc, nzc, ix, iy, iz, x0, y0, z0, h)
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    _check(lib.fdgpu_c2f_dims(C.byref(g), C.byref(nx), C.byref(ny), C.byref(nz)))
    if fine is None:
        fine = np.empty((2, nz.value, ny.value, nx.value), np.float32)
    cp = coarse.ctypes.data if isinstance(coarse, np.ndarray) else coarse.data_ptr()
    fp = fine.ctypes.data if isinstance(fine, np.ndarray) else fine.data_ptr()
    _check(lib.fdgpu_c2f(ctx.ptr, C.byref(g), C.c_void_p(cp), C.c_void_p(fp), C.c_void_p(stream_ptr)), ctx.ptr)
    return fine


class C2fPlan:
    """fdgpu_c2f_plan: c2f onto one grid, repeatedly, with device buffers."""

    def __init__(self, ctx: "Context", nxc, nyc, nzc, igridx, igridy, igridz, x0, y0, z0, h):
        self.lib = load()
        self.ctx = ctx
        self._ig = [(C.c_int * max(1, len(a)))(*a) for a in (igridx, igridy, igridz)]
        g = C2fGrid(nxc, nyc, nzc, *self._ig, x0, y0, z0, h)
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.fdgpu_c2f_dims(C.byref(g), C.byref(nx), C.byref(ny), C.byref(nz)))
        self.shape = (2, nz.value, ny.value, nx.value)
        self.ptr = C.c_void_p()
        _check(self.lib.fdgpu_c2f_plan_create(ctx.ptr, C.byref(g), C.byref(self.ptr)), ctx.ptr)

    def run(self, coarse_ptr: int, fine_ptr: int, stream_ptr: int = 0):
        _check(self.lib.fdgpu_c2f_run(self.ptr, C.c_void_p(coarse_ptr), C.c_void_p(fine_ptr),
                                      C.c_void_p(stream_ptr)), self.ctx.ptr)

    def close(self):
        if self.ptr:
            self.lib.fdgpu_c2f_plan_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sphfd_parlist(entries, timedir: str, devices=None):
    """Drop-in for the reference's main loop: entries like "par=/path/sta.par"; returns statuses.
    devices: a list of GPUs to deal the stations over (default: the current device)."""
    lib = load()
    n = len(entries)
    argv = (C.c_char_p * n)(*[e.encode() for e in entries])
    status = (C.c_int * n)()
    if devices:
        dv = (C.c_int * len(devices))(*devices)
        rc = lib.fdgpu_sphfd_parlist_devices(n, argv, timedir.encode(), status, len(devices), dv)
        if rc == -8:
            raise FdgpuError("fdgpu error -8 (ENODEV): a listed device does not exist")
    else:
        lib.fdgpu_sphfd_parlist(n, argv, timedir.encode(), status)
    return list(status)


def _addr(buf) -> int:
    """Address of a numpy array or of a tensor-like object with data_ptr()."""
    if isinstance(buf, np.ndarray):
        if not buf.flags.c_contiguous or buf.dtype != np.float32:
            raise FdgpuError("buffers must be C-contiguous float32")
        return buf.ctypes.data
    return int(buf.data_ptr())


class Server:
    """A serving session (fdgpu_serve_*): device-resident models, requests solved as they arrive by
    a long-running grid of solver CTAs.  Buffers passed to submit() are kept referenced until their
    result has been polled."""

    def __init__(self, device: int = 0, hbm_bytes: int = 0, max_inflight: int = 0, reserve_sms: int = -1,
                 max_models: int = 2, idle_stop_us: int = 0):
        self.lib = load()
        self.ptr = C.c_void_p()
        opts = ServeOpts(hbm_bytes, max_inflight, reserve_sms, max_models, idle_stop_us)
        _check(self.lib.fdgpu_serve_open(device, C.byref(opts), C.byref(self.ptr)))
        self._keep = {}

    def _check(self, rc):
        if rc != FDGPU_OK:
            extra = self.lib.fdgpu_serve_last_error(self.ptr).decode() if self.ptr else ""
            msg = self.lib.fdgpu_strerror(rc).decode() + (": " + extra if extra else "")
            raise FdgpuError(f"fdgpu error {rc} ({ERRORS.get(rc, '?')}): {msg}")

    def set_model(self, model: int, velocity) -> int:
        """velocity: (nz, ny, nx) float32, a numpy array or a device tensor.  Returns the version."""
        mnz, mny, mnx = velocity.shape
        ver = C.c_int()
        self._check(self.lib.fdgpu_serve_set_model(self.ptr, model, C.c_void_p(_addr(velocity)), mnx, mny, mnz,
                                                   C.byref(ver)))
        return ver.value

    def submit(self, station: Station, model: int, out, init=None, tag: int = 0) -> int:
        """Queue a solve; out (nz, ny, nx) float32 receives the field (host array or device tensor)."""
        rid = C.c_uint64()
        ip = C.c_void_p(_addr(init)) if init is not None else None
        self._check(self.lib.fdgpu_serve_submit(self.ptr, C.byref(station), model, C.c_void_p(_addr(out)), ip, tag,
                                                C.byref(rid)))
        self._keep[rid.value] = (out, init)
        return rid.value

    def poll(self, max_results: int = 256, timeout_ms: int = 0):
        buf = (ServeResult * max_results)()
        n = C.c_int()
        self._check(self.lib.fdgpu_serve_poll(self.ptr, buf, max_results, timeout_ms, C.byref(n)))
        out = [buf[k].as_dict() for k in range(n.value)]
        for r in out:
            self._keep.pop(r["id"], None)
        return out

    def drain(self, timeout_ms: int = -1):
        self._check(self.lib.fdgpu_serve_drain(self.ptr, timeout_ms))

    def metrics(self) -> dict:
        m = ServeMetrics()
        self._check(self.lib.fdgpu_serve_metrics_get(self.ptr, C.byref(m)))
        return m.as_dict()

    def close(self):
        if self.ptr:
            rc = self.lib.fdgpu_serve_close(self.ptr)
            self.ptr = C.c_void_p()
            self._keep.clear()
            _check(rc)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
