"""sphrayderv's host side: the spec, station and event files read as the reference reads them, the
observations handed to a ray tracer (the GPU's fdgpu_raytrace, or any callable with its contract),
and the inversion files written from its results (reference src/sphrayderv.c).

The tracer does the per-observation work (residual and hypocentre derivatives at the event, the ray
traced back down the travel-time gradient, the ray's slowness derivatives on the coarse metagrid,
src/sphrayderv.c:1054-2232).  What stays here is sequential by nature: the event loop's bookkeeping
of which coarse nodes are unknowns (kbl, mhit, mndex per event; mbl, nhit, indx, jndx over the run,
:1548-1620) and the files built from it (:2262-2470, :2655-2692), reproduced with the reference's own
state, including what carries over from one event to the next when an event's first observation
does not reach its station.

Local earthquakes only: teleseisms and shots (dotel, doshot) are off by default in the reference and
need tables this build does not read; ivpvs (Vp/Vs unknowns) is not supported.  The files written:
dtdsfil, resfile, dtdhfil, bookfil, sclefil, hitfile.  The data-out files (idatout) and the error
summary and log texts are not written.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re
import struct

import numpy as np

DEGRAD = float(np.float32(0.017453292))   # 0.017453292f (:84)
HPI = float(np.float32(1.570796))          # 1.570796f (:83)
REARTH = 6371.0
F32 = np.float32


class RayGrid(C.Structure):
    """fdgpu_ray_grid: fine and coarse grid in radians / km."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nxc", C.c_int), ("nyc", C.c_int),
                ("nzc", C.c_int), ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
                ("h", C.c_double), ("dq", C.c_double), ("df", C.c_double), ("gx", C.POINTER(C.c_float)),
                ("gy", C.POINTER(C.c_float)), ("gz", C.POINTER(C.c_float))]


class RayObs(C.Structure):
    """fdgpu_ray_obs: one observation (event, station-phase)."""

    _fields_ = [("ex", C.c_double), ("ey", C.c_double), ("ez", C.c_double), ("xs", C.c_double),
                ("ys", C.c_double), ("zs", C.c_double), ("field", C.c_int), ("phase", C.c_int),
                ("obstime", C.c_float), ("pwt", C.c_float), ("tc", C.c_float), ("pad", C.c_int)]


class RayResult(C.Structure):
    """fdgpu_ray_result."""

    _fields_ = [("status", C.c_int), ("nseg", C.c_int), ("dt", C.c_double), ("resmin", C.c_float),
                ("wet", C.c_float), ("am", C.c_float * 4), ("nnz", C.c_int), ("pad", C.c_int)]


RAY_OK, RAY_NOTIME, RAY_LEFT, RAY_STEPS, RAY_COARSE, RAY_OUTSIDE = range(6)


def glat(hlat: float) -> float:
    """geographic -> geocentric latitude (lib/common/geographic_method.c:7-16)"""
    halfpi, polfac, elfac = float(F32(1.570796)), float(F32(0.010632)), float(F32(0.993277))
    if halfpi - abs(hlat) >= 0.05:
        return math.atan(elfac * math.sin(hlat) / math.cos(hlat))
    return hlat / elfac - abs(polfac) * (1 if hlat >= 0 else -1)


def _isleap(y: int) -> int:
    return 1 if (y % 4 == 0 and y % 100 != 0) or y % 400 == 0 else 0


def htoe(iyear: int, iday: int, ihour: int, imin: int, sec: float) -> float:
    """epoch seconds (lib/common/time_process.c:85-109)"""
    days = 0
    if iyear > 1970:
        for y in range(1970, iyear):
            days += 365 + _isleap(y)
    elif iyear < 1970:
        for y in range(iyear, 1970):
            days -= 365 + _isleap(y)
    days += iday - 1
    return float(days * 86400) + 3600.0 * ihour + 60.0 * imin + sec


# ------------------------------------------------------------------------------------------------
# spec, stations, events


def read_spec(path: str) -> dict:
    """The variables sphrayderv reads (:195-470): first occurrence of each name."""
    vals: dict[str, str] = {}
    with open(path) as fh:
        for line in fh:
            parts = line.split(None, 1)
            if not parts or parts[0].startswith("#"):
                continue
            vals.setdefault(parts[0], parts[1].strip() if len(parts) > 1 else "")

    def num(name, cast, default=None):
        return cast(vals[name].split()[0]) if name in vals else default

    sp = dict(nxc=num("nxc", int), nyc=num("nyc", int), nzc=num("nzc", int), h=num("h", float),
              x0=num("x0", float, 0.0), y0=num("y0", float, 0.0), z0=num("z0", float, 0.0),
              dq=num("dq", float, 0.0), df=num("df", float, 0.0), ivs=num("ivs", int, 1),
              ivpvs=num("ivpvs", int, 0), dotel=num("dotel", int, 0), doshot=num("doshot", int, 0),
              nomat=num("nomat", int, 0), timedir=vals.get("timedir", "./ttimes").split()[0])
    if sp["ivs"] not in (0, 1):
        sp["ivs"] = 0
    for ax, n in (("igridx", "nxc"), ("igridy", "nyc"), ("igridz", "nzc")):
        sp[ax] = [int(v) for v in vals[ax].split()[: sp[n] - 1]]
    for f in ("stafile", "locdfil", "dtdsfil", "resfile", "hitfile", "dtdhfil", "bookfil", "sclefil"):
        sp[f] = vals[f].split()[0]
    return sp


def grid_from_spec(sp: dict, spacing_rule: bool = True):
    """Fine and coarse grid (:470-525, :779-788).  Returns (RayGrid, arrays to keep alive).

    The reference replaces a spacing below 1e-4 rad (about 0.0057 degrees) by h / rearth (:515-518),
    where sphfd keeps the spacing it is given: for finer grids the two programs' frames then differ
    and rays aim at a station the field does not have.  spacing_rule=False keeps dq and df as given,
    for tracing through fields computed with that spacing."""
    nx = 1 + sum(sp["igridx"])
    ny = 1 + sum(sp["igridy"])
    nz = 1 + sum(sp["igridz"])
    h = sp["h"]
    x0 = sp["x0"] * DEGRAD
    y0 = HPI - glat(sp["y0"] * DEGRAD)
    dq = sp["dq"] * DEGRAD
    df = sp["df"] * DEGRAD
    if abs(dq) < 0.0001 and (spacing_rule or dq == 0):
        dq = h / REARTH
    if abs(df) < 0.0001 and (spacing_rule or df == 0):
        df = abs(h / (REARTH * math.sin(y0)))
    z0 = sp["z0"]

    def axis(start, step, cells):
        g = [F32(start)]
        for c in cells:
            g.append(F32(float(g[-1]) + step * c))
        return np.array(g, dtype=np.float32)

    gx, gy, gz = axis(x0, df, sp["igridx"]), axis(y0, dq, sp["igridy"]), axis(z0, h, sp["igridz"])
    g = RayGrid(nx, ny, nz, sp["nxc"], sp["nyc"], sp["nzc"], x0, y0, z0, h, dq, df,
                gx.ctypes.data_as(C.POINTER(C.c_float)), gy.ctypes.data_as(C.POINTER(C.c_float)),
                gz.ctypes.data_as(C.POINTER(C.c_float)))
    return g, (gx, gy, gz)


def read_stations(path: str) -> list[dict]:
    """Station list (:818-851): lat/lon of columns 5-6, elevation (m) of column 3, corrections 7-8."""
    out = []
    with open(path) as fh:
        for line in fh:
            f = line.split()
            if not f:
                break
            slat, slon = F32(f[4]), F32(f[5])
            out.append(dict(name=f[3], xs=float(F32(float(slon) * DEGRAD)),
                            ys=float(F32(HPI - glat(float(slat) * DEGRAD))),
                            zs=float(-(F32(int(f[2])) / F32(1000.0))),
                            tc=(float(F32(f[6])), float(F32(f[7])))))
    return out


_FLOAT = re.compile(r"\s*[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?")


def read_events(path: str) -> list[dict]:
    """Local earthquake file (:880-1048): a header line per event, one line per phase, a blank line."""
    events = []
    with open(path) as fh:
        lines = fh.read().split("\n")
    i = 0
    while i < len(lines):
        if not lines[i].strip():
            i += 1
            continue
        f = lines[i].split()
        ev = dict(kyr=int(f[0]), kday=int(f[1]), khr=int(f[2]), kmn=int(f[3]), esec=float(F32(f[4])),
                  xlat=float(f[5]), xlon=float(f[6]), dep=float(F32(f[7])), evid=f[8] if len(f) > 8 else "",
                  obs=[])
        i += 1
        while i < len(lines) and lines[i].strip():
            # "%s %d %d %d %d %f %99[^\n]" then " %c %f" on the rest, whose leading '*' (an outlier
            # mark written straight after the seconds) is blanked first (:1017-1030)
            g = lines[i].strip().split(None, 5)
            m = _FLOAT.match(g[5])
            rest = g[5][m.end():].lstrip()
            if rest.startswith("*"):
                rest = " " + rest[1:]
            rest = rest.lstrip()
            ph = rest[:1]
            mw = _FLOAT.match(rest[1:])
            rwt = F32(mw.group(0)) if mw else F32(0)
            ph = {"0": "P", "1": "S"}.get(ph, ph)
            ev["obs"].append(dict(sta=g[0], iyr=int(g[1]), jday=int(g[2]), ihr=int(g[3]), imn=int(g[4]),
                                  sec=float(F32(m.group(0))), phase=ph, rwt=rwt))
            i += 1
        events.append(ev)
    return events


# ------------------------------------------------------------------------------------------------
# observations for the tracer


def event_cell(grid: RayGrid, ev: dict):
    """(ex, ey, ez) and whether the event lies inside the model (:924-947)."""
    ex = ev["xlon"] * DEGRAD
    ey = HPI - glat(ev["xlat"] * DEGRAD)
    ez = ev["dep"]
    ies = int((ex - grid.x0) / grid.df)
    jes = int((ey - grid.y0) / grid.dq)
    kes = int((ez - grid.z0) / grid.h)
    inside = not ((ex < grid.x0 or ies >= grid.nx - 1) or (ey < grid.y0 or jes >= grid.ny - 1)
                  or (ez < grid.z0 or kes >= grid.nz - 1))
    return (ex, ey, ez), inside


def build_observations(sp: dict, grid: RayGrid, stations: list[dict], events: list[dict]):
    """Observations of the events inside the model, in file order, with the time fields they need.

    Returns (obs array, plan, fields) where plan[e] = (inside, [(obs index or -1, phase index)]) per
    event and fields = [(station, 'p'|'s')] in first-use order."""
    by_name: dict[str, int] = {}
    for k, s in enumerate(stations):
        by_name.setdefault(s["name"], k)
    fields: list[tuple[str, str]] = []
    fidx: dict[tuple[str, str], int] = {}
    obs = []
    plan = []
    for ev in events:
        (ex, ey, ez), inside = event_cell(grid, ev)
        rows = []
        if inside:
            dpot = htoe(ev["kyr"], ev["kday"], ev["khr"], ev["kmn"], ev["esec"])
            for o in ev["obs"]:
                iph = 1 if o["phase"] == "S" else 0
                kn = by_name.get(o["sta"])
                if kn is None:
                    rows.append((-1, iph))
                    continue
                st = stations[kn]
                key = (o["sta"], "p" if (o["phase"] == "P" or sp["ivs"] == 0) else "s")
                if key not in fidx:
                    fidx[key] = len(fields)
                    fields.append(key)
                tarr = htoe(o["iyr"], o["jday"], o["ihr"], o["imn"], o["sec"])
                pwt = F32(1.0) / (o["rwt"] * o["rwt"])
                rows.append((len(obs), iph))
                obs.append(RayObs(ex, ey, ez, st["xs"], st["ys"], st["zs"], fidx[key], iph,
                                  float(F32(tarr - dpot)), float(pwt), st["tc"][iph], 0))
        plan.append((inside, rows))
    arr = (RayObs * max(1, len(obs)))(*obs)
    return arr, len(obs), plan, fields


def load_fields(sp: dict, grid: RayGrid, fields: list[tuple[str, str]]) -> list[np.ndarray]:
    """The time files (:1160-1218): a 232-byte header when the file starts with HEAD."""
    n = grid.nx * grid.ny * grid.nz
    out = []
    for sta, ph in fields:
        with open(os.path.join(sp["timedir"], f"{sta}.{ph}times"), "rb") as fh:
            raw = fh.read()
        off = 232 if raw[:4] == b"HEAD" else 0
        out.append(np.frombuffer(raw, dtype=np.float32, count=n, offset=off).copy())
    return out


# ------------------------------------------------------------------------------------------------
# the inversion files


class Assembler:
    """The event loop's bookkeeping and the six output files, as the reference keeps them."""

    def __init__(self, grid: RayGrid):
        nxyzc = grid.nxc * grid.nyc * grid.nzc
        self.maxvarc = nxyzc
        self.mhit = np.zeros(2 * nxyzc + 8, dtype=np.int32)
        self.mndex = np.zeros(2 * nxyzc + 8, dtype=np.int64)
        self.nhit = np.zeros(2 * nxyzc + 8, dtype=np.int64)
        self.indx = np.zeros(2 * nxyzc + 8, dtype=np.int64)
        self.mndm: dict[int, int] = {}
        self.jndx: list[int] = []
        self.kbl = 0
        self.vmp: dict[tuple[int, int], np.float32] = {}
        self.dat: dict[int, np.float32] = {}
        self.nev = 0
        self.dts = bytearray()
        self.res = bytearray()
        self.dth: list[str] = []
        self.bok: list[str] = []

    def event(self, inside: bool, rows, results, off, idx, du):
        """One event: rows[i] = (observation index or -1, phase); results, off, idx, du the tracer's
        (observation o's derivatives at idx/du[off[o] .. off[o] + nnz))."""
        self.nev += 1
        if not inside:
            return
        nsta = len(rows)
        isgood = [0] * nsta
        inbk = [0] * nsta
        vm: dict[tuple[int, int], np.float32] = {}
        ind: dict[tuple[int, int], int] = {}
        am = {}
        for i, (o, iph) in enumerate(rows):
            if o < 0:
                continue
            r = results[o]
            isgood[i] = 1
            if r.status != RAY_OK:
                isgood[i] = 0
                continue
            if i == 0:
                self.kbl = 0
                self.mhit[:] = 0
            wet = F32(r.wet)
            self.dat[i] = F32(r.dt * float(wet))
            am[i] = [F32(v) for v in r.am]
            nbk = 0
            base = int(off[o])
            for q in range(r.nnz):
                jb = int(idx[base + q])
                j = jb + (self.maxvarc if iph == 1 else 0)
                vm[(nbk, i)] = F32(du[base + q]) * wet
                ind[(nbk, i)] = j
                nbk += 1
                if self.mhit[j] == 0:
                    self.mndm[self.kbl] = j
                    self.mndex[j] = self.kbl
                    self.mhit[j] = 1
                    self.kbl += 1
                if self.nhit[j] == 0:
                    self.indx[j] = len(self.jndx)
                    self.jndx.append(j)
                self.nhit[j] += 1
            inbk[i] = nbk
        kbl = self.kbl
        for j1 in range(nsta):
            for j2 in range(kbl):
                if (j2, j1) in self.vmp:
                    self.vmp[(j2, j1)] = F32(0)
        for k in range(nsta):
            if isgood[k]:
                for j1 in range(inbk[k]):
                    jnd = int(self.mndex[ind[(j1, k)]])
                    self.vmp[(jnd, k)] = F32(self.vmp.get((jnd, k), F32(0)) + vm[(j1, k)])
        nwrt = 0
        for j1 in range(nsta):
            if not isgood[j1]:
                continue
            ja = [i1 for i1 in range(kbl) if self.vmp.get((i1, j1), F32(0)) != 0]
            if not ja:
                continue
            self.dts += struct.pack("<i", len(ja))
            for i1 in ja:
                self.dts += struct.pack("<if", int(self.indx[self.mndm[i1]]) + 1, self.vmp[(i1, j1)])
            self.res += struct.pack("<f", self.dat.get(j1, F32(0)))
            for v in am[j1]:
                self.dth.append("%f\n" % float(v))
            nwrt += 1
        self.bok.append("%d %d\n" % (self.nev, nwrt))

    def files(self) -> dict[str, bytes]:
        mbl = len(self.jndx)
        dts = bytes(self.dts) + struct.pack("<ii", -1, mbl) + struct.pack(f"<{mbl}i", *self.jndx)
        msc = "%d\n" % mbl + "".join("%d\n" % j for j in self.jndx)
        hit = "%d" % mbl + "".join("%d %d\n" % (j, self.nhit[j]) for j in self.jndx)
        bok = "".join(self.bok) + "%d %d\n" % (-2, -2)
        return dict(dtdsfil=dts, resfile=bytes(self.res), dtdhfil="".join(self.dth).encode(),
                    bookfil=bok.encode(), sclefil=msc.encode(), hitfile=hit.encode())


def default_max_seg(grid: RayGrid) -> int:
    """Segments after which a ray is abandoned (status RAY_STEPS).  The reference has no limit; a ray
    that reaches its station crosses each cell wall about once, so this is far above any real ray."""
    return 16 * (grid.nx + grid.ny + grid.nz) + 256


def default_cap(grid: RayGrid) -> int:
    """Room for one ray's nonzero coarse derivatives."""
    return 8 * (grid.nx + grid.ny + grid.nz) + 64


def run(specfile: str, trace, cap: int | None = None, spacing_rule: bool = True,
        write: bool | None = None) -> dict[str, bytes]:
    """sphrayderv on one spec: trace(grid, fields, obs, nobs, cap) -> (results, off, idx, du) does
    the rays (fields as host arrays); returns the file contents by spec name and writes them where
    the spec says.  spacing_rule: as grid_from_spec.  write: None writes unless `trace` is a sharded
    tracer on a rank other than 0 (ranks that share a file system then do not write the same files
    at once); every rank returns the contents."""
    sp = read_spec(specfile)
    if sp["ivpvs"] or sp["dotel"] or sp["doshot"] or sp["nomat"]:
        raise ValueError("only local earthquakes with ivpvs 0 and nomat 0 are supported")
    grid, keep = grid_from_spec(sp, spacing_rule)
    stations = read_stations(sp["stafile"])
    events = read_events(sp["locdfil"])
    obs, nobs, plan, fields = build_observations(sp, grid, stations, events)
    tfields = load_fields(sp, grid, fields)
    if cap is None:
        cap = default_cap(grid)
    results, off, idx, du = trace(grid, tfields, obs, nobs, cap)
    asm = Assembler(grid)
    for inside, rows in plan:
        asm.event(inside, rows, results, off, idx, du)
    out = asm.files()
    if write is None:
        writer = getattr(trace, "writes", None)
        write = writer() if writer else True
    if write:
        for name, data in out.items():
            with open(sp[name], "wb") as fh:
                fh.write(data)
    del keep
    return out


def gpu_trace(ctx=None, device: int | None = None):
    """A tracer for run(): the fields go to the device and fdgpu_raytrace traces the rays.  The device
    defaults to $LOCAL_RANK (0 when unset), so that each rank of a sharded run uses its own GPU."""
    from . import lib as L
    if device is None:
        device = ctx.device if ctx is not None and hasattr(ctx, "device") else int(os.environ.get("LOCAL_RANK", 0))

    def trace(grid, fields, obs, nobs, cap):
        import torch
        dev = [torch.from_numpy(np.ascontiguousarray(f, dtype=np.float32)).to(f"cuda:{device}") for f in fields]
        own = ctx is None
        c = L.Context(device) if own else ctx
        try:
            return L.raytrace(c, grid, [t.data_ptr() for t in dev], obs, nobs, cap=cap)
        finally:
            if own:
                c.close()

    return trace


def sharded(trace, group=None):
    """A tracer that splits the observations over the ranks of a torch.distributed group: rank r traces
    the r-th contiguous slice with `trace` (on its own GPU), and one all-gather of the results gives
    every rank the whole run, in observation order, so that each can write the files.  Observations are
    independent; the tracing itself exchanges nothing."""

    def run(grid, fields, obs, nobs, cap):
        import torch.distributed as dist
        world = dist.get_world_size(group)
        rank = dist.get_rank(group)
        lo, hi = nobs * rank // world, nobs * (rank + 1) // world
        sub = (RayObs * max(1, hi - lo))(*[obs[i] for i in range(lo, hi)])
        res, off, idx, du = trace(grid, fields, sub, hi - lo, cap)
        mine = (C.string_at(C.addressof(res), C.sizeof(RayResult) * (hi - lo)),
                np.asarray(idx[: int(off[hi - lo])], dtype=np.int32).tobytes(),
                np.asarray(du[: int(off[hi - lo])], dtype=np.float32).tobytes())
        parts = [None] * world
        dist.all_gather_object(parts, mine, group=group)
        all_res = (RayResult * max(1, nobs))()
        raw = b"".join(p[0] for p in parts)
        C.memmove(C.addressof(all_res), raw, len(raw))
        idx_all = np.frombuffer(b"".join(p[1] for p in parts), dtype=np.int32)
        du_all = np.frombuffer(b"".join(p[2] for p in parts), dtype=np.float32)
        off_all = np.zeros(nobs + 1, dtype=np.int64)
        np.cumsum([all_res[o].nnz for o in range(nobs)], out=off_all[1:])
        return all_res, off_all, idx_all, du_all

    def writes():
        import torch.distributed as dist
        return dist.get_rank(group) == 0

    run.writes = writes
    return run
