"""Seeded cases for sphrayderv's ray tracing (reference src/sphrayderv.c).

A case is a fine grid with a coarse metagrid over it, stations at arbitrary surface points, and for
each station a P and an S travel-time field: straight-ray distance in the reference's spherical
frame divided by a velocity, times a smooth factor (1 + a sin(..) cos(..)) so that the gradient, and
with it the rays, bend.  Events sit inside the grid; their picks are the fields' times at the event
plus seeded noise.  Some picks name a station missing from the list, and one event in some cases
lies outside the model, so that the reference's skip paths run too.

make_ray_golden.py writes each case as the reference's inputs, runs the reference's own sphrayderv
on them and keeps its six output files; the tests rebuild the inputs here and compare.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from fdtomoc_gb300 import rayderv as R
from fdtomoc_gb300.formats import VHead, write_grid

HERE = os.path.dirname(os.path.abspath(__file__))
SEEDS = (1, 2, 3, 4, 5, 6)
# further cases pinned on the CPU: 7 ivs 0 (S phases read the P tables), 8 dq = df = 0 (spacing from h),
# 9 events inside their stations' cells, 10 a finer and larger grid
EXTRA_SEEDS = (7, 8, 9, 10)


def make_case(seed: int) -> dict:
    rng = np.random.default_rng(1000 + seed)
    nxc, nyc, nzc = int(rng.integers(5, 8)), int(rng.integers(5, 8)), int(rng.integers(4, 6))
    big = seed == 10
    p = dict(seed=seed, nxc=nxc, nyc=nyc, nzc=nzc,
             igridx=[int(v) for v in rng.integers(6 if big else 3, 12 if big else 8, nxc - 1)],
             igridy=[int(v) for v in rng.integers(6 if big else 3, 12 if big else 8, nyc - 1)],
             igridz=[int(v) for v in rng.integers(2, 5, nzc - 1)],
             h=0.5 if big else float(rng.choice([1.0, 2.0])), x0=120.5, y0=23.5, z0=-1.0,
             dq=0.006 if big else 0.01, df=0.006 if big else 0.01,
             vp=6.0, vs=3.5, amp=float(rng.uniform(0.0, 0.05)), kx=float(rng.uniform(1, 3)),
             ky=float(rng.uniform(1, 3)), ivs=0 if seed == 7 else 1)
    if seed == 8:
        p["dq"] = p["df"] = 0.0
    nx, ny, nz = 1 + sum(p["igridx"]), 1 + sum(p["igridy"]), 1 + sum(p["igridz"])
    p.update(nx=nx, ny=ny, nz=nz)
    dlat = p["dq"] or math.degrees(p["h"] / R.REARTH)
    dlon = p["df"] or dlat / math.cos(math.radians(p["y0"]))
    lat_top, lat_bot = p["y0"], p["y0"] - (ny - 1) * dlat
    lon_w, lon_e = p["x0"], p["x0"] + (nx - 1) * dlon
    st = []
    for k in range(int(rng.integers(6, 10))):
        st.append(dict(name=f"ST{k:02d}", lat=round(float(rng.uniform(lat_bot + 0.02, lat_top - 0.02)), 5),
                       lon=round(float(rng.uniform(lon_w + 0.02, lon_e - 0.02)), 5),
                       elev=int(rng.integers(0, 900)),
                       tcp=round(float(rng.uniform(-0.1, 0.1)), 3), tcs=round(float(rng.uniform(-0.1, 0.1)), 3)))
    p["stations"] = st
    # odd seeds: one station's P table has no times (> 1e9) below mid-depth, as sphfd leaves nodes
    # it never reached; even seeds: one station's tables come from a source beyond the east edge, so
    # rays that follow them leave the model
    p["notime"] = dict(station=int(rng.integers(0, len(st))), k=int(nz // 2)) if seed % 2 else None
    p["moved"] = dict(station=int(rng.integers(0, len(st))), dlon=0.4) if seed % 2 == 0 else None
    zmax = p["z0"] + (nz - 1) * p["h"]
    events = []
    for e in range(int(rng.integers(4, 8))):
        ev = dict(evid=f"E{seed:02d}{e:02d}", year=2021, jday=int(rng.integers(1, 365)),
                  hour=int(rng.integers(0, 24)), minute=int(rng.integers(0, 60)),
                  sec=round(float(rng.uniform(0, 50)), 2),
                  lat=round(float(rng.uniform(lat_bot + 0.03, lat_top - 0.03)), 5),
                  lon=round(float(rng.uniform(lon_w + 0.03, lon_e - 0.03)), 5),
                  dep=round(float(rng.uniform(1.0, zmax - 1.5)), 3), picks=[])
        if e == 2 and seed % 3 == 0:
            ev["lon"] = round(lon_e + 0.05, 5)     # outside the model: the event is skipped
        if seed == 9 and e % 2 == 0:               # in (or next to) a station's cell
            s0 = st[e % len(st)]
            ev["lat"], ev["lon"] = round(s0["lat"] + 0.0004, 5), round(s0["lon"] - 0.0004, 5)
            ev["dep"] = round(float(rng.uniform(-0.5, 0.8)), 3)
        events.append(ev)
    p["events"] = events
    return p


def _frame(p):
    sp = spec_dict(p, "")
    g, keep = R.grid_from_spec(sp)
    return sp, g, keep


def _xyz(lon, colat, r):
    return r * np.sin(colat) * np.cos(lon), r * np.sin(colat) * np.sin(lon), r * np.cos(colat)


def field(p, g, s, phase, moved=0.0) -> np.ndarray:
    """straight-ray time from the station (its longitude moved by `moved` degrees), scaled by a
    smooth factor, on the fine grid"""
    i = np.arange(g.nx, dtype=np.float64)
    j = np.arange(g.ny, dtype=np.float64)
    k = np.arange(g.nz, dtype=np.float64)
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    lon = g.x0 + g.df * I
    colat = g.y0 + g.dq * J
    r = R.REARTH - (g.z0 + g.h * K)
    x, y, z = _xyz(lon, colat, r)
    sx, sy, sz = _xyz(s["xs"] + moved * R.DEGRAD, s["ys"], R.REARTH - s["zs"])
    d = np.sqrt((x - sx) ** 2 + (y - sy) ** 2 + (z - sz) ** 2)
    v = p["vp"] if phase == "P" else p["vs"]
    fac = 1.0 + p["amp"] * np.sin(p["kx"] * np.pi * I / (g.nx - 1)) * np.cos(p["ky"] * np.pi * J / (g.ny - 1))
    return (d / v * fac).astype(np.float32)


def _time_at(f, g, ex, ey, ez):
    fi, fj, fk = (ex - g.x0) / g.df, (ey - g.y0) / g.dq, (ez - g.z0) / g.h
    i, j, k = int(fi), int(fj), int(fk)
    a, b, c = fi - i, fj - j, fk - k
    v = 0.0
    for dk in (0, 1):
        for dj in (0, 1):
            for di in (0, 1):
                w = (a if di else 1 - a) * (b if dj else 1 - b) * (c if dk else 1 - c)
                v += w * float(f[k + dk, j + dj, i + di])
    return v


def spec_dict(p, d):
    return dict(nxc=p["nxc"], nyc=p["nyc"], nzc=p["nzc"], h=p["h"], x0=p["x0"], y0=p["y0"], z0=p["z0"],
                dq=p["dq"], df=p["df"], ivs=p["ivs"], ivpvs=0, dotel=0, doshot=0, nomat=0,
                timedir=os.path.join(d, "ttimes"), igridx=p["igridx"], igridy=p["igridy"], igridz=p["igridz"])


def spec_text(p, d) -> str:
    lines = [f"nxc {p['nxc']}", f"nyc {p['nyc']}", f"nzc {p['nzc']}", f"h {p['h']}",
             f"stafile {d}/stations.txt", f"locdfil {d}/events.txt", f"oldvfil {d}/old.mod",
             f"telrerr {d}/out/telrerr.txt", f"dtdsfil {d}/out/dtds.bin", f"resfile {d}/out/res.bin",
             f"hitfile {d}/out/hit.txt", f"dtdhfil {d}/out/dtdh.txt", f"bookfil {d}/out/book.txt",
             f"sclefil {d}/out/scle.txt", f"timedir {d}/ttimes", "idatout 0", "iraystat 0", "iray 0",
             f"ivs {p['ivs']}", f"x0 {p['x0']}", f"y0 {p['y0']}", f"z0 {p['z0']}", f"dq {p['dq']}",
             f"df {p['df']}", "ittnum 0",
             "igridx " + " ".join(map(str, p["igridx"])), "igridy " + " ".join(map(str, p["igridy"])),
             "igridz " + " ".join(map(str, p["igridz"]))]
    return "\n".join(lines) + "\n"


def write_inputs(p, d) -> str:
    """Spec, station list, events and time files under d; returns the spec path."""
    os.makedirs(os.path.join(d, "ttimes"), exist_ok=True)
    os.makedirs(os.path.join(d, "out"), exist_ok=True)
    with open(os.path.join(d, "stations.txt"), "w") as fh:
        for s in p["stations"]:
            fh.write(f"{s['lat']:.5f} {s['lon']:.5f} {s['elev']} {s['name']} {s['lat']:.5f} {s['lon']:.5f} "
                     f"{s['tcp']:.3f} {s['tcs']:.3f}\n")
    sp, g, keep = _frame(p)
    stations = R.read_stations(os.path.join(d, "stations.txt"))
    rng = np.random.default_rng(2000 + p["seed"])
    head = VHead(header=b"HEADFINESPHRPTIM", nx=g.nx, ny=g.ny, nz=g.nz, dz=g.h)
    fields = {}
    for n, s in enumerate(stations):
        for ph in ("P", "S"):
            mv = p["moved"]["dlon"] if p.get("moved") and p["moved"]["station"] == n else 0.0
            f = field(p, g, s, ph, mv)
            if p.get("notime") and p["notime"]["station"] == n and ph == "P":
                f[p["notime"]["k"]:] = np.float32(1.0e10)
            fields[(s["name"], ph)] = f
            write_grid(os.path.join(d, "ttimes", f"{s['name']}.{ph.lower()}times"), head, f)
    with open(os.path.join(d, "events.txt"), "w") as fh:
        for ev in p["events"]:
            fh.write(f"{ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} {ev['sec']:.2f} "
                     f"{ev['lat']:.5f} {ev['lon']:.5f} {ev['dep']:.3f} {ev['evid']}\n")
            (ex, ey, ez), inside = R.event_cell(g, dict(xlat=ev["lat"], xlon=ev["lon"], dep=ev["dep"]))
            first_unknown = rng.random() < 0.4
            if first_unknown:      # the event's first phase fails: its bookkeeping starts from the last
                fh.write(f"YY77  {ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} {ev['sec'] + 2.0:7.3f} S"
                         f" {0.2:11.3f}\n")
            for s in stations:
                for ph in ("P", "S"):
                    if rng.random() < 0.25:
                        continue
                    tt = _time_at(fields[(s["name"], ph)], g, ex, ey, ez) if inside else 10.0
                    if tt > 1e6:
                        tt = 12.0
                    tt += float(rng.normal(0, 0.05))
                    mark = "*" if rng.random() < 0.05 else " "
                    fh.write(f"{s['name']}  {ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} "
                             f"{ev['sec'] + tt:7.3f}{mark}{ph} {float(rng.choice([0.05, 0.1, 0.2])):11.3f}\n")
            if rng.random() < 0.5:
                fh.write(f"XX99  {ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} {ev['sec'] + 3.0:7.3f} P"
                         f" {0.1:11.3f}\n")
            fh.write("\n")
    with open(os.path.join(d, "spec"), "w") as fh:
        fh.write(spec_text(p, d))
    del keep
    return os.path.join(d, "spec")


OUT_FILES = {"dtdsfil": "dtds.bin", "resfile": "res.bin", "dtdhfil": "dtdh.txt", "bookfil": "book.txt",
             "sclefil": "scle.txt", "hitfile": "hit.txt"}


def golden_dir(seed):
    return os.path.join(HERE, f"ray_{seed}")


def load_golden(seed) -> dict[str, bytes]:
    d = golden_dir(seed)
    out = {}
    for k, name in OUT_FILES.items():
        with open(os.path.join(d, name), "rb") as fh:
            out[k] = fh.read()
    return out


def save_case_json(p, d):
    with open(os.path.join(d, "case.json"), "w") as fh:
        json.dump(p, fh, indent=1)


__all__ = ["SEEDS", "make_case", "write_inputs", "load_golden", "golden_dir", "OUT_FILES", "math"]
