"""Seeded location cases for sphfdloc's grid search (reference src/sphfdloc.c), and the reference's
output text rebuilt from a location result.

A case is a small fine grid, a set of stations with synthetic P and S time fields (straight rays in
a constant-velocity half-space, in a flat local frame: only +, *, / and sqrt, so the fields are the
same on every machine), and events whose picks are the fields' times at a true hypocentre plus
seeded noise, with a few gross outliers so that the outlier / recovery passes run.

make_loc_golden.py writes each case as the reference's inputs (spec, time files, event list), runs
the reference's own sphfdloc on them and stores its output files as the golden fixtures; the tests
locate the same events with the oracle and the GPU path and rebuild the output text with
format_outputs() below.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from fdtomoc_gb300.formats import VHead, write_grid

HERE = os.path.dirname(os.path.abspath(__file__))


def make_case(seed: int) -> dict:
    rng = np.random.default_rng(seed)
    nxc, nyc, nzc = 5, 5, 5
    gx, gy, gz = int(rng.integers(6, 11)), int(rng.integers(6, 11)), int(rng.integers(3, 6))
    nx, ny, nz = 1 + gx * (nxc - 1), 1 + gy * (nyc - 1), 1 + gz * (nzc - 1)
    h = float(rng.choice([1.0, 2.0]))
    p = dict(seed=seed, nxc=nxc, nyc=nyc, nzc=nzc, igridx=[gx] * (nxc - 1), igridy=[gy] * (nyc - 1),
             igridz=[gz] * (nzc - 1), nx=nx, ny=ny, nz=nz, h=h, x0=120.5, y0=24.0, z0=-2.0,
             kmin=2, ndiv=int(rng.choice([4, 10, 20])), ndiv2=int(rng.choice([4, 10, 20])), nthres=6,
             resthres=0.5, resthrep=5.0, stdmax=15.0, vp=6.0, vs=3.5)
    if seed >= 5:
        p["ivs"], p["vpvs"] = 0, 1.75   # S times taken as the S field's times x vpvs (:745-747)
    nst = int(rng.integers(8, 14))
    p["stations"] = [dict(name=f"S{k:02d}", i=int(rng.integers(0, nx)), j=int(rng.integers(0, ny)), k=0)
                     for k in range(nst)]
    events = []
    for e in range(int(rng.integers(4, 8))):
        hx, hy, hz = rng.uniform(1, nx - 2), rng.uniform(1, ny - 2), rng.uniform(2.5, nz - 1.5)
        picks = []
        for s in p["stations"]:
            for ph in ("P", "S"):
                if rng.random() < 0.2:
                    continue
                tt = travel_time(p, s, ph, hx, hy, hz)
                if ph == "S" and p.get("ivs") == 0:
                    tt *= p["vpvs"]   # consistent with how ivs 0 reads an S time
                noise = float(rng.normal(0, 0.02))
                if rng.random() < 0.08:
                    noise += float(rng.choice([-1.5, 2.5]))   # a gross outlier
                picks.append(dict(sta=s["name"], phase=ph, t=tt + noise,
                                  rwt=float(rng.choice([0.05, 0.1, 0.2]))))
        events.append(dict(evid=f"EV{seed:03d}{e:02d}", year=2020, jday=int(rng.integers(1, 300)),
                           hour=int(rng.integers(0, 24)), minute=int(rng.integers(0, 60)),
                           sec=round(float(rng.uniform(0, 59)), 2), picks=picks))
    p["events"] = events
    return p


def _dx_km(p):
    # flat local frame: 0.01 deg of longitude and latitude per grid step, as km
    return 0.01 * 111.19 * math.cos(math.radians(p["y0"])), 0.01 * 111.19


def travel_time(p, s, phase, x, y, z):
    dx, dy = _dx_km(p)
    v = p["vp"] if phase == "P" else p["vs"]
    return math.sqrt(((x - s["i"]) * dx) ** 2 + ((y - s["j"]) * dy) ** 2 + ((z - s["k"]) * p["h"]) ** 2) / v


def field(p, s, phase) -> np.ndarray:
    dx, dy = _dx_km(p)
    v = p["vp"] if phase == "P" else p["vs"]
    k, j, i = np.meshgrid(np.arange(p["nz"], dtype=np.float64), np.arange(p["ny"], dtype=np.float64),
                          np.arange(p["nx"], dtype=np.float64), indexing="ij")
    d = np.sqrt(((i - s["i"]) * dx) ** 2 + ((j - s["j"]) * dy) ** 2 + ((k - s["k"]) * p["h"]) ** 2)
    return (d / v).astype(np.float32)


def fields(p):
    """{(station, phase): (nz, ny, nx) float32}"""
    return {(s["name"], ph): field(p, s, ph) for s in p["stations"] for ph in ("P", "S")}


def event_text(p) -> str:
    """The event list the reference reads (leqsfil): a header line per event, one line per pick
    with its absolute arrival time, a blank line after each event."""
    out = []
    for ev in p["events"]:
        out.append(f"{ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} {ev['sec']:.2f} 24.0 121.0 5.0 {ev['evid']}\n")
        for pk in ev["picks"]:
            # arrival = origin + travel time, written as seconds past the origin minute
            out.append(f"{pk['sta']} {ev['year']} {ev['jday']} {ev['hour']} {ev['minute']} "
                       f"{ev['sec'] + pk['t']:.3f} {pk['phase']} {pk['rwt']:.2f}\n")
        out.append("\n")
    return "".join(out)


def spec_text(p, d) -> str:
    lines = [f"nxc {p['nxc']}", f"nyc {p['nyc']}", f"nzc {p['nzc']}", f"h {p['h']}",
             f"leqsfil {d}/events.txt", f"fsumfil {d}/out/sum.txt", f"outlfil {d}/out/out.txt",
             f"fhedfil {d}/out/fhd.txt", f"fdatfil {d}/out/dat.txt", f"timedir {d}/ttimes",
             f"eqkdir {d}/eqkdir/", f"x0 {p['x0']}", f"y0 {p['y0']}", f"z0 {p['z0']}",
             f"kmin {p['kmin'] + 1}", f"ndiv {p['ndiv']}", f"ndiv2 {p['ndiv2']}", f"nthres {p['nthres']}",
             f"resthres {p['resthres']}", f"resthrep {p['resthrep']}", f"stdmax {p['stdmax']}",
             "igridx " + " ".join(map(str, p["igridx"])), "igridy " + " ".join(map(str, p["igridy"])),
             "igridz " + " ".join(map(str, p["igridz"]))]
    if "ivs" in p:
        lines += [f"ivs {p['ivs']}", f"vpvs {p['vpvs']}"]
    return "\n".join(lines) + "\n"


def write_reference_inputs(p, d):
    os.makedirs(os.path.join(d, "ttimes"), exist_ok=True)
    os.makedirs(os.path.join(d, "out"), exist_ok=True)
    os.makedirs(os.path.join(d, "eqkdir"), exist_ok=True)
    head = VHead(header=b"HEADFINESPHRPTIM", nx=p["nx"], ny=p["ny"], nz=p["nz"], dz=p["h"])
    for (name, ph), f in fields(p).items():
        write_grid(os.path.join(d, "ttimes", f"{name}.{ph.lower()}times"), head, f)
    with open(os.path.join(d, "events.txt"), "w") as fh:
        fh.write(event_text(p))
    with open(os.path.join(d, "spec"), "w") as fh:
        fh.write(spec_text(p, d))
    return os.path.join(d, "spec")


def parsed_events(p, htoe):
    """Events as the reference reads them (:583-667): origin epoch from the header's float seconds,
    obstime = float(arrival epoch - origin epoch), weight 1/rwt^2 in float."""
    out = []
    for ev in p["events"]:
        dsec = float(np.float32(float(f"{ev['sec']:.2f}")))
        dpot = htoe(ev["year"], ev["jday"], ev["hour"], ev["minute"], dsec)
        obs = []
        for pk in ev["picks"]:
            sec = float(np.float32(float(f"{ev['sec'] + pk['t']:.3f}")))
            tarr = htoe(ev["year"], ev["jday"], ev["hour"], ev["minute"], sec)
            rwt = np.float32(float(f"{pk['rwt']:.2f}"))
            obs.append(dict(sta=pk["sta"], phase=pk["phase"], obstime=float(np.float32(tarr - dpot)),
                            pwt=float(np.float32(1.0) / (rwt * rwt)), rwt=float(rwt)))
        out.append(dict(evid=ev["evid"], dpot=dpot, obs=obs))
    return out


def f32(x):
    return float(np.float32(x))


def format_outputs(p, events, results, ora):
    """The reference's four output files (fhedfil, fdatfil, fsumfil, outlfil; :1129-1250) for located
    events.  results[e] = dict(status, nxx, nyy, nzz, exm, eym, ezm, stdmin, avrmin, ngood,
    good[], resmin[], tps[]); ora gives htoe/etoh/glathinv and the grid's z0r."""
    fhd, dat, sm, out = [], [], [], []
    hpi, degrad, z0, z0r = ora["hpi"], ora["degrad"], p["z0"], ora["z0r"]
    for nev, (ev, r) in enumerate(zip(events, results)):
        nsta = len(ev["obs"])
        xlon = f32(r["exm"] / degrad)
        lat, ezmr = ora["glathinv"](hpi - r["eym"], z0r - (r["ezm"] - z0))
        xlat = f32(lat / degrad)
        iyr, jday, ihr, imn, dsec = ora["etoh"](ev["dpot"] + r["avrmin"])
        sec = f32(dsec)
        stdmin = r["stdmin"]
        res_dm = [f32(r["resmin"][i] - r["avrmin"]) for i in range(nsta)]
        if r["status"] == 1:
            if stdmin == float("inf"):
                out.append("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s    **********\n"
                           % (iyr, jday, ihr, imn, sec, xlat, xlon, ezmr, ev["evid"]))
            else:
                out.append("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n"
                           % (iyr, jday, ihr, imn, sec, xlat, xlon, ezmr, ev["evid"], stdmin))
            for j, o in enumerate(ev["obs"]):
                tarr = f32(o["obstime"] + ev["dpot"])
                y2, d2, h2, m2, s2 = ora["etoh"](tarr)
                out.append("%s %4d %3d %2d %2d %7.3f*%c %15.3f %10.3f\n"
                           % (o["sta"], y2, d2, h2, m2, s2, o["phase"], o["rwt"], res_dm[j]))
            out.append("\n")
            continue
        if r["status"] != 0:
            continue   # stdmin above stdmax: the reference writes nothing
        line = ("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n"
                % (iyr, jday, ihr, imn, sec, xlat, xlon, ezmr, ev["evid"], stdmin))
        dat.append(line)
        fhd.append(line)
        if r["ngood"] < nsta:
            out.append("%4d %3d %2d %2d %8.4f %9.5f %10.5f %8.4f %12s %13.3f\n"
                       % (iyr, jday, ihr, imn, sec, r["exm"], r["eym"], ezmr, ev["evid"], stdmin))
        sm.append("\n\n")
        sm.append("  Minimum Standard Deviation   : %12.8f\n" % stdmin)
        sm.append("  Info Density Maximum for event %12d\n" % nev)
        sm.append("%4d %3d %2d %2d %8.4f  %8.5f %10.5f %8.4f %12s %13.3f\n"
                  % (iyr, jday, ihr, imn, sec, r["exm"], r["eym"], ezmr, ev["evid"], stdmin))
        sm.append(" Event ID: %7s\n" % ev["evid"])
        sm.append("  Minimum Standard Deviation   : %12.8f\n" % stdmin)
        sm.append("  Maximum Sigma                :   2.51547135E+15\n")
        sm.append("  Total Sigma                  :    0.0000000    \n")
        sm.append("  Optimal Grid point (nx,ny,nz): %12d %11d %11d\n" % (r["nxx"] + 1, r["nyy"] + 1, r["nzz"] + 1))
        sm.append("  Average residual             :   %10.8f\n" % r["avrmin"])
        sm.append("  Hypocenter (lat, lon ,z )    :   %12.3f  %12.3f  %12.3f\n\n" % (xlat, xlon, ezmr))
        sm.append("  Station statistics at this point: \n")
        sm.append(" Code  Ph  Demeaned    True   Expected  Used   Tobs     Tcalc     To-Tc \n")
        sm.append("           Residual   Weight   Uncert.  Flag    Abs      Abs     \n\n")
        for i, o in enumerate(ev["obs"]):
            wt = o["pwt"]
            sm.append("%4s   %c %10.4f %9.3E %9.4f %3d %9.4f %9.4f %9.4f\n"
                      % (o["sta"], o["phase"], res_dm[i], wt, 1.0 / f32(math.sqrt(wt)), r["good"][i], o["obstime"],
                         r["tps"][i], f32(o["obstime"] - r["tps"][i])))
        sm.append("\n")
        for j, o in enumerate(ev["obs"]):
            y2, d2, h2, m2, s2 = ora["etoh"](o["obstime"] + ev["dpot"])
            if r["good"][j]:
                t = ("%-6s%4d %3d %2d %2d %7.3f %c %15.3f %10.3f\n"
                     % (o["sta"], y2, d2, h2, m2, s2, o["phase"], o["rwt"], res_dm[j]))
            else:
                t = ("%-6s%4d %3d %2d %2d %7.3f*%c %15.3f %10.3f\n"
                     % (o["sta"], y2, d2, h2, m2, s2, o["phase"], o["rwt"], res_dm[j]))
                out.append(t)
            dat.append(t)
        dat.append(" \n")
    return dict(fhd="".join(fhd), dat="".join(dat), sum="".join(sm), out="".join(out))


def golden_dir(seed):
    return os.path.join(HERE, f"loc_{seed}")


def load_golden(seed):
    d = golden_dir(seed)
    p = json.load(open(os.path.join(d, "case.json")))
    outs = {k: open(os.path.join(d, f"ref_{k}.txt")).read() for k in ("fhd", "dat", "sum", "out")}
    return p, outs


SEEDS = (1, 2, 3, 4, 5, 6)
