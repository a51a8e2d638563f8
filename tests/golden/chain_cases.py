"""sphfdloc then sphrayderv on one spec, as run.sh runs them (reference src/sphfdloc.c, src/sphrayderv.c):
the location cases of loc_cases.py, whose located-event report (fdatfil) is sphrayderv's event file,
plus the station list sphrayderv reads.  Stations sit on their fields' source nodes in sphrayderv's
frame (spacing derived from h, as neither program is given dq or df here).

make_chain_golden.py runs the reference's two programs in turn and keeps their ten output files; the
tests run the two drop-ins (fdgpu_sphfdloc, fdgpu_sphrayderv) on the same inputs and compare.
"""
from __future__ import annotations

import json
import math
import os

import loc_cases as LC

from fdtomoc_gb300 import rayderv as R

HERE = os.path.dirname(os.path.abspath(__file__))
SEEDS = (1, 2, 3, 4)
LOC_FILES = {"fhd": "fhd.txt", "dat": "dat.txt", "sum": "sum.txt", "out": "out.txt"}
RAY_FILES = {"dtdsfil": "dtds.bin", "resfile": "res.bin", "dtdhfil": "dtdh.txt", "bookfil": "book.txt",
             "sclefil": "scle.txt", "hitfile": "hit.txt"}


def _station_lines(p):
    """lat/lon of each station's source node in sphrayderv's frame (geographic, through glat's inverse)"""
    x0 = p["x0"] * R.DEGRAD
    y0 = R.HPI - R.glat(p["y0"] * R.DEGRAD)
    dq = p["h"] / R.REARTH
    df = abs(p["h"] / (R.REARTH * math.sin(y0)))
    elfac = float(R.F32(0.993277))
    lines = []
    for s in p["stations"]:
        lon = (x0 + s["i"] * df) / R.DEGRAD
        gc = R.HPI - (y0 + s["j"] * dq)
        lat = math.atan(math.tan(gc) / elfac) / R.DEGRAD
        elev = int(round(-p["z0"] * 1000.0))          # on the top layer, z = z0
        lines.append(f"{lat:.6f} {lon:.6f} {elev} {s['name']} {lat:.6f} {lon:.6f} 0.000 0.000\n")
    return "".join(lines)


def write_inputs(p, d) -> str:
    """The location case's inputs plus sphrayderv's entries in the same spec; returns the spec path."""
    spec = LC.write_reference_inputs(p, d)
    with open(os.path.join(d, "stations.txt"), "w") as fh:
        fh.write(_station_lines(p))
    os.makedirs(os.path.join(d, "ray"), exist_ok=True)
    with open(spec, "a") as fh:
        fh.write(f"stafile {d}/stations.txt\nlocdfil {d}/out/dat.txt\noldvfil {d}/old.mod\n"
                 f"telrerr {d}/ray/telrerr.txt\ndtdsfil {d}/ray/dtds.bin\nresfile {d}/ray/res.bin\n"
                 f"hitfile {d}/ray/hit.txt\ndtdhfil {d}/ray/dtdh.txt\nbookfil {d}/ray/book.txt\n"
                 f"sclefil {d}/ray/scle.txt\nidatout 0\n")
    return spec


def golden_dir(seed):
    return os.path.join(HERE, f"chain_{seed}")


def load_golden(seed):
    d = golden_dir(seed)
    with open(os.path.join(d, "case.json")) as fh:
        p = json.load(fh)
    out = {}
    for k, name in list(LOC_FILES.items()) + list(RAY_FILES.items()):
        with open(os.path.join(d, name), "rb") as fh:
            out[k] = fh.read()
    return p, out
