"""Seeded coarse models for c2f (reference src/c2f.c): grid specs with uneven node spacing and
spacings that are not exact binary fractions (so the float node coordinates and the fine-node
positions disagree in their last bits, the edge the cell scan must get right), and velocities made
with +, * and / only (the same on every machine).

make_c2f_golden.py runs the reference's own c2f on them and records the SHA-256 of its three output
files' data (the 232-byte header excluded); the tests rebuild the data with the oracle and the GPU.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from fdtomoc_gb300.formats import VHead, write_grid

HERE = os.path.dirname(os.path.abspath(__file__))
SEEDS = (1, 2, 3, 4, 5)


def make_case(seed: int) -> dict:
    rng = np.random.default_rng(100 + seed)
    nxc, nyc, nzc = (int(rng.integers(3, 10)) for _ in range(3))
    h = float(rng.choice([0.3, 0.5, 0.7, 1.0, 0.1]))
    p = dict(seed=seed, nxc=nxc, nyc=nyc, nzc=nzc, h=h,
             igridx=[int(v) for v in rng.integers(1, 8, nxc - 1)],
             igridy=[int(v) for v in rng.integers(1, 8, nyc - 1)],
             igridz=[int(v) for v in rng.integers(1, 5, nzc - 1)],
             x0=float(rng.choice([-40.0, -12.3, 0.0])), y0=float(rng.choice([-30.0, -7.7, 0.0])),
             z0=float(rng.choice([-2.0, -1.1, 0.0])))
    nz_f = 1 + sum(p["igridz"])
    if nz_f > 61:
        p["igridz"] = [1] * (nzc - 1)
    return p


def dims(p):
    return 1 + sum(p["igridx"]), 1 + sum(p["igridy"]), 1 + sum(p["igridz"])


def coarse_model(p) -> np.ndarray:
    """(2, nzc, nyc, nxc) float32: P then S velocities"""
    k, j, i = np.meshgrid(np.arange(p["nzc"], dtype=np.float64), np.arange(p["nyc"], dtype=np.float64),
                          np.arange(p["nxc"], dtype=np.float64), indexing="ij")
    vp = 4.5 + 0.35 * k + 0.01 * ((7 * i + 13 * j + 5 * k) % 11) + 0.02 * ((3 * i * j + k) % 7)
    vs = vp / 1.73 + 0.005 * ((i + 2 * j) % 5)
    return np.stack([vp, vs]).astype(np.float32)


def write_reference_inputs(p, d):
    os.makedirs(d, exist_ok=True)
    coarse = coarse_model(p)
    head = VHead(header=b"HEADCORSCARTBMODNOFLc2f case", nx=p["nxc"], ny=p["nyc"], nz=p["nzc"], dz=p["h"])
    with open(os.path.join(d, "coarse.mod"), "wb") as f:
        # a coarse model file: header, the node steps (int32, src/c2f.c:522-524), then P and S
        f.write(head.pack())
        for key in ("igridx", "igridy", "igridz"):
            f.write(np.asarray(p[key], dtype="<i4").tobytes())
        f.write(np.ascontiguousarray(coarse, dtype="<f4").tobytes())
    spec = [f"nxc {p['nxc']}", f"nyc {p['nyc']}", f"nzc {p['nzc']}", f"h {p['h']}",
            f"oldvfil {d}/coarse.mod", f"tgrdfil {d}/grid.txt", f"finevel {d}/fine",
            f"x0 {p['x0']}", f"y0 {p['y0']}", f"z0 {p['z0']}",
            "igridx " + " ".join(map(str, p["igridx"])), "igridy " + " ".join(map(str, p["igridy"])),
            "igridz " + " ".join(map(str, p["igridz"]))]
    with open(os.path.join(d, "spec"), "w") as f:
        f.write("\n".join(spec) + "\n")
    return os.path.join(d, "spec")


def digests(fine: np.ndarray) -> dict:
    """SHA-256 of the three files' data: combined (P then S), P, S"""
    a = np.ascontiguousarray(fine, dtype="<f4").reshape(-1)
    n = a.size // 2
    return {"fine": hashlib.sha256(a.tobytes()).hexdigest(), "pvel": hashlib.sha256(a[:n].tobytes()).hexdigest(),
            "svel": hashlib.sha256(a[n:].tobytes()).hexdigest()}


def golden_path():
    return os.path.join(HERE, "c2f_reference.json")


def load_golden():
    return json.load(open(golden_path()))
