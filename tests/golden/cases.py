"""Seeded small sphfd cases that exercise the solver's branches.

Each case is a small grid with strong velocity contrasts (inversions, a fast inclusion) so that head
waves, restarts from every wall and the stale-(t0,t4) inheritance all occur, plus the par options of
src/sphfd.c:383-413 (NCUBE, growth rates, reverse, headpref, maxoff, parse, integer sources).
Used by make_golden.py to produce reference outputs and by the tests to regenerate inputs.
"""
from __future__ import annotations

import os

import numpy as np

from fdtomoc_gb300.formats import VHead, write_grid, write_par


def random_case(seed: int) -> dict:
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(rng.integers(6, 29)) for _ in range(3))
    h = float(rng.choice([0.5, 1.0, 2.0]))
    dl = float(rng.choice([0.005, 0.01, 0.02]))
    z0 = -float(rng.choice([0.0, 1.0, 2.0]))
    x0, y0 = 120.5, 23.5
    # layered velocity with inversions + perturbation + an optional fast block
    nl = int(rng.integers(1, 5))
    cuts = np.sort(rng.integers(0, nz, size=nl - 1))
    vl = rng.uniform(3.0, 8.0, size=nl)
    layer = np.searchsorted(cuts, np.arange(nz), side="right")
    v = vl[layer][:, None, None] * (1 + 0.1 * rng.uniform(-1, 1, size=(nz, ny, nx)))
    if rng.random() < 0.5:
        a0, a1 = sorted(rng.integers(0, nx, 2)); b0, b1 = sorted(rng.integers(0, ny, 2)); c0, c1 = sorted(rng.integers(0, nz, 2))
        v[c0:c1 + 1, b0:b1 + 1, a0:a1 + 1] *= rng.uniform(1.2, 1.6)
    vel = v.astype(np.float32)
    par = dict(nx=nx, ny=ny, nz=nz, x0=x0, y0=y0, z0=z0, h=h)
    if rng.random() < 0.8:
        par.update(dq=dl, df=dl)
    if rng.random() < 0.25:
        par.update(floatsrc=0, xs=int(rng.integers(0, nx)), ys=int(rng.integers(0, ny)), zs=int(rng.integers(0, nz)))
    else:
        fx = rng.uniform(0, nx - 1); fy = rng.uniform(0, ny - 1)
        fz = rng.uniform(0, nz - 1.0)
        # keep the rounded node inside the grid after the geocentric conversion
        fx = min(max(fx, 0.6), nx - 1.6); fy = min(max(fy, 0.6), ny - 1.6); fz = min(max(fz, 0.6), nz - 1.6)
        par.update(fxs=f"{x0 + fx * dl:.6f}", fys=f"{y0 - fy * dl:.6f}", fzs=f"{z0 + fz * h:.5f}")
        if "dq" not in par:
            par.update(fxs=f"{x0 + fx * h / 6371.0 * 57.29578 / np.cos(np.radians(y0)):.6f}",
                       fys=f"{y0 - fy * h / 6371.0 * 57.29578:.6f}")
    if rng.random() < 0.3:
        par["NCUBE"] = int(rng.integers(1, 4))
    for k in ("iplus", "iminus", "jplus", "jminus", "kplus", "kminus"):
        if rng.random() < 0.1:
            par[k] = int(rng.integers(1, 3))
    par["reverse"] = int(rng.choice([0, 1, 2, 50, 50, 50]))
    if rng.random() < 0.2:
        par["headpref"] = int(rng.choice([-1, 0]))
    if rng.random() < 0.1:
        par["maxoff"] = f"{rng.uniform(2, 10) * h:.3f}"
    if rng.random() < 0.1:
        par["parse"] = 2
    return dict(seed=seed, vel=vel, par=par)


def write_random_case(case: dict, dirname: str) -> str:
    """Write the case's model and par file; returns the par-file path (timefile 'case.ptimes')."""
    os.makedirs(dirname, exist_ok=True)
    p = case["par"]
    velfile = os.path.join(dirname, "vp.mod")
    head = VHead(header=b"HEADFINESPHRVPMDNOFLcase", x0=p["x0"], y0=p["y0"], z0=p["z0"],
                 nx=p["nx"], ny=p["ny"], nz=p["nz"], dz=p["h"])
    write_grid(velfile, head, case["vel"])
    par = dict(case["par"], timefile="case.ptimes", velfile=velfile)
    pf = os.path.join(dirname, "case.par")
    write_par(pf, par)
    return pf
