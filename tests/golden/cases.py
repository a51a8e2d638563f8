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


START_KINDS = ("oldt", "walls", "box")


def start_case(seed: int, kind: str) -> dict:
    """A random case turned into a solve from a supplied start: "oldt" (srctype 3: a whole starting
    field, times on the source wall's layer and 1e10 elsewhere), "walls" (srctype 2: a wall file of six
    records, the valid ones starting above -1e-20) or "box" (srctype 1 with fill=1: the source box's
    times from a box file).  The supplied times are straight-line times from a seeded node, made with
    +, *, / and sqrt only, so they are the same on every machine.  Returns the case with its extra
    files under "files" (name -> bytes)."""
    c = random_case(seed)
    p = dict(c["par"])
    nx, ny, nz = p["nx"], p["ny"], p["nz"]
    rng = np.random.default_rng(seed + 7000)
    i0, j0, k0 = (int(rng.integers(0, n)) for n in (nx, ny, nz))
    kk, jj, ii = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                             np.arange(nx, dtype=np.float64), indexing="ij")
    base = (np.sqrt(((ii - i0) * 1.1) ** 2 + ((jj - j0) * 1.05) ** 2 + ((kk - k0) * p["h"]) ** 2) / 6.0 + 0.25
            ).astype(np.float32)
    files = {}
    if kind in ("oldt", "walls"):
        for key in ("fxs", "fys", "fzs", "xs", "ys", "zs", "floatsrc", "NCUBE"):
            p.pop(key, None)
        srcwall = int(rng.integers(1, 7))
        p["srctype"] = 3 if kind == "oldt" else 2
        p["srcwall"] = srcwall
        # the layer of srcwall (src/sphfd.c:877-926): 1 x=0, 2 x=nx-1, 3 y=0, 4 y=ny-1, 5 z=0, 6 z=nz-1
        sel = [np.s_[:, :, 0], np.s_[:, :, nx - 1], np.s_[:, 0, :], np.s_[:, ny - 1, :], np.s_[0, :, :],
               np.s_[nz - 1, :, :]]
        if kind == "oldt":
            t = np.full((nz, ny, nx), 1.0e10, np.float32)
            t[sel[srcwall - 1]] = base[sel[srcwall - 1]]
            files["oldt.bin"] = t.tobytes()
            p["oldtfile"] = "@oldt.bin"
        else:
            nwall = ny * nz if (nx <= ny and nx <= nz) else (nx * nz if (ny <= nx and ny <= nz) else nx * ny)
            recs = []
            extra = int(rng.integers(0, 6))
            for w in range(6):
                rec = np.full(nwall, -1.0, np.float32)
                if w == srcwall - 1 or w == extra:
                    vals = base[sel[w]].reshape(-1)   # wall order: (k, j) for x walls, (k, i) for y, (j, i) for z
                    rec[:vals.size] = vals
                recs.append(rec)
            files["walls.bin"] = np.concatenate(recs).tobytes()
            p["wallfile"] = "@walls.bin"
    elif kind == "box":
        nc = int(p.get("NCUBE", 2))
        w = 2 * nc + 1
        box = (0.05 + 0.01 * np.arange(w ** 3, dtype=np.float64) % 0.7).astype(np.float32)
        head = VHead(header=b"HEADFINESPHRPTIMbox", nx=w, ny=w, nz=w, dz=p["h"])
        files["box.bin"] = head.pack() + box.tobytes()
        p["fill"] = 1
        p["boxfile"] = "@box.bin"
    else:
        raise ValueError(kind)
    c = dict(c, par=p, files=files, kind=kind)
    return c


def write_start_case(case: dict, dirname: str) -> str:
    """Write a start_case: its files, then model and par file with '@name' values pointing at them."""
    os.makedirs(dirname, exist_ok=True)
    par = dict(case["par"])
    for name, data in case["files"].items():
        path = os.path.join(dirname, name)
        with open(path, "wb") as f:
            f.write(data)
        for k, v in list(par.items()):
            if v == "@" + name:
                par[k] = path
    return write_random_case(dict(case, par=par), dirname)


START_SEEDS = (3, 8, 14, 27, 40, 61)


# ---- byte-swapped models and times (par key swab, src/sphfd.c:667-686 and :5774-5795) ----------

SWAB_SEEDS = (3, 8, 21)


def write_swab_case(case: dict, dirname: str, swab: int) -> str:
    """A random case with swab = 1, 2 or 3.  For swab 1 and 3 the model is written the way the
    reference expects to swap it back: every header number (not the text) and every velocity
    byte-reversed."""
    pf = write_random_case(case, dirname)
    if swab in (1, 3):
        p = case["par"]
        head = VHead(header=b"HEADFINESPHRVPMDNOFLcase", x0=p["x0"], y0=p["y0"], z0=p["z0"],
                     nx=p["nx"], ny=p["ny"], nz=p["nz"], dz=p["h"])
        with open(os.path.join(dirname, "vp.mod"), "wb") as f:
            f.write(head.pack(">"))
            f.write(np.ascontiguousarray(case["vel"], dtype=">f4").tobytes())
    with open(pf, "a") as f:
        f.write(f"swab={swab}\n")
    return pf


# ---- one inversion iteration's P and S par files (make_par_file's dialect) ---------------------

def ps_station_case(dirname: str, n_sta: int = 4, seed: int = 5):
    """P and S solves of n_sta surface stations on a shared 41x37x23 grid, written as the reference's
    make_par_file writes them (fdtomoc_gb300.parfiles, grid size given), with VP.mod and VS.mod in
    dirname.  Returns (par paths in parlist order, VP model, VS model)."""
    from fdtomoc_gb300 import parfiles
    from fdtomoc_gb300.workloads import Grid, head_for, layered_model
    g = Grid(41, 37, 23, 0.01, 0.01, 1.0, x0=120.5, y0=23.5, z0=-2.0)
    vp = layered_model(g, 0.05, 5.0, seed)
    rng = np.random.default_rng(seed + 100)
    vs = (vp / np.float32(1.73) * (1 + 0.02 * rng.uniform(-1, 1, size=vp.shape))).astype(np.float32)
    os.makedirs(dirname, exist_ok=True)
    write_grid(os.path.join(dirname, "VP.mod"), head_for(g), vp)
    write_grid(os.path.join(dirname, "VS.mod"), head_for(g, b"HEADFINESPHRVSMDNOFLsynthetic"), vs)
    # spec: the grid origin and spacing that make_par_file copies into every par file
    spec = os.path.join(dirname, "mpf.spec")
    with open(spec, "w") as f:
        f.write(f"x0 {g.x0}\ny0 {g.y0}\nz0 {g.z0}\nh {g.h}\nsph 1\ntimedir ttimes\n")
    sta = os.path.join(dirname, "stations.txt")
    with open(sta, "w") as f:
        for k in range(n_sta):
            fx, fy = rng.uniform(3, g.nx - 4), rng.uniform(3, g.ny - 4)
            elev = int(rng.integers(0, 1900))
            lat, lon = g.y0 - fy * g.dlat, g.x0 + fx * g.dlon
            f.write(f"{lat:.3f} {lon:.3f} {elev} ST{k:02d} {lat:.5f} {lon:.5f}\n")
    # make_par_file names the models without a directory; these par files are read from dirname,
    # so the velfile lines are given with it
    paths = parfiles.make_par_files(spec, sta, dirname, nx=g.nx, ny=g.ny, nz=g.nz,
                                    p_model=os.path.join(dirname, "VP.mod"),
                                    s_model=os.path.join(dirname, "VS.mod"))
    # the grid's angular spacing, which make_par_file leaves out, appended to each par file
    for p in paths:
        with open(p, "a") as f:
            f.write(f"dq={g.dlat}\ndf={g.dlon}\n")
    return paths, vp, vs


# ---- the reference make_par_file's inputs --------------------------------------------------------

PARFILE_CASES = {
    "plain": {
        "spec": "x0 120.9\ny0 23.8\nz0 -4.0\nh 2.0\nsph 0\ntimedir ./ttimes\n",
        "stations": "23.12651 121.37915 0.198 M001\n22.98765 120.55555 1.234 TW02\n"
                    "23.50000 121.00000 0.000 ABCDE\n\nIGNORED 1 2 3\n",
    },
    "spherical": {
        "spec": "x0 120.25\ny0 23.75\nz0 -3.5\nh 0.25\nsph 1\ntimedir ./ttimes\n",
        "stations": "23.126 121.379 198 M001 23.12651 121.37915\n22.988 120.556 1234 TW02 22.98765 120.55555\n"
                    "23.5 121.0 -15 LOW 23.50000 121.00000\n",
    },
}
