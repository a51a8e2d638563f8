"""Par files of an inversion iteration, in the dialect the reference's make_par_file writes.

The reference turns a station list into one P par file (<sta>.par) and one S par file (<sta>.spar)
per station, plus a shell list that runs sphfd on each (src/make_par_file.c:68-105).  sphfd then
reads them through a parlist (src/sphfd.c:214-243).  This module writes the same files, byte for
byte, and the parlist and spec the batch driver (fdgpu_sphfd_parlist, bin/sphfd_gpu) reads, so the
P and S solves of all stations run as one process with each model read once.

What the reference does, kept here:
  - the spec keys x0, y0, z0, h are read with get_vars and sscanf "%f" (float); "sph" is read with
    "%f" into an int, so any value whose float bits are not zero selects the spherical station
    format;
  - station lines are "fys fxs fzs sta" (plain) or "sty stx zs sta fys fxs" (spherical: zs is the
    elevation in metres); reading stops at the first empty line or at the end of the file;
  - fzs is always written as zs / -1000 (so -0.000 for the plain format, whose zs stays 0);
  - the grid size is fixed in the reference (301 x 301 x 61) and the velocity files are VP.mod
    and VS.mod; both are parameters here, with the reference's values as defaults;
  - values go through C floats and printf's formats: "fxs=%.5f", "fys=%.5f", "fzs=%.3f",
    "nx=%f " (with its trailing space), "x0=%.1f " ..., "reverse=50".
"""
from __future__ import annotations

import os

import numpy as np


def _f32(text: str) -> float:
    """sscanf "%f": the decimal text rounded to a float (returned as the double holding it)."""
    return float(np.float32(float(text)))


def _get_var(lines, name):
    """get_vars (lib/common/parseprogs.c:9-79): the value after the first line whose first word is
    `name`, or None."""
    for ln in lines:
        parts = ln.split(None, 1)
        if parts and parts[0] == name:
            return parts[1].strip() if len(parts) > 1 else ""
    return None


def read_spec_grid(spec_path: str):
    """The spec keys make_par_file reads: (x0, y0, z0, h, sph) as it reads them."""
    with open(spec_path) as f:
        lines = f.read().splitlines()
    vals = []
    for key in ("x0", "y0", "z0", "h"):
        v = _get_var(lines, key)
        vals.append(_f32(v.split()[0]) if v else 0.0)
    sv = _get_var(lines, "sph")
    sph = bool(sv) and np.float32(float(sv.split()[0])).view(np.int32) != 0
    return vals[0], vals[1], vals[2], vals[3], sph


def read_station_lines(station_path: str, sph: bool):
    """Station entries (name, fxs, fys, fzs) as the reference parses them (fgets of 100 bytes)."""
    out = []
    with open(station_path, "rb") as f:
        data = f.read().decode("latin-1")
    pos = 0
    while pos < len(data):
        # fgets(str, 100, fp): up to 99 bytes or through the newline
        end = data.find("\n", pos)
        stop = len(data) if end < 0 else end + 1
        if stop - pos > 99:
            stop = pos + 99
        line = data[pos:stop]
        pos = stop
        if line.startswith("\n"):
            break
        tok = line.split()
        zs = 0
        if sph:
            sty, stx, zs, sta, fys, fxs = (_f32(tok[0]), _f32(tok[1]), int(tok[2]), tok[3], _f32(tok[4]),
                                           _f32(tok[5]))
        else:
            fys, fxs, sta = _f32(tok[0]), _f32(tok[1]), tok[3]
        fzs = float(np.float32(zs / -1000.0))
        out.append((sta, fxs, fys, fzs))
    return out


def par_text(fxs, fys, fzs, nx, ny, nz, x0, y0, z0, h, timefile, velfile) -> str:
    """One par file as the reference prints it."""
    return (f"fxs={fxs:.5f}\nfys={fys:.5f}\nfzs={fzs:.3f}\n"
            f"nx={float(np.float32(nx)):f} \nny={float(np.float32(ny)):f} \nnz={float(np.float32(nz)):f} \n"
            f"x0={x0:.1f} \ny0={y0:.1f} \nz0={z0:.1f} \nh={h:.1f} \n"
            f"timefile={timefile}\nvelfile={velfile}\nreverse=50\n")


def make_par_files(spec_path: str, station_path: str, outdir: str = ".", nx: int = 301, ny: int = 301,
                   nz: int = 61, p_model: str = "VP.mod", s_model: str = "VS.mod"):
    """Write <sta>.par and <sta>.spar for every station, and runsphfd01.sh, into outdir (the
    reference writes them into its working directory).  Returns the par-file paths in the order
    the reference lists them (P then S for each station)."""
    x0, y0, z0, h, sph = read_spec_grid(spec_path)
    os.makedirs(outdir, exist_ok=True)
    paths, script = [], []
    for sta, fxs, fys, fzs in read_station_lines(station_path, sph):
        for j, (ext, tf, vf) in enumerate(((".par", ".ptimes", p_model), (".spar", ".stimes", s_model))):
            script.append(f"./sphfd par=../parfiles_P/{sta}{ext}\n")
            p = os.path.join(outdir, sta + ext)
            with open(p, "w") as f:
                f.write(par_text(fxs, fys, fzs, nx, ny, nz, x0, y0, z0, h, sta + tf, vf))
            paths.append(p)
    with open(os.path.join(outdir, "runsphfd01.sh"), "w") as f:
        f.write("".join(script))
    return paths


def write_parlist(par_paths, parlist_path: str, timedir: str, spec_path: str | None = None) -> str:
    """The parlist ("par=<file>" per line) and, if asked, the spec (parlist, timedir) that sphfd's
    main reads (src/sphfd.c:214-243); returns the spec path or the parlist path."""
    with open(parlist_path, "w") as f:
        f.write("".join(f"par={p}\n" for p in par_paths))
    if spec_path:
        with open(spec_path, "w") as f:
            f.write(f"parlist {parlist_path}\ntimedir {timedir}\n")
        return spec_path
    return parlist_path
