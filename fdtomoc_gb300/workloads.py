"""Seeded synthetic workloads for the sphfd path.

FDtomoC's own data are not available, so every workload is generated: a layered 1-D P-velocity
profile (5.0 km/s at 0 km rising linearly to 6.8 km/s at 25 km, 6.8 km/s to 30 km, a Moho step to
7.8 km/s below), multiplied by (1 + A*g) where g is Gaussian-smoothed N(0,1) noise normalised to
max|g| = 1.  Grids start at 120.5E, 23.5N (the north edge: sphfd's y index runs south) and 2 km
above sea level (z0 = -2 km, depth positive down), so stations with 0-2 km elevation lie inside.
Velocities above 0 km take the 0 km value.  Par files carry what the reference's make_par_file
writes (reverse=50, NCUBE=2 default) plus dq/df in degrees.

Configurations (sizes are the benchmark's):
  1  61x61x31, 0.01 deg x 0.01 deg x 1 km, 3 % / 5 km, one station (seed 1)
  2  201x201x81, 0.005 deg x 0.005 deg x 0.5 km, 5 % / 10 km, 64 stations (seed 2)
  3  401x401x161 model (seed 4); 500 windows 41..301 x 41..301 x 41..121 (seed 3)
  4  config-3 model as P, S = P/1.73 * (1 + 2 % independent field); 800 stations
  5  401x401x161 with a 30-degree dipping +8 % slab, 15 km thick (seed 5); 1200 stations
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

from .formats import VHead, write_grid, write_par

KM_PER_DEG = 111.19


@dataclasses.dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dlon: float  # degrees
    dlat: float  # degrees
    h: float  # km
    x0: float = 120.5  # west edge, degrees east
    y0: float = 23.5  # north edge, degrees north
    z0: float = -2.0  # depth of the top layer, km (negative = above sea level)

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)


def vp_1d(depth_km: np.ndarray) -> np.ndarray:
    d = np.maximum(depth_km, 0.0)
    return np.where(d < 25.0, 5.0 + 1.8 * d / 25.0, np.where(d < 30.0, 6.8, 7.8))


def smooth_noise(shape, spacing_km, corr_km: float, seed: int) -> np.ndarray:
    """Gaussian-smoothed N(0,1) field (sigma = corr_km), normalised to max |g| = 1."""
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(shape)
    ks = [np.fft.fftfreq(n, d) for n, d in zip(shape, spacing_km)]
    kz, ky, kx = np.meshgrid(*ks, indexing="ij", sparse=True)
    filt = np.exp(-2.0 * (math.pi * corr_km) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))
    g = np.real(np.fft.ifftn(np.fft.fftn(r) * filt))
    return g / np.abs(g).max()


def layered_model(grid: Grid, pert: float, corr_km: float, seed: int) -> np.ndarray:
    depth = grid.z0 + grid.h * np.arange(grid.nz)
    v = vp_1d(depth)[:, None, None]
    dx = grid.dlon * KM_PER_DEG * math.cos(math.radians(grid.y0))
    dy = grid.dlat * KM_PER_DEG
    g = smooth_noise(grid.shape, (grid.h, dy, dx), corr_km, seed)
    return (v * (1.0 + pert * g)).astype(np.float32)


def add_slab(grid: Grid, vel: np.ndarray, amp=0.08, thick_km=15.0, dip_deg=30.0) -> np.ndarray:
    """Config 5: a high-velocity layer dipping east at dip_deg, thick_km thick."""
    x_km = np.arange(grid.nx) * grid.dlon * KM_PER_DEG * math.cos(math.radians(grid.y0))
    depth = grid.z0 + grid.h * np.arange(grid.nz)
    top = 5.0 + math.tan(math.radians(dip_deg)) * (x_km - x_km.mean() / 2)
    inside = (depth[:, None] >= top[None, :]) & (depth[:, None] <= top[None, :] + thick_km / math.cos(math.radians(dip_deg)))
    out = vel.copy()
    out *= np.where(inside[:, None, :], 1.0 + amp, 1.0).astype(np.float32)
    return out


def head_for(grid: Grid, text: bytes = b"HEADFINESPHRVPMDNOFLsynthetic") -> VHead:
    return VHead(header=text, x0=grid.x0, y0=grid.y0, z0=grid.z0, clat=grid.y0, clon=grid.x0,
                 cz=grid.z0, dx=grid.dlon, dy=grid.dlat, dz=grid.h, nx=grid.nx, ny=grid.ny, nz=grid.nz)


def stations(grid: Grid, n: int, seed: int, margin: int = 2):
    """n stations uniform on the surface (in node units away from the edges), elevation 0-2 km."""
    rng = np.random.default_rng(seed + 1000)
    out = []
    for i in range(n):
        fx = rng.uniform(margin, grid.nx - 1 - margin)
        fy = rng.uniform(margin, grid.ny - 1 - margin)
        elev = rng.uniform(0.0, 2.0)
        out.append(dict(name=f"S{i:04d}", lon=grid.x0 + fx * grid.dlon, lat=grid.y0 - fy * grid.dlat,
                        elev=elev))
    return out


def par_for(grid: Grid, st: dict, velfile: str, timefile: str, **extra) -> dict:
    p = dict(fxs=f"{st['lon']:.6f}", fys=f"{st['lat']:.6f}", fzs=f"{-st['elev']:.4f}", nx=grid.nx,
             ny=grid.ny, nz=grid.nz, x0=grid.x0, y0=grid.y0, z0=grid.z0, h=grid.h, dq=grid.dlat,
             df=grid.dlon, timefile=timefile, velfile=velfile, reverse=50)
    p.update(extra)
    return p


def config(n: int):
    """(grid, velocity, station list) for configs 1, 2 and 5; config 3/4 use config3_windows."""
    if n == 1:
        g = Grid(61, 61, 31, 0.01, 0.01, 1.0)
        return g, layered_model(g, 0.03, 5.0, 1), stations(g, 1, 1)
    if n == 2:
        g = Grid(201, 201, 81, 0.005, 0.005, 0.5)
        return g, layered_model(g, 0.05, 10.0, 2), stations(g, 64, 2)
    if n == 3:
        g = Grid(401, 401, 161, 0.005, 0.005, 0.5)
        return g, layered_model(g, 0.05, 10.0, 4), []
    if n == 5:
        g = Grid(401, 401, 161, 0.005, 0.005, 0.5)
        return g, add_slab(g, layered_model(g, 0.05, 10.0, 5)), stations(g, 1200, 5)
    raise ValueError(n)


def window_par(grid: Grid, w: dict, velfile: str, timefile: str) -> dict:
    """Par values of a config-3 window: its own grid, its north-west corner at (ox, oy) of the model,
    z from the model's top, and a surface station at (fx, fy) of the window."""
    x0 = grid.x0 + w["ox"] * grid.dlon
    y0 = grid.y0 - w["oy"] * grid.dlat
    st = dict(lon=x0 + w["fx"] * grid.dlon, lat=y0 - w["fy"] * grid.dlat, elev=w["elev"])
    g = Grid(w["nx"], w["ny"], w["nz"], grid.dlon, grid.dlat, grid.h, x0=x0, y0=y0, z0=grid.z0)
    return par_for(g, st, velfile, timefile)


def config3_windows(n_windows: int = 500, seed: int = 3):
    """Window sizes and offsets into the 401x401x161 model: uniform in [41,301]x[41,301]x[41,121]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_windows):
        wx, wy, wz = int(rng.integers(41, 302)), int(rng.integers(41, 302)), int(rng.integers(41, 122))
        ox, oy = int(rng.integers(0, 401 - wx + 1)), int(rng.integers(0, 401 - wy + 1))
        sx, sy = float(rng.uniform(2, wx - 3)), float(rng.uniform(2, wy - 3))
        out.append(dict(name=f"W{i:04d}", nx=wx, ny=wy, nz=wz, ox=ox, oy=oy, fx=sx, fy=sy,
                        elev=float(rng.uniform(0, 2))))
    return out


def write_case(dirname: str, grid: Grid, vel: np.ndarray, sts: list, **extra) -> str:
    """Write model, par files, parlist and spec for the reference's driver; returns the spec path."""
    os.makedirs(os.path.join(dirname, "out"), exist_ok=True)
    velfile = os.path.join(dirname, "vp.mod")
    write_grid(velfile, head_for(grid), vel)
    lines = []
    for st in sts:
        pf = os.path.join(dirname, st["name"] + ".par")
        write_par(pf, par_for(grid, st, velfile, st["name"] + ".ptimes", **extra))
        lines.append("par=" + pf)
    with open(os.path.join(dirname, "parlist"), "w") as f:
        f.write("\n".join(lines) + "\n")
    spec = os.path.join(dirname, "spec")
    with open(spec, "w") as f:
        f.write(f"parlist {os.path.join(dirname, 'parlist')}\ntimedir {os.path.join(dirname, 'out')}\n")
    return spec
