"""Known answer: in a homogeneous model the travel time is the straight-line distance times the
slowness.  The reference computes exactly that inside the source box (src/sphfd.c:727-749) and
approximates it with its finite-difference stencils outside.  On a 41x41x21 grid at 6 km/s (a surface
station, 0.01 deg x 0.01 deg x 1 km) the oracle's box times equal the straight-line times to float
rounding, and every other node is within 3 % (measured: at most 2.5 %, 99 % of nodes within 0.85 %);
the GPU's field equals the oracle's bit for bit."""
import math
import os

import numpy as np
import pytest

from oracle_util import run_oracle


def _case(tmp_path):
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_grid, write_par
    g = W.Grid(41, 41, 21, 0.01, 0.01, 1.0, x0=120.5, y0=23.5, z0=-1.0)
    v = np.full(g.shape, 6.0, np.float32)
    vf = str(tmp_path / "vp.mod")
    write_grid(vf, W.head_for(g), v)
    st = dict(name="K", lon=120.5 + 20.3 * 0.01, lat=23.5 - 17.6 * 0.01, elev=0.4)
    pf = str(tmp_path / "k.par")
    write_par(pf, W.par_for(g, st, vf, "k.ptimes"))
    return g, v, pf


def _straight_line(s, g, speed):
    """|source - node| / speed with the reference's spherical-to-Cartesian conversion."""
    fx, fy, fz = s.src_geo
    x1, y1, z1 = fz * math.cos(fy), fz * math.sin(fy) * math.cos(fx), fz * math.sin(fy) * math.sin(fx)
    kk, jj, ii = np.meshgrid(np.arange(g.nz), np.arange(g.ny), np.arange(g.nx), indexing="ij")
    r, q, f = s.z0r - s.h * kk, s.y0 + s.dq * jj, s.x0 + s.df * ii
    x2, y2, z2 = r * np.cos(q), r * np.sin(q) * np.cos(f), r * np.sin(q) * np.sin(f)
    box = (abs(kk - s.zs) <= s.ncube) & (abs(jj - s.ys) <= s.ncube) & (abs(ii - s.xs) <= s.ncube)
    return np.sqrt((x1 - x2) ** 2 + (y1 - y2) ** 2 + (z1 - z2) ** 2) / speed, box


def test_homogeneous_model_oracle(gpu_lib, tmp_path):
    g, v, pf = _case(tmp_path)
    run_oracle(pf, str(tmp_path / "o"))
    t = np.fromfile(tmp_path / "o" / "k.ptimes", dtype="<f4", offset=232).reshape(g.shape).astype(np.float64)
    s, _, _ = gpu_lib.station_from_par("par=" + pf)
    ta, box = _straight_line(s, g, 6.0)
    assert (s.xs, s.ys, s.zs, s.ncube) == (20, 18, 1, 2)
    assert box.sum() == 4 * 5 * 5            # the 5x5x5 source box, its top layer above the grid
    assert np.all(np.abs(t - ta)[box] <= 1.2e-7 * np.maximum(ta[box], 1e-3))
    rel = np.abs(t - ta)[~box] / ta[~box]
    assert rel.max() < 0.03 and np.percentile(rel, 99) < 0.01


@pytest.mark.gpu
def test_homogeneous_model_gpu(gpu_lib, tmp_path):
    g, v, pf = _case(tmp_path)
    run_oracle(pf, str(tmp_path / "o"))
    os.makedirs(tmp_path / "g")
    assert gpu_lib.sphfd_parlist(["par=" + pf], str(tmp_path / "g")) == [0]
    assert (tmp_path / "g" / "k.ptimes").read_bytes() == (tmp_path / "o" / "k.ptimes").read_bytes()
