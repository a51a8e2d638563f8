"""File formats of the path: getpar par files and the 232-byte vhead grid files."""
import numpy as np

from fdtomoc_gb300.formats import VHEAD_SIZE, VHead, read_grid, read_par, write_grid


def test_par_last_definition_wins_comments_quotes_and_recursion(tmp_path):
    inner = tmp_path / "inner.par"
    inner.write_text("h=2.0 nz=31\n# comment\nvelfile='/a b/c'\n")
    outer = tmp_path / "outer.par"
    outer.write_text(f"nx=41 h=1.0\npar={inner}\nnz=33  # trailing\n")
    p = read_par(outer)
    assert p["nx"] == "41" and p["h"] == "2.0" and p["nz"] == "33" and p["velfile"] == "/a b/c"


def test_vhead_roundtrip(tmp_path):
    assert VHEAD_SIZE == 232
    h = VHead(header=b"HEADFINESPHRVPMDNOFLx", x0=120.5, y0=23.5, z0=-2.0, dx=0.01, dy=0.01, dz=1.0, nx=3, ny=4,
              nz=5, fxs=2.1, fys=0.9, fzs=6370.0)
    v = np.arange(60, dtype=np.float32).reshape(5, 4, 3)
    write_grid(tmp_path / "g.mod", h, v)
    h2, v2 = read_grid(tmp_path / "g.mod")
    assert h2.nx == 3 and h2.nz == 5 and h2.fzs == 6370.0 and h2.header.rstrip(b"\0") == h.header
    assert np.array_equal(v, v2)
