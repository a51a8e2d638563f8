"""Input errors of the drop-in entry points, found on the host before any device work, so they need
no GPU: where the reference asserts, reads short or exits (src/sphfd.c:560-665, getpar's
exit(GETPAR_ERROR)), fdgpu_sphfd_parlist returns a status per par file and writes no time file."""
import os

import numpy as np

from cases import random_case, write_random_case

ERR = {"EINVAL": -1, "EIO": -4, "EPAR": -5, "ESOURCE": -6}


def _case(tmp_path, seed=3):
    c = random_case(seed)
    return c, write_random_case(c, str(tmp_path / "case"))


def test_truncated_velocity_file(gpu_lib, tmp_path):
    """The reference reads what is there and solves on garbage; the drop-in reports EIO."""
    c, pf = _case(tmp_path)
    vf = tmp_path / "case" / "vp.mod"
    data = vf.read_bytes()
    vf.write_bytes(data[:len(data) - 4])          # one velocity short
    out = tmp_path / "out"
    os.makedirs(out)
    assert gpu_lib.sphfd_parlist(["par=" + pf], str(out)) == [ERR["EIO"]]
    assert os.listdir(out) == []


def test_headerless_file_too_short_for_its_grid(gpu_lib, tmp_path):
    """A file without the "HEAD" text is read from its first byte (src/sphfd.c:622-662); with fewer
    than nx*ny*nz values it is the same EIO."""
    c, pf = _case(tmp_path)
    vf = tmp_path / "case" / "vp.mod"
    vf.write_bytes(np.ascontiguousarray(c["vel"], dtype="<f4").tobytes()[:-8])
    out = tmp_path / "out"
    os.makedirs(out)
    assert gpu_lib.sphfd_parlist(["par=" + pf], str(out)) == [ERR["EIO"]]


def test_missing_velocity_file_and_bad_par_files(gpu_lib, tmp_path):
    """Each par file gets its own status: a missing velocity file (EIO), a par file without a
    required key (EPAR: the reference's mstpar exits), a source outside the grid (ESOURCE: the
    reference asserts, src/sphfd.c:533-538), a missing par file (EIO)."""
    from fdtomoc_gb300.formats import read_par, write_par
    c, pf = _case(tmp_path)
    par = read_par(pf)
    bad = {}
    q = dict(par, velfile=str(tmp_path / "nowhere.mod"))
    bad["novel"] = q
    q = dict(par)
    q.pop("nx")
    bad["nokey"] = q
    q = {k: v for k, v in par.items() if k not in ("fxs", "fys", "fzs", "xs", "ys", "zs", "floatsrc")}
    q.update(floatsrc=0, xs=int(par["nx"]) + 3, ys=0, zs=0)
    bad["outside"] = q
    entries = []
    for name, q in bad.items():
        p = tmp_path / f"{name}.par"
        write_par(p, q)
        entries.append("par=" + str(p))
    entries.append("par=" + str(tmp_path / "absent.par"))
    out = tmp_path / "out"
    os.makedirs(out)
    st = gpu_lib.sphfd_parlist(entries, str(out))
    assert st == [ERR["EIO"], ERR["EPAR"], ERR["ESOURCE"], ERR["EIO"]], st
    assert os.listdir(out) == []
