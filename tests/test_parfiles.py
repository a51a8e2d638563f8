"""The par-file writer (fdtomoc_gb300.parfiles) against the reference's make_par_file: the files it
writes for two station lists (plain and spherical station formats) equal, byte for byte, the files
the reference binary wrote (tests/golden/parfiles_reference.json, made by make_parfile_golden.py)."""
import json
import os

import pytest

from cases import PARFILE_CASES

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("name", sorted(PARFILE_CASES))
def test_par_files_equal_the_reference(tmp_path, name):
    from fdtomoc_gb300 import parfiles
    gold = json.load(open(os.path.join(HERE, "golden", "parfiles_reference.json")))[name]
    case = PARFILE_CASES[name]
    spec, sta = tmp_path / "in.spec", tmp_path / "in.sta"
    spec.write_text(case["spec"])
    sta.write_text(case["stations"])
    out = tmp_path / "work"
    paths = parfiles.make_par_files(str(spec), str(sta), str(out))
    got = {f: (out / f).read_text() for f in sorted(os.listdir(out))}
    assert sorted(got) == sorted(gold)
    for f in gold:
        assert got[f] == gold[f], f
    # P then S per station, in the station list's order
    assert [os.path.basename(p) for p in paths] == [os.path.basename(ln.split("par=")[1])
                                                    for ln in gold["runsphfd01.sh"].splitlines()]


def test_parlist_and_spec(tmp_path):
    from fdtomoc_gb300 import parfiles
    spec = parfiles.write_parlist(["/a/x.par", "/a/x.spar"], str(tmp_path / "pl"), "/t", str(tmp_path / "spec"))
    assert (tmp_path / "pl").read_text() == "par=/a/x.par\npar=/a/x.spar\n"
    assert open(spec).read() == f"parlist {tmp_path / 'pl'}\ntimedir /t\n"


def test_driver_reads_spec_and_parlist(tmp_path):
    """sphfd's main reads "parlist" and "timedir" from its spec, then every "par=" line (at most
    MAXNUMPAR = 2000, src/sphfd.c:143); the rank-aware driver does the same."""
    import pytest
    from fdtomoc_gb300 import driver
    (tmp_path / "pl").write_text("par=/a/x.par\n\npar=/a/y.spar\n")
    (tmp_path / "spec").write_text(f"timedir /t/out\nother 1\nparlist {tmp_path / 'pl'}\n")
    assert driver.read_spec(str(tmp_path / "spec")) == (str(tmp_path / "pl"), "/t/out")
    assert driver.read_parlist(str(tmp_path / "pl")) == ["par=/a/x.par", "par=/a/y.spar"]
    (tmp_path / "big").write_text("".join(f"par=/a/{k}.par\n" for k in range(driver.MAXNUMPAR + 1)))
    with pytest.raises(ValueError):
        driver.read_parlist(str(tmp_path / "big"))
    (tmp_path / "bad").write_text("parlist x\n")
    with pytest.raises(ValueError):
        driver.read_spec(str(tmp_path / "bad"))
    # without torch.distributed the driver is the plain parlist call
    seen = []
    st = driver.run_entries(["par=/a/x.par"], str(tmp_path / "o"), lambda e, d: seen.append((e, d)) or [0])
    assert st == [0] and seen == [(["par=/a/x.par"], str(tmp_path / "o"))]
