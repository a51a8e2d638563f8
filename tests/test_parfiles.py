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
