"""The GPU drop-in against the reference's own outputs: the M001 golden file and the reference
binary's time files for the seeded cases (SHA-256 recorded by tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

from cases import random_case, write_random_case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF = json.load(open(os.path.join(GOLDEN, "reference_outputs.json")))


def test_m001_golden(gpu_lib, tmp_path):
    from fdtomoc_gb300.formats import write_par
    z = np.load(os.path.join(GOLDEN, "m001.npz"))
    vf = tmp_path / "m001.vel"
    vf.write_bytes(z["velocity_file"].tobytes())
    pf = tmp_path / "M001.par"
    write_par(pf, dict(REF["m001"]["par"], velfile=str(vf)))
    os.makedirs(tmp_path / "out")
    assert gpu_lib.sphfd_parlist([f"par={pf}"], str(tmp_path / "out")) == [0]
    assert (tmp_path / "out" / "M001.ptimes").read_bytes() == z["expected"].tobytes()


@pytest.mark.parametrize("seed", sorted(int(s) for s in REF["cases"]))
def test_seeded_cases_reference_hash(gpu_lib, tmp_path, seed):
    pf = write_random_case(random_case(seed), str(tmp_path))
    os.makedirs(tmp_path / "out")
    assert gpu_lib.sphfd_parlist([f"par={pf}"], str(tmp_path / "out")) == [0]
    got = hashlib.sha256((tmp_path / "out" / "case.ptimes").read_bytes()).hexdigest()
    assert got == REF["cases"][str(seed)]["sha256"]


@pytest.mark.parametrize("key", sorted(REF["start_cases"]))
def test_start_cases_reference_hash(gpu_lib, tmp_path, key):
    """srctype 3 (starting field), srctype 2 (wall file) and fill=1 (box file) through the drop-in,
    against the reference binary's time files."""
    from cases import start_case, write_start_case
    seed, kind = key.split("_")
    pf = write_start_case(start_case(int(seed), kind), str(tmp_path))
    os.makedirs(tmp_path / "out")
    assert gpu_lib.sphfd_parlist([f"par={pf}"], str(tmp_path / "out")) == [0]
    b = (tmp_path / "out" / "case.ptimes").read_bytes()
    want = REF["start_cases"][key]["sha256" if kind == "box" else "sha256_source_zeroed"]
    assert hashlib.sha256(b).hexdigest() == want   # srctype 2/3: header source point written as zeros
