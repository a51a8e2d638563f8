"""GPU parity: the CUDA solver through the C ABI against the CPU oracle, bit for bit."""
import os

import numpy as np
import pytest

from cases import random_case, write_random_case
from oracle_util import run_oracle

pytestmark = pytest.mark.gpu


def _cmp_files(a, b):
    A = open(a, "rb").read()
    B = open(b, "rb").read()
    assert len(A) == len(B)
    x = np.frombuffer(A[232:], "<f4")
    y = np.frombuffer(B[232:], "<f4")
    nd = int((x != y).sum())
    assert A[:232] == B[:232], "header differs"
    assert nd == 0, f"{nd} nodes differ, max |dt| = {np.abs(x.astype(np.float64) - y).max()}"


@pytest.mark.parametrize("seed", list(range(0, 40)))
def test_random_case_dropin(gpu_lib, tmp_path, seed):
    """Drop-in sphfd (par file in, time file out) equals the oracle's time file byte for byte."""
    c = random_case(seed)
    pf = write_random_case(c, str(tmp_path))
    run_oracle(pf, str(tmp_path / "orc"))
    os.makedirs(tmp_path / "gpu", exist_ok=True)
    st = gpu_lib.sphfd_parlist(["par=" + pf], str(tmp_path / "gpu"))
    assert st == [0]
    _cmp_files(tmp_path / "orc" / "case.ptimes", tmp_path / "gpu" / "case.ptimes")


def test_config1_station(gpu_lib, tmp_path):
    from fdtomoc_gb300 import workloads as W
    g, v, sts = W.config(1)
    spec = W.write_case(str(tmp_path), g, v, sts)
    pf = str(tmp_path / "S0000.par")
    run_oracle(pf, str(tmp_path / "orc"))
    st = gpu_lib.sphfd_parlist(["par=" + pf], str(tmp_path / "out"))
    assert st == [0]
    _cmp_files(tmp_path / "orc" / "S0000.ptimes", tmp_path / "out" / "S0000.ptimes")

