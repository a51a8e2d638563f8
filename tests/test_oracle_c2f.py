"""The c2f oracle against the reference's own c2f: for the seeded coarse models of
tests/golden/c2f_cases.py the oracle's fine model has the SHA-256 the reference's three output files'
data had (tests/golden/c2f_reference.json, made by make_c2f_golden.py)."""
import pytest

import c2f_cases as CC
from oracle_util import oracle_c2f

GOLD = CC.load_golden()


@pytest.mark.parametrize("seed", CC.SEEDS)
def test_oracle_reproduces_reference_c2f(seed):
    g = GOLD[str(seed)]
    p = g["case"]
    fine = oracle_c2f(p, CC.coarse_model(p))
    d = CC.digests(fine)
    assert d == {"fine": g["fine"], "pvel": g["pvel"], "svel": g["svel"]}
