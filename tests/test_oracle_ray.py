"""The sphrayderv oracle (oracle/fd_ray.c) and the host side (fdtomoc_gb300/rayderv.py) against the
reference's own sphrayderv: on the seeded cases of tests/golden/ray_cases.py the six output files
(dt/ds matrix, residuals, hypocentre derivatives, bookkeeping, index vector, hit counts) must equal
the reference's byte for byte, with the C library's trig functions (as the reference calls them)
and with the double-double ones the device uses.
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))

import ray_cases as RC  # noqa: E402
from oracle_util import oracle_trace, ray_lib  # noqa: E402

from fdtomoc_gb300 import rayderv as R  # noqa: E402


@pytest.mark.parametrize("seed", RC.SEEDS + RC.EXTRA_SEEDS)
@pytest.mark.parametrize("trig", [0, 1])
def test_files_equal_reference(seed, trig, tmp_path):
    p = RC.make_case(seed)
    spec = RC.write_inputs(p, str(tmp_path))
    out = R.run(spec, oracle_trace(trig))
    gold = RC.load_golden(seed)
    for name in RC.OUT_FILES:
        assert out[name] == gold[name], f"{name} differs"


def test_cases_cover_the_failure_paths(tmp_path):
    """rays that leave the model, cells without times, events whose first phase fails"""
    seen = set()
    first_fails = 0
    for seed in RC.SEEDS + RC.EXTRA_SEEDS:
        p = RC.make_case(seed)
        spec = RC.write_inputs(p, str(tmp_path / str(seed)))
        sp = R.read_spec(spec)
        g, keep = R.grid_from_spec(sp)
        obs, nobs, plan, fields = R.build_observations(sp, g, R.read_stations(sp["stafile"]),
                                                       R.read_events(sp["locdfil"]))
        res, off, idx, du = oracle_trace(0)(g, R.load_fields(sp, g, fields), obs, nobs, R.default_cap(g))
        seen |= {res[o].status for o in range(nobs)}
        first_fails += sum(1 for inside, rows in plan
                           if inside and rows and (rows[0][0] < 0 or res[rows[0][0]].status != R.RAY_OK))
    assert {R.RAY_OK, R.RAY_LEFT, R.RAY_NOTIME} <= seen
    assert first_fails >= 3


def test_double_double_trig_is_within_one_ulp_of_libm():
    """The device's sin/cos/atan2 differ from the C library's in a small fraction of arguments, by one
    unit in the last place (where they differ, the double-double result is the correctly rounded one)."""
    lib = ray_lib()
    rng = np.random.default_rng(11)
    diff = n = 0
    for x in rng.uniform(-4.0, 4.0, 20000):
        for w in (0, 1):
            a, b = lib.fdr_trig(1, w, x, 0.0), lib.fdr_trig(0, w, x, 0.0)
            n += 1
            if a != b:
                diff += 1
                assert abs(a - b) <= math.ulp(b)
    for _ in range(10000):
        y, x = rng.uniform(-5000, 5000), rng.uniform(-5000, 5000)
        a, b = lib.fdr_trig(1, 2, y, x), lib.fdr_trig(0, 2, y, x)
        n += 1
        if a != b:
            diff += 1
            assert abs(a - b) <= math.ulp(b)
    assert diff <= n * 0.01


def test_double_double_trig_is_correctly_rounded():
    """sin, cos and atan2 of fd_trig.h against 40-digit values: every result is the correctly rounded
    double (the functions the device uses; see the module for the method)"""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    lib = ray_lib()
    rng = np.random.default_rng(23)
    bad = []
    for x in np.concatenate([rng.uniform(-7.0, 7.0, 1500), rng.uniform(0.3, 2.3, 1500)]):
        if lib.fdr_trig(1, 0, x, 0.0) != float(mp.sin(mp.mpf(x))):
            bad.append(("sin", x))
        if lib.fdr_trig(1, 1, x, 0.0) != float(mp.cos(mp.mpf(x))):
            bad.append(("cos", x))
    for _ in range(1500):
        y, x = rng.uniform(-7000, 7000), rng.uniform(-7000, 7000)
        if lib.fdr_trig(1, 2, y, x) != float(mp.atan2(mp.mpf(y), mp.mpf(x))):
            bad.append(("atan2", y, x))
    assert not bad, bad[:5]
