"""The location oracle against the reference's own sphfdloc: the four output files the reference
wrote for the seeded cases (tests/golden/loc_<seed>/, made by make_loc_golden.py) are rebuilt, byte
for byte, from the oracle's locations."""
import numpy as np
import pytest

import loc_cases as LC
from oracle_util import loc_grid, loc_helpers, oracle_locate


def locate_case(p):
    grid = loc_grid(p)
    ora = loc_helpers(grid)
    fl = LC.fields(p)
    keys = list(fl)
    index = {k: i for i, k in enumerate(keys)}
    field_list = [np.ascontiguousarray(fl[k]) for k in keys]
    events = LC.parsed_events(p, ora["htoe"])
    results = []
    for ev in events:
        obs = [(index[(o["sta"], o["phase"])], o["obstime"], o["pwt"], o["phase"], 1) for o in ev["obs"]]
        results.append(oracle_locate(grid, field_list, obs))
    return events, results, ora


@pytest.mark.parametrize("seed", LC.SEEDS)
def test_oracle_reproduces_reference_outputs(seed):
    p, ref = LC.load_golden(seed)
    events, results, ora = locate_case(p)
    got = LC.format_outputs(p, events, results, ora)
    for k in ("fhd", "sum", "dat", "out"):
        assert got[k] == ref[k], k


def test_cases_exercise_the_outlier_passes():
    passes, rejected = 0, 0
    for seed in LC.SEEDS:
        p, _ = LC.load_golden(seed)
        _, results, _ = locate_case(p)
        passes += sum(r["passes"] > 1 for r in results)
        rejected += sum(r["status"] != 0 for r in results)
    assert passes > 0 and rejected > 0


def test_library_grid_setup_equals_oracle(gpu_lib):
    """fdgpu_loc_grid_from_spec (host code, no GPU) and the oracle convert a spec identically."""
    import ctypes as C
    for seed in LC.SEEDS:
        p, _ = LC.load_golden(seed)
        a = loc_grid(p)
        b = gpu_lib.loc_grid_from_spec(p["nx"], p["ny"], p["nz"], p["x0"], p["y0"], p["z0"], p["h"])
        for name, _t in gpu_lib.LocGrid._fields_:
            if name in ("kmin", "ndiv", "ndiv2", "nthres", "resthres", "resthrep", "stdmax", "ivs", "vpvs"):
                continue
            x, y = getattr(a, name), getattr(b, name)
            assert np.float64(x).tobytes() == np.float64(y).tobytes(), (seed, name, x, y)
