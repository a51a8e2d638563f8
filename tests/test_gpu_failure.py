"""The solver's bounded waits, made to run out on purpose, on a real solve: the station's solve ends
with FDGPU_ESCHED and the detail code of the wait that gave up, nothing hangs, and the next solve on
the same context is bit-identical to the oracle.  The bounds are the context's (fdgpu_set_wait_limits),
set very low here; nothing else about the solve is unusual."""
import ctypes as C
import os

import numpy as np
import pytest

from cases import random_case, write_random_case
from oracle_util import run_oracle

pytestmark = pytest.mark.gpu
ESCHED = -7


def _solve(lib, ctx, st, slow, vel_shape, out):
    """fdgpu_solve_device on one station; returns (status, stats)."""
    nz, ny, nx = vel_shape
    L = lib.load()
    arr = (lib.Station * 1)(st)
    tp = (C.c_void_p * 1)(out.data_ptr())
    stats = (lib.Stats * 1)()
    rc = L.fdgpu_solve_device(ctx.ptr, 1, arr, C.c_void_p(slow.data_ptr()), nx, nx * ny, tp, 0, stats, None)
    return rc, stats[0].as_dict()


@pytest.mark.parametrize("limits, detail", [((0, 20000), 17), ((64, 0), 8)])
def test_a_wait_that_runs_out_is_reported(gpu_lib, tmp_path, limits, detail):
    import torch
    lib = gpu_lib
    c = random_case(14)
    pf = write_random_case(c, str(tmp_path))
    run_oracle(pf, str(tmp_path / "orc"))
    ref = np.fromfile(tmp_path / "orc" / "case.ptimes", dtype="<f4", offset=232)
    st, _, _ = lib.station_from_par("par=" + pf)
    if "parse" in c["par"]:
        pytest.skip("decimated output")
    with lib.Context(0) as ctx:
        v = torch.from_numpy(np.ascontiguousarray(c["vel"]).reshape(-1)).cuda()
        slow = torch.empty_like(v)
        ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel())
        out = torch.empty(st.shape, dtype=torch.float32, device="cuda")
        ctx.set_wait_limits(*limits)
        rc, s = _solve(lib, ctx, st, slow, c["vel"].shape, out)
        assert rc == ESCHED and s["status"] == ESCHED and s["detail"] == detail, (rc, s)
        ctx.set_wait_limits(0, 0)
        rc, s = _solve(lib, ctx, st, slow, c["vel"].shape, out)
        torch.cuda.synchronize()
        assert rc == 0 and s["status"] == 0, (rc, s)
        assert np.array_equal(out.cpu().numpy().reshape(-1).view(np.uint32), ref.view(np.uint32))
