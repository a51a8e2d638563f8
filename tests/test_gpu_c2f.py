"""c2f on the device (fdgpu_c2f) against the reference's own c2f (digests of its output files) and
the c2f oracle, with host and device buffers."""
import numpy as np
import pytest

import c2f_cases as CC
from oracle_util import oracle_c2f

pytestmark = pytest.mark.gpu
GOLD = CC.load_golden()


def run(lib, ctx, p, coarse, on_device):
    import torch
    args = (p["nxc"], p["nyc"], p["nzc"], p["igridx"], p["igridy"], p["igridz"], p["x0"], p["y0"], p["z0"], p["h"])
    if not on_device:
        return lib.c2f(ctx, *args, np.ascontiguousarray(coarse))
    nx, ny, nz = CC.dims(p)
    src = torch.from_numpy(np.ascontiguousarray(coarse)).cuda()
    dst = torch.empty((2, nz, ny, nx), dtype=torch.float32, device="cuda")
    lib.c2f(ctx, *args, src, dst)
    return dst.cpu().numpy()


@pytest.mark.parametrize("seed", CC.SEEDS)
@pytest.mark.parametrize("on_device", [False, True])
def test_gpu_c2f_equals_reference(gpu_lib, seed, on_device):
    g = GOLD[str(seed)]
    p = g["case"]
    with gpu_lib.Context(0) as ctx:
        fine = run(gpu_lib, ctx, p, CC.coarse_model(p), on_device)
    assert CC.digests(fine) == {"fine": g["fine"], "pvel": g["pvel"], "svel": g["svel"]}


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_gpu_c2f_equals_oracle_large(gpu_lib, seed):
    rng = np.random.default_rng(seed)
    nxc, nyc, nzc = int(rng.integers(20, 60)), int(rng.integers(20, 60)), int(rng.integers(8, 20))
    p = dict(nxc=nxc, nyc=nyc, nzc=nzc, h=float(rng.choice([0.1, 0.3, 0.7])),
             igridx=[int(v) for v in rng.integers(1, 9, nxc - 1)], igridy=[int(v) for v in rng.integers(1, 9, nyc - 1)],
             igridz=[int(v) for v in rng.integers(1, 5, nzc - 1)], x0=-55.5, y0=-41.3, z0=-3.1)
    coarse = (4.0 + 4.0 * rng.random((2, nzc, nyc, nxc))).astype(np.float32)
    with gpu_lib.Context(0) as ctx:
        fine = run(gpu_lib, ctx, p, coarse, True)
    want = oracle_c2f(p, coarse)
    assert np.array_equal(fine.view(np.uint32), want.view(np.uint32))


def test_gpu_c2f_plan_reused(gpu_lib):
    """A plan interpolates successive coarse models (an inversion's iterations) like one-shot calls."""
    import torch
    g = GOLD["2"]
    p = g["case"]
    args = (p["nxc"], p["nyc"], p["nzc"], p["igridx"], p["igridy"], p["igridz"], p["x0"], p["y0"], p["z0"], p["h"])
    with gpu_lib.Context(0) as ctx:
        plan = gpu_lib.C2fPlan(ctx, *args)
        out = torch.empty(plan.shape, dtype=torch.float32, device="cuda")
        for it in range(3):
            coarse = CC.coarse_model(p) * np.float32(1.0 + 0.01 * it)
            src = torch.from_numpy(np.ascontiguousarray(coarse)).cuda()
            plan.run(src.data_ptr(), out.data_ptr())
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle_c2f(p, coarse).view(np.uint32))
        plan.close()
