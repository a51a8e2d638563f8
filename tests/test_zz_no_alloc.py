"""fdgpu_solve_noalloc — the entry point for callers that cannot let the library allocate device
memory (loops that must not pay cudaFree's device-wide synchronisation, applications whose GPU
memory belongs to another allocator).  Its scratch is one static device array shared by every
call, so it is checked against the allocating entry point on two calls in a row: the second call
must not be disturbed by what the first left in the array.

This file sorts last so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cases import random_case, write_random_case

pytestmark = pytest.mark.gpu


def _bind(lib):
    L = lib.load()
    L.fdgpu_solve_noalloc.argtypes = [C.POINTER(lib.Station), C.c_void_p, C.c_longlong, C.c_longlong, C.c_void_p,
                                      C.POINTER(lib.Stats), C.c_void_p]
    L.fdgpu_solve_noalloc.restype = C.c_int
    return L


def _case(lib, tmp_path, seed):
    c = random_case(seed)
    pf = write_random_case(c, str(tmp_path / f"c{seed}"))
    st, _, _ = lib.station_from_par("par=" + pf)
    return st, c["vel"]


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib, tmp_path):
    import torch
    lib = gpu_lib
    L = _bind(lib)
    cases = [_case(lib, tmp_path, s) for s in (4, 13)]
    with lib.Context(0) as ctx:
        for st, vel in cases:
            if st.srctype != 1:
                continue
            nz, ny, nx = vel.shape
            v = torch.from_numpy(np.ascontiguousarray(vel).reshape(-1)).cuda()
            slow = torch.empty_like(v)
            ctx.velocity_to_slowness(v.data_ptr(), slow.data_ptr(), v.numel())
            ref = torch.empty((st.nz, st.ny, st.nx), dtype=torch.float32, device="cuda")
            ctx.solve_device([st], slow.data_ptr(), nx, nx * ny, [ref.data_ptr()])
            torch.cuda.synchronize()
            for call in range(2):
                out = torch.full((st.nz, st.ny, st.nx), -1.0, dtype=torch.float32, device="cuda")
                stats = lib.Stats()
                rc = L.fdgpu_solve_noalloc(C.byref(st), slow.data_ptr(), nx, nx * ny, out.data_ptr(), C.byref(stats),
                                           None)
                assert rc == 0, lib.load().fdgpu_strerror(rc)
                torch.cuda.synchronize()
                assert stats.status == 0 and stats.sweeps >= 1
                assert torch.equal(out.view(torch.int32), ref.view(torch.int32)), f"call {call} differs"


def test_noalloc_rejects_too_large(gpu_lib, tmp_path):
    import torch
    lib = gpu_lib
    L = _bind(lib)
    st, vel = _case(lib, tmp_path, 4)
    big = lib.Station.from_buffer_copy(st)
    big.nx, big.ny, big.nz = 401, 401, 161          # about 50 MB of tables and scratch
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = L.fdgpu_solve_noalloc(C.byref(big), dummy.data_ptr(), 401, 401 * 401, dummy.data_ptr(), None, None)
    assert rc == -9
    assert b"exceeds the memory" in lib.load().fdgpu_strerror(rc)
