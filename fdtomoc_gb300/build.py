"""Build of libfdgpu.so and the drop-in sphfd, sphfdloc and sphrayderv executables for sm_103a (nvcc, no
cmake)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfdgpu.so")
EXE = os.path.join(HERE, "bin", "sphfd_gpu")
EXE_RAY = os.path.join(HERE, "bin", "sphrayderv_gpu")
EXE_LOC = os.path.join(HERE, "bin", "sphfdloc_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: the solver's FP64 arithmetic must not be contracted into fused multiply-adds;
# -ffp-contract=off does the same for host code (aarch64 gcc contracts by default).
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "--expt-relaxed-constexpr",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose: bool = False, defines=(), lib_path: str | None = None) -> str:
    """Compile the library.  `defines` (e.g. ["FDGPU_PHASE_TIMERS"]) and `lib_path` build a
    separately named profiling variant."""
    nvcc = _nvcc()
    lib_out = lib_path or LIB
    tag = "_".join(defines)
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(EXE), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "fdgpu.h"))
    units = [("fdgpu_kernels.cu", []), ("fdgpu_host.cpp", []), ("fdgpu_noalloc.cu", []), ("fdgpu_serve.cpp", []), ("fdgpu_locate.cu", []), ("fdgpu_c2f.cu", []), ("fdgpu_ray.cu", []), ("fdgpu_rayderv.cpp", []), ("fdgpu_sphfdloc.cpp", [])]
    objs = []
    jobs = []
    for src, extra in units:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + (("." + tag) if tag else "") + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + NVFLAGS + extra + ["-D" + d for d in defines] + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stderr)
    if force or _stale(lib_out, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", lib_out] + objs + ["-lpthread"])
    if lib_path:
        return lib_out
    for exe, main in ((EXE, "sphfd_main.cpp"), (EXE_RAY, "sphrayderv_main.cpp"), (EXE_LOC, "sphfdloc_main.cpp")):
        main = os.path.join(CSRC, main)
        if force or _stale(exe, [main, LIB]):
            _run([nvcc] + ARCH + NVFLAGS + [main, "-o", exe, "-L" + HERE, "-lfdgpu", "-Xlinker", "-rpath=" + HERE])
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
