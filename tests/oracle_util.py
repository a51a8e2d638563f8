"""Test-side access to the CPU oracle (oracle/): build it and run it on par files."""
import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_lib = None


class OracleStats(C.Structure):
    _fields_ = [("node_updates", C.c_int64), ("calls", C.c_int64 * 5), ("skipped", C.c_int64 * 5),
                ("inherit_points", C.c_int64), ("faces", C.c_int64), ("sweeps", C.c_int),
                ("restarts", C.c_int * 7), ("changed_per_sweep", C.c_int64 * 64),
                ("depth_per_sweep", C.c_int64 * 64), ("updates_per_sweep", C.c_int64 * 64)]


def load_oracle():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so", "sphfd_oracle"], check=True)
        lib = C.CDLL(os.path.join(ORACLE_DIR, "liboracle.so"))
        lib.fdo_sphfd.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_char_p, C.c_int, C.POINTER(OracleStats)]
        _lib = lib
    return _lib


def run_oracle(parfile: str, timedir: str, fast: bool = False):
    """Run the oracle's whole-station driver; returns its statistics."""
    lib = load_oracle()
    os.makedirs(timedir, exist_ok=True)
    argv = (C.c_char_p * 2)(b"sphfd", ("par=" + parfile).encode())
    st = OracleStats()
    rc = lib.fdo_sphfd(2, argv, timedir.encode(), 1 if fast else 0, C.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle failed on {parfile}: {rc}")
    return st
