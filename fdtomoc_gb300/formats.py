"""File formats of the sphfd path: the 232-byte ``vhead`` grid files and getpar-style par files.

The velocity input and the travel-time output of sphfd share one layout (reference:
include/common/vhead.h:4-11): a 120-byte text header, twelve float64 fields, one float32 and three
int32, then nx*ny*nz float32 values with x fastest.  Travel-time files carry "PTIM" in bytes 12-15
and the geocentric source (lon rad, colat rad, radius km) in fxs/fys/fzs (src/sphfd.c:5743-5801).
Downstream consumers read exactly this: sphfdloc (src/sphfdloc.c:1390-1475) and sphrayderv
(src/sphrayderv.c:1163-1218).
"""
from __future__ import annotations

import dataclasses
import os
import struct

import numpy as np

VHEAD_FMT = "<120s12df3i"
VHEAD_SIZE = struct.calcsize(VHEAD_FMT)
assert VHEAD_SIZE == 232


@dataclasses.dataclass
class VHead:
    """The 232-byte header (include/common/vhead.h:4-11)."""

    header: bytes = b"HEADFINESPHRVPMDNOFL"
    fxs: float = 0.0
    fys: float = 0.0
    fzs: float = 0.0
    clat: float = 0.0
    clon: float = 0.0
    cz: float = 0.0
    x0: float = 0.0
    y0: float = 0.0
    z0: float = 0.0
    dx: float = 0.0
    dy: float = 0.0
    dz: float = 0.0
    az: float = 0.0
    nx: int = 0
    ny: int = 0
    nz: int = 0

    def pack(self, byteorder: str = "<") -> bytes:
        text = self.header[:120].ljust(120, b"\0")
        return struct.pack(byteorder + VHEAD_FMT[1:], text, self.fxs, self.fys, self.fzs, self.clat,
                           self.clon, self.cz, self.x0, self.y0, self.z0, self.dx, self.dy, self.dz,
                           self.az, self.nx, self.ny, self.nz)

    @classmethod
    def unpack(cls, raw: bytes, byteorder: str = "<") -> "VHead":
        v = struct.unpack(byteorder + VHEAD_FMT[1:], raw[:VHEAD_SIZE])
        return cls(v[0], *v[1:])


def write_grid(path: str | os.PathLike, head: VHead, values: np.ndarray) -> None:
    """Write a vhead file; ``values`` is (nz, ny, nx) float32, x fastest on disk."""
    arr = np.ascontiguousarray(values, dtype="<f4")
    with open(path, "wb") as f:
        f.write(head.pack())
        f.write(arr.tobytes())


def read_grid(path: str | os.PathLike, nxyz: int | None = None) -> tuple[VHead, np.ndarray]:
    """Read a vhead file; returns the header and the (nz, ny, nx) float32 array (little-endian)."""
    raw = open(path, "rb").read()
    head = VHead.unpack(raw)
    n = head.nx * head.ny * head.nz if nxyz is None else nxyz
    data = np.frombuffer(raw, dtype="<f4", count=n, offset=VHEAD_SIZE)
    if nxyz is None:
        data = data.reshape(head.nz, head.ny, head.nx)
    return head, data


def write_par(path: str | os.PathLike, params: dict) -> None:
    """Write a getpar parameter file: one ``name=value`` per line (src/make_par_file.c:95-105)."""
    with open(path, "w") as f:
        for k, v in params.items():
            f.write(f"{k}={v}\n")


def read_par(path: str | os.PathLike, _level: int = 0) -> dict:
    """Parse a getpar file: whitespace-separated name=value tokens, '#' comments at token start,
    quoted values, ``par=<file>`` recursion; the last definition of a name wins
    (src/sphfd.c:6716-6766, search-backwards lookup at :6566)."""
    if _level > 20:
        raise ValueError("too many nested par files")
    out: dict = {}
    with open(path) as f:
        for line in f:
            i, n = 0, len(line)
            while True:
                while i < n and line[i] in " \t":
                    i += 1
                if i >= n or line[i] in "\n#":
                    break
                j = i
                while j < n and line[j] not in "= \t\n":
                    j += 1
                name = line[i:j]
                if j < n and line[j] == "=":
                    j += 1
                if j < n and line[j] in "\"'":
                    q = line[j]
                    j += 1
                    k = j
                    while k < n and line[k] not in (q, "\n"):
                        k += 1
                    value = line[j:k]
                    if k < n and line[k] == q:
                        k += 1
                else:
                    k = j
                    while k < n and line[k] not in " \t\n":
                        k += 1
                    value = line[j:k]
                out.pop(name, None)
                out[name] = value
                if name == "par":
                    out.update(read_par(value, _level + 1))
                i = k
    return out
