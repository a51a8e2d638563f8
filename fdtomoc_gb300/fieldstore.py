"""Travel-time fields of many stations, device-resident up to a memory budget, spilled to pinned host
memory beyond it.

An inversion iteration solves every station's P and S field (the reference writes each to a time
file, src/sphfd.c:5800-5801, and sphfdloc / sphrayderv read them back).  Kept on the device, the
fields feed those consumers without a file round trip; but 1200 stations of 401x401x161 are about
125 GB, so a store gives each finished field a place: on the device while the fields held there fit
`device_budget` bytes, otherwise in pinned host memory.  When a new request needs device room, the
oldest finished resident fields are spilled to pinned host memory first (a device-to-host copy on
the store's own stream; the device buffer is released once the copy is done).  A request that still
does not fit is solved straight into a pinned host buffer: the serving session copies it out when
the solve finishes.  Solving itself is the serving session's (fdtomoc_gb300.lib.Server): it admits
requests by its own device-memory budget and solves them as they arrive.

The store changes where a field lives, never its values: every field is bit-identical to the same
station solved alone.
"""
from __future__ import annotations

import collections


class FieldStore:
    def __init__(self, server, device_budget: int, device: int = 0):
        import torch
        self.sv = server
        self.budget = int(device_budget)
        self.device = device
        self.used = 0                      # bytes of device-resident fields (finished or in flight)
        self.dev = {}                      # key -> device tensor
        self.host = {}                     # key -> pinned host tensor
        self.pending = {}                  # request id -> key
        self.resident = collections.OrderedDict()   # finished device-resident keys, oldest first
        self.copies = []                   # (event, device tensor) of spills not yet known complete
        self.spill_event = {}              # key -> the event of its spill copy
        self.stream = torch.cuda.Stream(device)
        self.results = {}                  # key -> the request's result
        self.spilled = 0
        self.direct_to_host = 0

    @staticmethod
    def _bytes(station) -> int:
        return 4 * station.nx * station.ny * station.nz

    def _reap(self, wait: bool = False):
        keep = []
        for ev, t in self.copies:
            if wait:
                ev.synchronize()
            if not ev.query():
                keep.append((ev, t))
        self.copies = keep

    def _spill(self, key):
        import torch
        t = self.dev.pop(key)
        self.resident.pop(key)
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        with torch.cuda.stream(self.stream):
            self.stream.wait_stream(torch.cuda.current_stream(self.device))
            h.copy_(t, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.stream)
        t.record_stream(self.stream)
        self.copies.append((ev, t))
        self.spill_event[key] = ev
        self.host[key] = h
        self.used -= t.numel() * 4
        self.spilled += 1

    def submit(self, key, station, model: int, init=None, tag: int = 0) -> int:
        """Queue a solve whose field will be found under `key`."""
        import torch
        need = self._bytes(station)
        while self.used + need > self.budget and self.resident:
            self._spill(next(iter(self.resident)))
        on_device = self.used + need <= self.budget
        if on_device:
            out = torch.empty(station.shape, dtype=torch.float32, device=f"cuda:{self.device}")
        else:
            out = torch.empty(station.shape, dtype=torch.float32, pin_memory=True)
        rid = self.sv.submit(station, model, out, init=init, tag=tag)   # raises before anything is kept
        if on_device:
            self.dev[key] = out
            self.used += need
        else:
            self.host[key] = out
            self.direct_to_host += 1
        self.pending[rid] = key
        return rid

    def poll(self, max_results: int = 256, timeout_ms: int = 0):
        """Collect finished requests (see Server.poll); returns their results."""
        res = self.sv.poll(max_results, timeout_ms)
        for r in res:
            key = self.pending.pop(r["id"])
            self.results[key] = r
            if key in self.dev:
                self.resident[key] = True
        self._reap()
        return res

    def drain(self, timeout_ms: int = -1):
        """Wait for every request and every spill copy."""
        self.sv.drain(timeout_ms)
        while self.pending:
            self.poll(256, 1000)
        self._reap(wait=True)

    def get(self, key):
        """The field: a device tensor if resident, else a pinned host tensor (once its spill copy, if
        any, has finished).  Call it after the request's result has been polled."""
        ev = self.spill_event.pop(key, None)
        if ev is not None:
            ev.synchronize()
        return self.dev.get(key, self.host.get(key))

    def where(self, key) -> str:
        return "device" if key in self.dev else "host" if key in self.host else "none"
