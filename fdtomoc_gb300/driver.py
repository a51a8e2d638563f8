"""sphfd's driver (src/sphfd.c:200-257) over the ranks of a torch.distributed job.

The reference's main reads a spec ("parlist <file>", "timedir <dir>", src/sphfd.c:214-227), then
solves every "par=<file>" line of the par list (at most MAXNUMPAR = 2000, :143) with an OpenMP
parallel loop, one sphfd() per line, each writing <timedir>/<timefile>.  Stations are independent,
so the GPU counterpart shards them: rank r of a job of W ranks takes lines r, r + W, r + 2W, ...
and solves them on its own GPU (fdgpu_sphfd_parlist_devices with device $LOCAL_RANK); the time
files are gathered once, and rank 0 alone writes them, so ranks that share a file system never
write the same file.  Every rank returns the statuses of all lines.  Without torch.distributed (or
with one rank) it is the plain parlist drop-in.
"""
from __future__ import annotations

import os
import tempfile

MAXNUMPAR = 2000


def read_spec(spec_path: str):
    """The two keys sphfd's main reads from its spec (get_vars: first word, then the value)."""
    vals = {}
    with open(spec_path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2 and parts[0] in ("parlist", "timedir") and parts[0] not in vals:
                vals[parts[0]] = parts[1]
    if "parlist" not in vals or "timedir" not in vals:
        raise ValueError(f"{spec_path}: needs 'parlist' and 'timedir'")
    return vals["parlist"], vals["timedir"]


def read_parlist(parlist_path: str):
    """The par-list entries ("par=<file>" lines; blank lines skipped), at most MAXNUMPAR."""
    with open(parlist_path) as f:
        entries = [ln.strip() for ln in f if ln.strip()]
    if len(entries) > MAXNUMPAR:
        raise ValueError(f"{parlist_path}: {len(entries)} entries, more than {MAXNUMPAR}")
    return entries


def gpu_solver(device: int | None = None):
    """solve(entries, outdir) -> statuses with the GPU drop-in on `device` ($LOCAL_RANK by default)."""
    from . import lib
    dev = int(os.environ.get("LOCAL_RANK", 0)) if device is None else device

    def solve(entries, outdir):
        return lib.sphfd_parlist(entries, outdir, devices=[dev])

    return solve


def run_spec(spec_path: str, solve=None, group=None):
    """Solve every station of a spec's par list, sharded over the ranks of `group` (the default
    group when torch.distributed is initialised).  Returns the statuses in par-list order."""
    parlist, timedir = read_spec(spec_path)
    entries = read_parlist(parlist)
    return run_entries(entries, timedir, solve, group)


def run_entries(entries, timedir: str, solve=None, group=None):
    solve = solve or gpu_solver()
    dist = None
    try:
        import torch.distributed as _d
        if _d.is_available() and _d.is_initialized():
            dist = _d
    except ImportError:
        pass
    world = dist.get_world_size(group) if dist else 1
    rank = dist.get_rank(group) if dist else 0
    if world == 1:
        os.makedirs(timedir, exist_ok=True)
        return list(solve(entries, timedir))
    mine = list(range(rank, len(entries), world))
    with tempfile.TemporaryDirectory(prefix=f"sphfd_r{rank}_") as d:
        st = list(solve([entries[k] for k in mine], d)) if mine else []
        files = {}
        for name in sorted(os.listdir(d)):
            with open(os.path.join(d, name), "rb") as f:
                files[name] = f.read()
    parts = [None] * world
    dist.all_gather_object(parts, (mine, st, files), group=group)
    status = [0] * len(entries)
    for idx, s, _ in parts:
        for k, v in zip(idx, s):
            status[k] = v
    if rank == 0:
        os.makedirs(timedir, exist_ok=True)
        for _, _, fl in parts:
            for name, data in fl.items():
                with open(os.path.join(timedir, name), "wb") as f:
                    f.write(data)
    dist.barrier(group)
    return status
