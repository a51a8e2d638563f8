"""sphfd's driver (src/sphfd.c:200-257) over the ranks of a torch.distributed job.

The reference's main reads a spec ("parlist <file>", "timedir <dir>", src/sphfd.c:214-227), then
solves every "par=<file>" line of the par list (at most MAXNUMPAR = 2000, :143) with an OpenMP
parallel loop, one sphfd() per line, each writing <timedir>/<timefile>.  Stations are independent,
so the GPU counterpart shards them: rank r of a job of W ranks takes lines r, r + W, r + 2W, ...
and solves them on its own GPU (fdgpu_sphfd_parlist_devices with device $LOCAL_RANK).  The time
files reach the timedir in one of two ways:
  write="each"   every rank writes its own stations' files into the timedir, as the reference's
                 threads do (ranks on one node, or nodes sharing a file system: the stations are
                 disjoint, so no two ranks write one file, and no field crosses a link);
  write="rank0"  ranks without a shared file system send their files to rank 0 one at a time
                 (point-to-point), and rank 0 alone writes them; rank 0 holds one file at a time,
                 never the job's fields.
Every rank returns the statuses of all lines (one small all-gather).  Without torch.distributed (or
with one rank) it is the plain parlist drop-in.  Over NCCL, as for any object collective, each rank
selects its GPU (torch.cuda.set_device($LOCAL_RANK)) before calling.
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


def run_spec(spec_path: str, solve=None, group=None, write: str = "each"):
    """Solve every station of a spec's par list, sharded over the ranks of `group` (the default
    group when torch.distributed is initialised).  Returns the statuses in par-list order."""
    parlist, timedir = read_spec(spec_path)
    entries = read_parlist(parlist)
    return run_entries(entries, timedir, solve, group, write)


def _files_under(d: str):
    """relative paths of the files below d (a timefile may name a subdirectory)"""
    out = []
    for root, _, names in os.walk(d):
        for n in names:
            out.append(os.path.relpath(os.path.join(root, n), d))
    return sorted(out)


def run_entries(entries, timedir: str, solve=None, group=None, write: str = "each"):
    if write not in ("each", "rank0"):
        raise ValueError(f"write must be 'each' or 'rank0', not {write!r}")
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
    if write == "each":
        os.makedirs(timedir, exist_ok=True)
        st = list(solve([entries[k] for k in mine], timedir)) if mine else []
    else:
        with tempfile.TemporaryDirectory(prefix=f"sphfd_r{rank}_") as d:
            st = list(solve([entries[k] for k in mine], d)) if mine else []
            _collect(dist, group, rank, world, d, timedir)
    parts = [None] * world
    dist.all_gather_object(parts, (mine, st), group=group)
    status = [0] * len(entries)
    for idx, s in parts:
        for k, v in zip(idx, s):
            status[k] = v
    dist.barrier(group)
    return status


def _collect(dist, group, rank, world, d, timedir):
    """write="rank0": every rank's files to rank 0, one file per message, in rank order"""
    def peer(r):
        return dist.get_global_rank(group, r) if group is not None else r

    if rank == 0:
        os.makedirs(timedir, exist_ok=True)
        for name in _files_under(d):
            with open(os.path.join(d, name), "rb") as f:
                _write(timedir, name, f.read())
        for r in range(1, world):
            count = [None]
            dist.recv_object_list(count, src=peer(r), group=group)
            for _ in range(count[0]):
                msg = [None]
                dist.recv_object_list(msg, src=peer(r), group=group)
                _write(timedir, *msg[0])
    else:
        names = _files_under(d)
        dist.send_object_list([len(names)], dst=peer(0), group=group)
        for name in names:
            with open(os.path.join(d, name), "rb") as f:
                dist.send_object_list([(name, f.read())], dst=peer(0), group=group)


def _write(timedir, name, data):
    path = os.path.join(timedir, name)
    os.makedirs(os.path.dirname(path) or timedir, exist_ok=True)
    with open(path, "wb") as f:
        f.write(data)
