#!/usr/bin/env python3
"""Benchmark of the GB300 sphfd travel-time solver.

Metric: station travel-time fields per second (with node-updates/s).  Default workload: 500 station
windows sized uniformly in 41..301 x 41..301 x 41..121 (seed 3) over a 401x401x161 model at
0.005 deg x 0.005 deg x 0.5 km (layered 1-D model with a 5 % / 10 km perturbation, seed 4), solved as
one prepared batch: one step = one kernel launch over all 500 windows.  Every field is compared with
the reference binary's (SHA-256 pins made by tests/golden/make_headline_golden.py).  The same line
carries the config-2 legs: 64 stations of 201x201x81 in one launch, and the location, c2f, ray and
serving legs on their fields.

  python bench.py [--gpus N] [--steps K] [--warmup W]     GPU arm (torchrun for N > 1)
  python bench.py --impl reference ...                     CPU arm: the oracle on the host cores

The reference repository has no GPU code; the CPU arm runs this repository's C restatement of
its solver (oracle/, pinned bit-exact against the reference's own binary and golden file) on all
host cores, one process per core, as the reference's OpenMP driver does.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "station fields/s (batched, 201x201x81, bit-identical to reference)"
UNIT = "station fields/s"
STATIONS_PER_GPU = 64
CONFIG_NAME = "64 stations, 201x201x81 grid, 0.005deg x 0.005deg x 0.5km (config 2)"
CONFIG1_NAME = "1 station, 61x61x31 grid, 0.01deg x 0.01deg x 1km (config 1, profiling case)"
ALGO_BYTES_PER_NODE_UPDATE = 12  # slowness read, time read, time write


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--stations", type=int, default=None, help="stations per GPU (default 64; config 1: 1)")
    ap.add_argument("--rate", type=float, default=12.0, help="--config 4: request arrivals per second")
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3, 4, 5],
                    help="3 (default): the 500-window uneven batch, with the config-2 legs; 2: 64 stations of "
                         "201x201x81; 1: the one-station 61x61x31 case, for profiling; 4: served P/S requests; "
                         "5: stations on the full 401x401x161 grid with memory admission (each its own JSON line)")
    ap.add_argument("--no-config2", action="store_true", help="--config 3: leave out the config-2 legs")
    ap.add_argument("--field-budget", type=int, default=6,
                    help="--config 5: fields kept on the device (beyond it they spill to pinned host memory)")
    ap.add_argument("--session-gb", type=int, default=120, help="--config 5: the serving session's device memory")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=300,
                    help="requests of the serving leg (0: skip it)")
    ap.add_argument("--locate-events", type=int, default=256,
                    help="events of the location leg (0: skip it)")
    ap.add_argument("--no-c2f", action="store_true", help="skip the c2f leg")
    ap.add_argument("--ray-events", type=int, default=1024,
                    help="events of the sphrayderv ray leg (0: skip it)")
    ap.add_argument("--profile-legs", action="store_true",
                    help="only run a small fixed case of the c2f and location kernels (for ncu captures)")
    args = ap.parse_args()
    if args.stations is None:
        args.stations = STATIONS_PER_GPU if args.config == 2 else 16 if args.config == 5 else 1
    return args


def under_profiler() -> bool:
    """Whether a CUDA profiler (Nsight Compute) is injected into this process: it sets one of these
    variables (which one depends on the tool's version)."""
    return any(os.environ.get(k) for k in ("CUDA_INJECTION64_PATH", "NV_NSIGHT_INJECTION_TRANSPORT_TYPE",
                                            "NV_TPS_LAUNCH_TOKEN", "NVIDIA_PROCESS_INJECTION_XML_TARGET_SETTINGS"))


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def workload(rank: int, n: int, cfg: int = 2):
    """The model of config cfg and this rank's n stations (weak scaling: rank r takes its own)."""
    from fdtomoc_gb300 import workloads as W
    g, v, _ = W.config(cfg)
    sts = W.stations(g, n * (rank + 1), cfg)[n * rank:]
    return g, v, sts


def write_case(dirname, g, v, sts):
    from fdtomoc_gb300 import workloads as W
    return W.write_case(dirname, g, v, sts)


# ----------------------------------------------------------------------------------------------
# CPU side: the oracle, one process per core


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so", "sphfd_oracle"], check=True)
    return os.path.join(ROOT, "oracle", "sphfd_oracle")


def cpu_solve(case_dir, names, cores, mode="fast"):
    """Solve the named stations with the oracle, one process per core; returns (wall s, node updates)."""
    exe = build_oracle()
    out = os.path.join(case_dir, "cpu_out")
    os.makedirs(out, exist_ok=True)
    procs = []
    env = dict(os.environ, FDO_MODE=mode, OMP_NUM_THREADS="1")
    t0 = time.time()
    pending = list(names)
    running = []
    logs = {}
    while pending or running:
        while pending and len(running) < cores:
            nm = pending.pop(0)
            pl = os.path.join(case_dir, f"pl_{nm}")
            with open(pl, "w") as f:
                f.write(f"par={os.path.join(case_dir, nm + '.par')}\n")
            spec = os.path.join(case_dir, f"spec_{nm}")
            with open(spec, "w") as f:
                f.write(f"parlist {pl}\ntimedir {out}\n")
            p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                                 text=True, env=env)
            p.stdin.write(spec + "\n")
            p.stdin.close()
            running.append((nm, p))
        time.sleep(0.02)
        still = []
        for nm, p in running:
            if p.poll() is None:
                still.append((nm, p))
            else:
                logs[nm] = p.stderr.read()
                if p.returncode != 0:
                    raise RuntimeError(f"oracle failed on {nm}: {logs[nm]}")
        running = still
    wall = time.time() - t0
    nu = 0
    for nm in names:
        for tok in logs[nm].split():
            if tok.startswith("node_updates="):
                nu += int(tok.split("=")[1])
    return wall, nu, out


# ----------------------------------------------------------------------------------------------
# clocks sampled during the timed region


class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                                      "-i", str(self.index)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------------------------
# GPU arm


def serve_leg(args, lib, stations, v, batch_fields):
    """Serving: P and S requests for the workload's stations (S = P/1.73 with an independent 2 %
    perturbation), all submitted at once to a serving session that keeps both models and every
    field on the device; throughput, latency percentiles, and the P fields checked bit for bit
    against the batch step's."""
    import numpy as np
    import torch
    from fdtomoc_gb300 import workloads as W
    n = args.serve_requests
    vs = (v / 1.73 * (1.0 + 0.02 * W.smooth_noise(v.shape, (0.5, 0.556, 0.509), 10.0, 44))).astype(np.float32)
    reqs = [(stations[k // 2 % len(stations)], k % 2) for k in range(n)]
    outs = [torch.empty(st.shape, dtype=torch.float32, device="cuda") for st, _ in reqs]
    torch.cuda.synchronize()
    with lib.Server(torch.cuda.current_device(), hbm_bytes=min(96 << 30, (8 << 30) + n * (96 << 20))) as sv:
        sv.set_model(0, v)
        sv.set_model(1, vs)
        t0 = time.time()
        for k, (st, phase) in enumerate(reqs):
            sv.submit(st, phase, outs[k], tag=k)
        sv.drain(1800000)
        wall = time.time() - t0
        res = sv.poll(n + 8)
        m = sv.metrics()
    bad = sum(1 for r in res if r["status"] != 0)
    same = all(torch.equal(outs[2 * k], batch_fields[k]) for k in range(min(len(batch_fields), n // 2)))
    return {"requests": n, "phases": "P and S alternating", "fields_per_s": n / wall, "wall_s": wall,
            "node_updates_per_s": m["node_updates"] / wall, "latency_ms": {"p50": m["p50_ms"], "p99": m["p99_ms"]},
            "solve_ms": {"p50": m["solve_p50_ms"], "p99": m["solve_p99_ms"]}, "solver_ctas": m["solver_ctas"],
            "hbm_peak_bytes": m["hbm_peak"], "failed": bad, "p_fields_equal_batch": same,
            "what": "all requests submitted at once; latency = submission to field ready on the device"}


def locate_leg(args, lib, ctx, g, fields, stream):
    """Event location (sphfdloc's grid search, fdgpu_locate) against the batch step's 64 P fields
    still on the device: args.locate_events synthetic events, each with 24-40 picks taken from the
    fields at a random grid node plus 20 ms noise and a few gross outliers.  Timed through the public
    call (phases in from host memory, results out).  CPU baseline: the location oracle on the host
    cores (one event per thread) for a sample of the events, whose results are also compared with the
    GPU's bit for bit."""
    import ctypes as C
    from concurrent.futures import ThreadPoolExecutor
    import numpy as np
    import torch
    E = args.locate_events
    grid = lib.loc_grid_from_spec(g.nx, g.ny, g.nz, g.x0, g.y0, g.z0, g.h)
    rng = np.random.default_rng(7)
    ns = len(fields)
    hyp = np.stack([rng.integers(0, g.nx, E), rng.integers(0, g.ny, E), rng.integers(grid.kmin, g.nz, E)], 1)
    stack = torch.stack([f.reshape(-1) for f in fields])            # (ns, nxyz) on the device
    node = torch.from_numpy((hyp[:, 2] * g.ny * g.nx + hyp[:, 1] * g.nx + hyp[:, 0]).astype(np.int64)).cuda()
    tt = stack[:, node].T.cpu().numpy()                              # (E, ns) travel times
    events = []
    for e in range(E):
        sel = rng.choice(ns, size=int(rng.integers(24, 41)), replace=False)
        ob = []
        for s_ in sel:
            t = float(tt[e, s_]) + 5.0 + float(rng.normal(0, 0.02))
            if rng.random() < 0.05:
                t += float(rng.choice([-1.5, 2.5]))
            w = np.float32(rng.choice([0.05, 0.1, 0.2]))
            ob.append((int(s_), float(np.float32(t)), float(np.float32(1.0) / (w * w)), "P", 1))
        events.append(ob)
    ptrs = [f.data_ptr() for f in fields]
    res = lib.locate(ctx, grid, ptrs, events[:8], stream.cuda_stream)   # warm-up
    torch.cuda.synchronize()
    t0 = time.time()
    res = lib.locate(ctx, grid, ptrs, events, stream.cuda_stream)
    gpu_s = time.time() - t0
    nobs = sum(len(ob) for ob in events)

    # CPU: the oracle, one event per host thread (ctypes releases the GIL during the call)
    build_oracle()
    olib = C.CDLL(os.path.join(ROOT, "oracle", "liboracle.so"))

    class OObs(C.Structure):
        _fields_ = [("field", C.c_int), ("obstime", C.c_float), ("pwt", C.c_float), ("phase", C.c_char),
                    ("good", C.c_int)]
    olib.fdo_locate.argtypes = [C.POINTER(lib.LocGrid), C.POINTER(C.POINTER(C.c_float)), C.c_int, C.POINTER(OObs),
                                C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(lib.LocResult)]
    host = [f.cpu().numpy().reshape(-1) for f in fields]
    fp = (C.POINTER(C.c_float) * ns)(*[h.ctypes.data_as(C.POINTER(C.c_float)) for h in host])
    cores = os.cpu_count() or 1
    sample = list(range(min(E, cores)))

    def one(e):
        ob = events[e]
        arr = (OObs * len(ob))(*[OObs(f, t, w, ph.encode(), gd) for f, t, w, ph, gd in ob])
        rm = (C.c_float * len(ob))()
        tp = (C.c_float * len(ob))()
        r = lib.LocResult()
        olib.fdo_locate(C.byref(grid), fp, len(ob), arr, rm, tp, C.byref(r))
        return r, list(rm), [a.good for a in arr]

    t0 = time.time()
    with ThreadPoolExecutor(cores) as ex:
        cpu = list(ex.map(one, sample))
    cpu_s = time.time() - t0
    mism = 0
    for e, (r, rm, gd) in zip(sample, cpu):
        a = res[e]
        if (a["status"], a["nxx"], a["nyy"], a["nzz"], a["passes"], a["exm"], a["eym"], a["ezm"], a["stdmin"],
                a["avrmin"]) != (r.status, r.nxx, r.nyy, r.nzz, r.passes, r.exm, r.eym, r.ezm, r.stdmin, r.avrmin) \
                or np.asarray(a["resmin"], np.float32).tobytes() != np.asarray(rm, np.float32).tobytes() \
                or list(a["good"]) != gd:
            mism += 1
    return {"events": E, "phases": nobs, "fields": ns, "grid": [g.nx, g.ny, g.nz],
            "events_per_s": E / gpu_s, "wall_s": gpu_s,
            "accepted": sum(1 for r in res if r["status"] == 0),
            "passes_mean": sum(r["passes"] for r in res) / E,
            "cpu_baseline": {"events_per_s": len(sample) / cpu_s, "cores": len(sample), "kind": "port",
                             "sample": f"{len(sample)} of the {E} events, the location oracle, one event per host thread"},
            "parity": {"events_checked": len(sample), "events_differing": mism, "bit_identical": mism == 0},
            "what": "sphfdloc grid search (node search, two refinements, outlier passes) per event"}


def ray_leg(args, lib, ctx, g, sts, fields, stream):
    """sphrayderv's rays (fdgpu_raytrace) through the batch step's 64 P fields still on the device:
    args.ray_events synthetic events at random points inside the grid, each observed at 24-40 of the
    stations, on a 21x21x17 coarse metagrid (every 10th node across, every 5th down).  Timed through
    the public call (observations in from host memory, residuals, hypocentre derivatives and packed
    coarse derivatives out).  CPU baseline: the ray oracle with the C library's trig functions (as
    the reference's sphrayderv) on the host cores for a sample of the events; the same sample traced
    with the oracle's double-double trig is compared with the GPU's results bit for bit."""
    import ctypes as C
    from concurrent.futures import ThreadPoolExecutor
    import numpy as np
    import torch
    from fdtomoc_gb300 import rayderv as R
    E = args.ray_events
    sp = dict(nxc=21, nyc=21, nzc=17, igridx=[10] * 20, igridy=[10] * 20, igridz=[5] * 16, h=g.h, x0=g.x0, y0=g.y0,
              z0=g.z0, dq=g.dlat, df=g.dlon)
    assert 1 + sum(sp["igridx"]) == g.nx and 1 + sum(sp["igridy"]) == g.ny and 1 + sum(sp["igridz"]) == g.nz
    grid, keep = R.grid_from_spec(sp, spacing_rule=False)   # the fields' own 0.005-degree spacing
    st = [dict(xs=float(np.float32(s["lon"] * R.DEGRAD)), ys=float(np.float32(R.HPI - R.glat(s["lat"] * R.DEGRAD))),
               zs=float(-np.float32(s["elev"]))) for s in sts[:len(fields)]]
    rng = np.random.default_rng(11)
    ns = len(fields)
    obs = []
    bounds = []
    for e in range(E):
        bounds.append(len(obs))
        ex = grid.x0 + grid.df * rng.uniform(5, g.nx - 6)
        ey = grid.y0 + grid.dq * rng.uniform(5, g.ny - 6)
        ez = grid.z0 + grid.h * rng.uniform(6, g.nz - 6)
        for k in rng.choice(ns, size=int(rng.integers(24, 41)), replace=False):
            w = np.float32(rng.choice([0.05, 0.1, 0.2]))
            obs.append(R.RayObs(ex, ey, ez, st[k]["xs"], st[k]["ys"], st[k]["zs"], int(k), 0,
                                float(np.float32(rng.uniform(5, 40))), float(np.float32(1.0) / (w * w)),
                                float(np.float32(0.0)), 0))
    nobs = len(obs)
    bounds = [(bounds[e], bounds[e + 1] if e + 1 < E else nobs) for e in range(E)]
    arr = (R.RayObs * nobs)(*obs)
    ptrs = [f.data_ptr() for f in fields]
    cap = R.default_cap(grid)
    lib.raytrace(ctx, grid, ptrs, arr, min(nobs, 256), cap=cap, stream_ptr=stream.cuda_stream)   # warm-up
    torch.cuda.synchronize()
    reps = 3
    t0 = time.time()
    for _ in range(reps):
        got = lib.raytrace(ctx, grid, ptrs, arr, nobs, cap=cap, stream_ptr=stream.cuda_stream)
    gpu_s = (time.time() - t0) / reps
    res = got[0]
    segs = sum(res[o].nseg for o in range(nobs))
    ok = sum(1 for o in range(nobs) if res[o].status == R.RAY_OK)

    # CPU: the oracle, a sample of events, one event's rays per host thread
    build_oracle()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_util import oracle_trace
    host = [f.cpu().numpy().reshape(-1) for f in fields]
    cores = os.cpu_count() or 1
    sample = bounds[:min(E, 2 * cores)]

    def one(b, mode):
        a = (R.RayObs * (b[1] - b[0]))(*[arr[i] for i in range(b[0], b[1])])
        return oracle_trace(mode)(grid, host, a, b[1] - b[0], cap)

    t0 = time.time()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda b: one(b, 0), sample))
    cpu_s = time.time() - t0
    with ThreadPoolExecutor(cores) as ex:
        exact = list(ex.map(lambda b: one(b, 1), sample))
    mism = 0
    for b, (rr, off, idx, du) in zip(sample, exact):
        for i in range(b[1] - b[0]):
            x, y = res[b[0] + i], rr[i]
            a0, a1 = got[1][b[0] + i], got[1][b[0] + i + 1]
            if (x.status, x.nseg, x.nnz, x.dt, bytes(x.am)) != (y.status, y.nseg, y.nnz, y.dt, bytes(y.am)) or \
                    not np.array_equal(got[2][a0:a1], idx[off[i]:off[i + 1]]) or \
                    got[3][a0:a1].tobytes() != du[off[i]:off[i + 1]].tobytes():
                mism += 1
    nsample = sum(b[1] - b[0] for b in sample)
    del keep
    return {"events": E, "rays": nobs, "fields": ns, "grid": [g.nx, g.ny, g.nz], "coarse": [21, 21, 17],
            "rays_per_s": nobs / gpu_s, "wall_s": gpu_s, "reached_station": ok, "segments": segs,
            "nonzero_derivatives": int(got[1][nobs]),
            "cpu_baseline": {"rays_per_s": nsample / cpu_s, "cores": min(cores, len(sample)), "kind": "port",
                             "sample": f"{len(sample)} of the {E} events ({nsample} rays), the ray oracle with the "
                                       f"C library's trig, one event per host thread"},
            "parity": {"rays_checked": nsample, "rays_differing": mism, "bit_identical": mism == 0},
            "what": "sphrayderv per observation: residual, hypocentre derivatives, ray back-trace, coarse "
                    "slowness derivatives"}


def c2f_leg(args, lib, ctx, stream):
    """c2f (coarse-to-fine model) on the device: a 41x41x33 coarse P/S model onto the 401x401x161 fine
    grid of the largest workload (25.9 M fine nodes per phase), through a plan (tables built once, as
    an inversion loop reuses them), timed with CUDA events over repeated runs on its stream.  The
    interpolation kernel writes 8 bytes per fine node (P and S) and reads a coarse model held in L2:
    its roofline is HBM writes.  CPU baseline: the c2f oracle on one core (the reference's c2f is
    single-threaded), and the GPU result's digest against the oracle's."""
    import ctypes as C
    import hashlib
    import numpy as np
    import torch
    nxc, nyc, nzc = 41, 41, 33
    ig = dict(igridx=[10] * (nxc - 1), igridy=[10] * (nyc - 1), igridz=[5] * (nzc - 1))
    x0, y0, z0, h = -100.0, -100.0, -2.0, 0.5
    rng = np.random.default_rng(5)
    k, j, i = np.meshgrid(np.arange(nzc, dtype=np.float64), np.arange(nyc, dtype=np.float64),
                          np.arange(nxc, dtype=np.float64), indexing="ij")
    vp = 5.0 + 0.1 * k + 0.2 * rng.random((nzc, nyc, nxc))
    coarse = np.stack([vp, vp / 1.73]).astype(np.float32)
    plan = lib.C2fPlan(ctx, nxc, nyc, nzc, ig["igridx"], ig["igridy"], ig["igridz"], x0, y0, z0, h)
    src = torch.from_numpy(coarse).cuda()
    out = torch.empty(plan.shape, dtype=torch.float32, device="cuda")
    nfine = out.numel() // 2
    for _ in range(3):
        plan.run(src.data_ptr(), out.data_ptr(), stream.cuda_stream)
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        plan.run(src.data_ptr(), out.data_ptr(), stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    plan.close()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    algo = 8.0 * nfine
    gbs = algo / (ms * 1e-3) / 1e9
    # CPU: the oracle on one core, and the digests
    build_oracle()
    olib = C.CDLL(os.path.join(ROOT, "oracle", "liboracle.so"))

    class G(C.Structure):
        _fields_ = lib.C2fGrid._fields_
    olib.fdo_c2f.argtypes = [C.POINTER(G), C.POINTER(C.c_float), C.POINTER(C.c_float)]
    arrs = [(C.c_int * len(ig[key]))(*ig[key]) for key in ("igridx", "igridy", "igridz")]
    grid = G(nxc, nyc, nzc, *arrs, x0, y0, z0, h)
    fine = np.empty(plan.shape, np.float32)
    t0 = time.time()
    olib.fdo_c2f(C.byref(grid), coarse.ctypes.data_as(C.POINTER(C.c_float)), fine.ctypes.data_as(C.POINTER(C.c_float)))
    cpu_s = time.time() - t0
    same = hashlib.sha256(out.cpu().numpy().tobytes()).hexdigest() == hashlib.sha256(fine.tobytes()).hexdigest()
    return {"coarse": [nxc, nyc, nzc], "fine": list(plan.shape[:0:-1]), "ms_per_model": ms,
            "fine_nodes_per_s": 2 * nfine / (ms * 1e-3),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "algorithmic_bytes": algo, "note": "writes of the P and S fine models; the coarse model stays in L2"},
            "cpu_baseline": {"ms_per_model": cpu_s * 1e3, "cores": 1, "kind": "port",
                             "sample": "the whole model, the c2f oracle on one core"},
            "parity": {"bit_identical": same},
            "what": "c2f: coarse P/S velocities to the fine model sphfd reads, plan reused (fdgpu_c2f_run)"}


def profile_legs(args):
    """--profile-legs: a small fixed case of the c2f and location kernels for ncu captures (no timing,
    no JSON line): c2f 41x41x33 -> 401x401x161 three times through a plan, then 32 events of 30 picks
    located against 64 synthetic 201x201x81 fields (straight-ray times from surface stations)."""
    import numpy as np
    import torch
    from fdtomoc_gb300 import build, lib as L
    build.build()
    ctx = L.Context(0)
    nxc, nyc, nzc = 41, 41, 33
    plan = L.C2fPlan(ctx, nxc, nyc, nzc, [10] * 40, [10] * 40, [5] * 32, -100.0, -100.0, -2.0, 0.5)
    rng = np.random.default_rng(5)
    vp = (5.0 + 0.2 * rng.random((nzc, nyc, nxc))).astype(np.float32)
    src = torch.from_numpy(np.stack([vp, vp / 1.73]).astype(np.float32)).cuda()
    out = torch.empty(plan.shape, dtype=torch.float32, device="cuda")
    for _ in range(3):
        plan.run(src.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    plan.close()
    del out
    nx, ny, nz = 201, 201, 81
    k, j, i = torch.meshgrid(torch.arange(nz, device="cuda", dtype=torch.float32),
                             torch.arange(ny, device="cuda", dtype=torch.float32),
                             torch.arange(nx, device="cuda", dtype=torch.float32), indexing="ij")
    st = rng.integers(0, 201, (64, 2))
    fields = [(torch.sqrt(((i - float(st[s_, 0])) * 0.5) ** 2 + ((j - float(st[s_, 1])) * 0.55) ** 2 + (k * 0.5) ** 2)
               / 6.0).contiguous() for s_ in range(64)]
    grid = L.loc_grid_from_spec(nx, ny, nz, 120.5, 23.5, -2.0, 0.5)
    hyp = np.stack([rng.integers(0, nx, 32), rng.integers(0, ny, 32), rng.integers(2, nz, 32)], 1)
    events = []
    for e in range(32):
        ob = []
        for s_ in rng.choice(64, 30, replace=False):
            t = float(fields[s_][hyp[e, 2], hyp[e, 1], hyp[e, 0]].item()) + 5.0 + float(rng.normal(0, 0.02))
            ob.append((int(s_), float(np.float32(t)), 100.0, "P", 1))
        events.append(ob)
    res = L.locate(ctx, grid, [f.data_ptr() for f in fields], events)
    torch.cuda.synchronize()
    print("profile case done:", sum(r["status"] == 0 for r in res), "of", len(res), "events accepted")
    ctx.close()


HEADLINE = os.path.join(ROOT, "tests", "golden", "headline_reference.json")
C3_METRIC = "station fields/s (500 uneven windows in one launch, bit-identical to reference)"
C3_WORKLOAD = "500 windows 41..301 x 41..301 x 41..121 over a 401x401x161 model, 0.005deg x 0.005deg x 0.5km (config 3)"
CPU_WINDOW_MAX_S = 6.0   # windows in the CPU sample: at most this many oracle seconds each on the x86 build host


def headline_fixture():
    """Reference-binary pins of the config-2 stations and config-3 windows (make_headline_golden.py)."""
    return json.load(open(HEADLINE)) if os.path.exists(HEADLINE) else None


def field_sha(t) -> str:
    import hashlib
    return hashlib.sha256(t.cpu().numpy().tobytes()).hexdigest()


def config3_case(rank: int):
    """The config-3 model, this rank's windows (rank 0: the benchmark's 500; rank r > 0: its own 500,
    seed 3 + 1000 r) and a directory with their par files."""
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_par
    g, v, _ = W.config(3)
    wins = W.config3_windows(500, 3 + 1000 * rank)
    case_dir = tempfile.mkdtemp(prefix=f"fdbench_c3_r{rank}_")
    velfile = os.path.join(case_dir, "vp.mod")
    pars = []
    for w in wins:
        pf = os.path.join(case_dir, w["name"] + ".par")
        write_par(pf, W.window_par(g, w, velfile, w["name"] + ".ptimes"))
        pars.append(pf)
    return g, v, wins, case_dir, pars


def cpu_windows(g, v, wins, names, case_dir, cores):
    """The oracle (exact pruned mode) on the named windows, one process per core, each window with its
    own velocity file cut from the model where the GPU reads it.  Returns {name: (seconds, node
    updates)} and the output directory."""
    import numpy as np
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_grid, write_par
    exe = build_oracle()
    out = os.path.join(case_dir, "cpu_out")
    os.makedirs(out, exist_ok=True)
    by = {w["name"]: w for w in wins}
    env = dict(os.environ, FDO_MODE="fast", OMP_NUM_THREADS="1")
    pending, running, res = list(names), [], {}
    while pending or running:
        while pending and len(running) < cores:
            nm = pending.pop(0)
            w = by[nm]
            wg = W.Grid(w["nx"], w["ny"], w["nz"], g.dlon, g.dlat, g.h, x0=g.x0 + w["ox"] * g.dlon,
                        y0=g.y0 - w["oy"] * g.dlat, z0=g.z0)
            wf = os.path.join(case_dir, nm + ".mod")
            write_grid(wf, W.head_for(wg), np.ascontiguousarray(v[:w["nz"], w["oy"]:w["oy"] + w["ny"],
                                                                  w["ox"]:w["ox"] + w["nx"]]))
            pf = os.path.join(case_dir, nm + ".cpu.par")
            write_par(pf, W.window_par(g, w, wf, nm + ".ptimes"))
            pl = os.path.join(case_dir, f"pl_{nm}")
            with open(pl, "w") as f:
                f.write(f"par={pf}\n")
            spec = os.path.join(case_dir, f"spec_{nm}")
            with open(spec, "w") as f:
                f.write(f"parlist {pl}\ntimedir {out}\n")
            p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                                 text=True, env=env)
            p.stdin.write(spec + "\n")
            p.stdin.close()
            running.append((nm, p, time.time()))
        time.sleep(0.01)
        still = []
        for nm, p, t0 in running:
            if p.poll() is None:
                still.append((nm, p, t0))
                continue
            dt = time.time() - t0
            log = p.stderr.read()
            if p.returncode != 0:
                raise RuntimeError(f"oracle failed on {nm}: {log}")
            nu = 0
            for tok in log.split():
                if tok.startswith("node_updates="):
                    nu = int(tok.split("=")[1])
            res[nm] = (dt, nu)
            os.remove(os.path.join(case_dir, nm + ".mod"))
        running = still
    return res, out


def cpu_sample_names(wins, fix, cores, step):
    """A seeded sample of `cores` windows for CPU step `step`: windows taken in a seeded permutation of
    the 500, keeping those the oracle solved in at most CPU_WINDOW_MAX_S on the x86 build host (so a
    step stays short), consecutive slices for consecutive steps."""
    import numpy as np
    perm = np.random.default_rng(31).permutation(len(wins))
    ok = [wins[k]["name"] for k in perm
          if fix is None or fix["config3"][wins[k]["name"]]["oracle_s"] <= CPU_WINDOW_MAX_S]
    start = (step * cores) % max(1, len(ok) - cores + 1)
    return ok[start:start + cores]


def cpu_estimate(res, fix, cores):
    """Whole-workload CPU fields/s from a sample: node updates per core-second over the sample, times
    the cores, divided by the mean node updates of a window over all 500 windows (from the fixture)."""
    nu = sum(x[1] for x in res.values())
    sec = sum(x[0] for x in res.values())
    mean_nu = (sum(x["node_updates"] for x in fix["config3"].values()) / len(fix["config3"])) if fix else nu / len(res)
    return cores * (nu / sec) / mean_nu, nu / sec, mean_nu


def run_config3(args):
    """The benchmark (default): the 500 uneven windows of config 3 over the 401x401x161 model, solved
    as one prepared batch (fdgpu_batch_*: one kernel launch per step, capturable), launch order
    tuned by the first warm-up run's measured solve times.  Parity: every window's field is hashed and
    compared with the reference binary's (tests/golden/headline_reference.json).  Also: the plain form
    (one window per launch, a seeded sample), the same workload end to end through the host-buffer
    entry point, an extrapolated CPU baseline, the roofline, and the config-2 legs (64 stations of
    201x201x81 and the neighbours' kernels on their fields)."""
    import numpy as np
    rank, world, local = dist_env()
    fix = headline_fixture() if rank == 0 else None
    g, v, wins, case_dir, pars = config3_case(rank)
    ncores = os.cpu_count() or 1
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        names = cpu_sample_names(wins, fix, ncores, 0)
        t0 = time.time()
        res, cpu_out = cpu_windows(g, v, wins, names, case_dir, ncores)
        wall = time.time() - t0
        est, rate, mean_nu = cpu_estimate(res, fix, ncores)
        ora_ok = None
        if fix:
            ora_ok = sum(hashlib_file(os.path.join(cpu_out, nm + ".ptimes")) == fix["config3"][nm]["data_sha256"]
                         for nm in names)
        cpu = {"value": est, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": f"{len(names)} seeded windows of the 500 (oracle FAST mode, one process per core, "
                         f"{wall:.1f} s wall): {rate / 1e6:.3f} M node updates per core-second, extrapolated to "
                         f"the workload's mean of {mean_nu / 1e6:.2f} M node updates per window",
               "node_updates_per_s": rate * ncores, "extrapolated": True,
               "sample_equal_reference": None if ora_ok is None else f"{ora_ok}/{len(names)}"}
    import torch
    from fdtomoc_gb300 import build, lib
    build.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stations = []
    for w, pf in zip(wins, pars):
        st = lib.station_from_par("par=" + pf)[0]
        st.ox, st.oy, st.oz = w["ox"], w["oy"], 0
        stations.append(st)
    sizes = [w["nx"] * w["ny"] * w["nz"] for w in wins]
    ctx = lib.Context(local)
    stream = torch.cuda.Stream()
    vel_d = torch.from_numpy(v.reshape(-1)).cuda()
    slow = torch.empty_like(vel_d)
    ctx.velocity_to_slowness(vel_d.data_ptr(), slow.data_ptr(), v.size, stream.cuda_stream)
    stream.synchronize()
    del vel_d
    fields = [torch.empty(st.shape, dtype=torch.float32, device="cuda") for st in stations]
    batch = lib.Batch(ctx, stations, slow.data_ptr(), g.nx, g.nx * g.ny, [f.data_ptr() for f in fields])
    tuned = False
    for k in range(args.warmup):
        batch.run(stream.cuda_stream)
        if k == 0:
            # longest measured solve first from here on, tuned on the first run (launched largest grid
            # first) and kept: over nine runs on several boxes 21.4 - 23.5 s per step; re-tuning after
            # every run oscillated (22.3 - 25.7 s), tuning twice gave 22.4 s on one box and 25.5 s on
            # another
            batch.tune_order(stream.cuda_stream)
            tuned = True
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    e0.record(stream)
    for _ in range(args.steps):
        batch.run(stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    stats = batch.stats(stream.cuda_stream)
    nu = sum(s_["node_updates"] for s_ in stats)
    t_first = min(x["t_start_ns"] for x in stats)
    done = sorted((s_["t_end_ns"] - t_first) / 1e6 for s_ in stats)
    # parity: every field against the reference binary's
    parity = None
    if fix:
        same = sum(field_sha(f) == fix["config3"][w["name"]]["data_sha256"] for f, w in zip(fields, wins))
        sweeps_same = sum(s_["sweeps"] == fix["config3"][w["name"]]["sweeps"] for s_, w in zip(stats, wins))
        model_same = hashlib_bytes(np.ascontiguousarray(v, dtype="<f4").tobytes()) == fix["models"]["config3"]
        parity = {"windows_bit_identical_to_reference": f"{same}/{len(wins)}",
                  "sweep_counts_equal_reference": f"{sweeps_same}/{len(wins)}", "model_equal_pinned": model_same,
                  "against": "SHA-256 of the reference binary's time files (tests/golden/headline_reference.json)"}
    # plain form: one window per launch, a seeded sample
    rng = np.random.default_rng(33)
    sample = [int(k) for k in rng.choice(len(wins), 8, replace=False)]
    plain_ms, plain_same = [], 0
    for k in sample:
        out = torch.empty_like(fields[k])
        e0.record(stream)
        ctx.solve_device([stations[k]], slow.data_ptr(), g.nx, g.nx * g.ny, [out.data_ptr()],
                         stream_ptr=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
        plain_same += int(torch.equal(out, fields[k]))
    plain_fps = 1e3 / (sum(plain_ms) / len(plain_ms))
    value = len(wins) * world / (ms_step / 1e3)
    # end to end through the host-buffer entry point: the velocity model in from pinned memory, the
    # 500 fields out to pinned memory, every step
    import ctypes as C
    L = lib.load()
    vel_h = torch.from_numpy(v.reshape(-1).copy()).pin_memory()
    outs_h = [torch.empty(st.shape, dtype=torch.float32).pin_memory() for st in stations]
    arr = (lib.Station * len(stations))(*stations)
    outp = (C.POINTER(C.c_float) * len(stations))(*[C.cast(o.data_ptr(), C.POINTER(C.c_float)) for o in outs_h])
    del fields
    batch.close()
    torch.cuda.synchronize()
    t0 = time.time()
    rc = L.fdgpu_solve_host(ctx.ptr, len(stations), arr, C.cast(vel_h.data_ptr(), C.POINTER(C.c_float)), g.nx,
                            g.ny, g.nz, outp, None, None)
    e2e_s = time.time() - t0
    if rc != 0:
        raise RuntimeError(f"fdgpu_solve_host failed: {rc}")
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_same = None
    if fix:
        e2e_same = sum(hashlib_bytes(o.numpy().tobytes()) == fix["config3"][w["name"]]["data_sha256"]
                       for o, w in zip(outs_h, wins))
    e2e = {"value": len(wins) * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(v.size * 4),
           "d2h_bytes_per_step": int(sum(o.numel() * 4 for o in outs_h)), "steps": 1,
           "launch_order": "longest measured solve first (the context's order table, filled by the batch's runs)",
           "windows_bit_identical_to_reference": None if e2e_same is None else f"{e2e_same}/{len(wins)}"}
    del outs_h, vel_h
    # the config-2 legs: 64 stations of 201x201x81 in one launch, and the neighbours on their fields
    c2 = config2_legs(args, lib, ctx, stream, fix) if rank == 0 and not args.no_config2 else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = ALGO_BYTES_PER_NODE_UPDATE * nu / (ms_step / 1e3) / 1e9
    traffic = None
    traffic_note = None
    tpath = os.path.join(ROOT, "profiles", "fd_solve_traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath))
        traffic = tj["dram_bytes_per_node_update"] * nu
        traffic_note = (f"{tj['dram_bytes_per_node_update']} DRAM B per node update from an ncu capture of "
                        f"{tj['workload']}, scaled to this launch's node updates; a lower bound here: "
                        f"{tj['scaling_note']}")
    st_sum = [sum(s_["stencils"][k] for s_ in stats) for k in range(5)]
    fp64_ops = 116 * st_sum[0] + 70 * st_sum[1] + 69 * st_sum[2] + 25 * st_sum[3] + 6 * st_sum[4]
    fp64_peak = ctx.probe_fp64_gops()
    if rank == 0:
        line = {
            "metric": C3_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 stencils / f32 fields", "data": "synthetic (seeded, config 3 recipe)",
            "config": {"workload": C3_WORKLOAD, "windows_per_gpu": len(wins), "nodes_per_gpu": int(sum(sizes)),
                       "launch": "one prepared batch (fdgpu_batch_run), one kernel per step",
                       "launch_order": "longest measured solve first (tuned on the first warm-up run)" if tuned
                       else "largest grid first",
                       "l2": "inputs larger than L2 (500 fields, 4.7 GB, + 104 MB model)",
                       "parallelism": f"windows x{world}"},
            "node_updates_per_s": nu * world / (ms_step / 1e3),
            "latency_ms": {"p50": done[len(done) // 2], "p99": done[min(len(done) - 1, int(round(0.99 * (len(done) - 1))))],
                           "what": "window completion time within the step"},
            "plain": {"sample_windows": len(sample), "ms_per_window_mean": sum(plain_ms) / len(plain_ms),
                      "fields_per_s": plain_fps, "batched_over_plain": value / world / plain_fps,
                      "sample_equal_batch": f"{plain_same}/{len(sample)}"},
            "e2e": e2e,
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "traffic_note": traffic_note,
                         "peak_kind": "of measured (MEASURED_PEAKS.json hbm_gbs)",
                         "note": "the path is bound by FP64 issue and dependency latency, not HBM"},
            "fp64": {"achieved_gops": fp64_ops / (ms_step / 1e3) / 1e9, "peak_gops": fp64_peak,
                     "frac": fp64_ops / (ms_step / 1e3) / 1e9 / fp64_peak,
                     "peak_kind": "measured live (FP64 fused multiply-add chains, all SMs)"},
            "parity": parity,
            "clocks": clocks,
        }
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if c2 is not None:
            line["config2"] = c2
        print(json.dumps(line), flush=True)
    ctx.close()
    shutil.rmtree(case_dir, ignore_errors=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def hashlib_bytes(b: bytes) -> str:
    import hashlib
    return hashlib.sha256(b).hexdigest()


def hashlib_file(path: str) -> str:
    return hashlib_bytes(open(path, "rb").read()[232:])


def config2_legs(args, lib, ctx, stream, fix):
    """64 stations of config 2 in one launch (timed once, fields hashed against the reference's), then
    the location, c2f, ray and serving legs on those fields."""
    import torch
    g, v, sts = workload(0, STATIONS_PER_GPU, 2)
    case_dir = tempfile.mkdtemp(prefix="fdbench_c2_")
    write_case(case_dir, g, v, sts)
    stations = [lib.station_from_par("par=" + os.path.join(case_dir, s["name"] + ".par"))[0] for s in sts]
    vel_d = torch.from_numpy(v.reshape(-1)).cuda()
    slow = torch.empty_like(vel_d)
    ctx.velocity_to_slowness(vel_d.data_ptr(), slow.data_ptr(), v.size, stream.cuda_stream)
    fields = [torch.empty(s.shape, dtype=torch.float32, device="cuda") for s in stations]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    stats = ctx.solve_device(stations, slow.data_ptr(), g.nx, g.nx * g.ny, [f.data_ptr() for f in fields],
                             stream_ptr=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    out = {"workload": CONFIG_NAME, "fields_per_s": len(stations) / (ms / 1e3), "ms_per_step": ms,
           "node_updates_per_s": sum(s_["node_updates"] for s_ in stats) / (ms / 1e3), "steps": 1}
    if fix:
        same = sum(field_sha(f) == fix["config2"][s["name"]]["data_sha256"] for f, s in zip(fields, sts))
        out["stations_bit_identical_to_reference"] = f"{same}/{len(sts)}"
    # one station alone: the latency of a single 201x201x81 solve
    e0.record(stream)
    ctx.solve_device(stations[:1], slow.data_ptr(), g.nx, g.nx * g.ny, [fields[0].data_ptr()],
                     stream_ptr=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    out["single_station_ms"] = e0.elapsed_time(e1)
    if args.locate_events > 0:
        out["locate"] = locate_leg(args, lib, ctx, g, fields, stream)
    if not args.no_c2f:
        out["c2f"] = c2f_leg(args, lib, ctx, stream)
    if args.ray_events > 0:
        out["rays"] = ray_leg(args, lib, ctx, g, sts, fields, stream)
    profiled = under_profiler()
    if args.serve_requests > 0 and not profiled:
        out["serving"] = serve_leg(args, lib, stations, v, fields)
    shutil.rmtree(case_dir, ignore_errors=True)
    return out


def run_reference_config3(args):
    """Reference arm on the config-3 workload: the CPU restatement of the reference's solver (oracle/,
    pinned bit for bit against the reference binary; the reference's own sources do not exist on the
    GPU host) on all host cores, one process per core as the reference's OpenMP driver runs par files.
    Each step solves a seeded sample of one window per core (consecutive slices of a seeded
    permutation, windows of at most CPU_WINDOW_MAX_S oracle seconds so that a step stays short); the
    reported fields/s extrapolates the node updates per core-second to the workload's mean window."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    fix = headline_fixture()
    g, v, wins, case_dir, _ = config3_case(0)
    ncores = os.cpu_count() or 1
    for k in range(args.warmup):
        cpu_windows(g, v, wins, cpu_sample_names(wins, fix, ncores, 1000 + k)[:1], case_dir, 1)
    res_all, walls = {}, []
    for k in range(args.steps):
        t0 = time.time()
        res, _ = cpu_windows(g, v, wins, cpu_sample_names(wins, fix, ncores, k), case_dir, ncores)
        walls.append(time.time() - t0)
        res_all.update({f"{k}:{n}": x for n, x in res.items()})
    est, rate, mean_nu = cpu_estimate(res_all, fix, ncores)
    line = {
        "impl": "reference", "metric": C3_METRIC, "value": est, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(walls) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 stencils / f32 fields",
        "data": "synthetic (seeded, config 3 recipe)",
        "config": {"workload": C3_WORKLOAD, "parallelism": f"{ncores} processes x 1 thread"},
        "node_updates_per_s": rate * ncores,
        "cpu_baseline": {"value": est, "unit": UNIT, "cores": ncores, "kind": "port", "extrapolated": True,
                         "sample": f"{ncores} seeded windows per step (oracle FAST mode, exact), "
                                   f"{rate / 1e6:.3f} M node updates per core-second, extrapolated to the workload's "
                                   f"mean of {mean_nu / 1e6:.2f} M node updates per window"},
        "e2e": {"value": est, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    shutil.rmtree(case_dir, ignore_errors=True)


def run_config5(args):
    """--config 5: stations on the full 401x401x161 grid with a dipping fast slab (1200 stations, seed
    5; args.stations of them, the pinned sample first), served by a serving session whose fields stay
    on the device up to a budget (args.field_budget fields) and are spilled to pinned host memory
    beyond it (fdtomoc_gb300.fieldstore).  Against the plain form (one station per launch) and, for the
    pinned sample, against the reference binary's fields.  Prints one JSON line."""
    import numpy as np
    import torch
    from fdtomoc_gb300 import build, lib, workloads as W
    from fdtomoc_gb300.fieldstore import FieldStore
    fix = headline_fixture()
    g, v, sts = W.config(5)
    pinned = sorted(fix["config5"]) if fix and "config5" in fix else []
    names = pinned + [s["name"] for s in sts if s["name"] not in pinned]
    names = names[:max(1, args.stations)]
    by = {s["name"]: s for s in sts}
    case_dir = tempfile.mkdtemp(prefix="fdbench_c5_")
    W.write_case(case_dir, g, v, [by[n] for n in names])
    build.build()
    stations = [lib.station_from_par("par=" + os.path.join(case_dir, n + ".par"))[0] for n in names]
    field_bytes = 4 * g.nx * g.ny * g.nz
    with lib.Server(0, hbm_bytes=args.session_gb << 30) as sv:
        sv.set_model(0, v)
        store = FieldStore(sv, args.field_budget * field_bytes)
        t0 = time.time()
        for n, st in zip(names, stations):
            store.submit(n, st, 0)
            store.poll(64, 0)
        store.drain(3600000)
        wall = time.time() - t0
        m = sv.metrics()
        failed = sum(r["status"] != 0 for r in store.results.values())
        resident = sum(store.where(n) == "device" for n in names)
        same = None
        if pinned:
            ok = 0
            for n in pinned:
                f = store.get(n)
                ok += hashlib_bytes((f.cpu() if f.is_cuda else f).numpy().tobytes()) == fix["config5"][n]["data_sha256"]
            same = f"{ok}/{len(pinned)}"
        spilled, direct = store.spilled, store.direct_to_host
        del store
    # plain form: one station per launch
    with lib.Context(0) as ctx:
        vel = torch.from_numpy(v.reshape(-1)).cuda()
        slow = torch.empty_like(vel)
        ctx.velocity_to_slowness(vel.data_ptr(), slow.data_ptr(), v.size)
        # the pinned station with the fewest sweeps (full-grid solves with many restarts take minutes)
        kp = min(range(len(pinned)), key=lambda k: fix["config5"][pinned[k]]["sweeps"]) if pinned else 0
        out = torch.empty(stations[kp].shape, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        tp = time.time()
        (ps,) = ctx.solve_device([stations[kp]], slow.data_ptr(), g.nx, g.nx * g.ny, [out.data_ptr()])
        plain_s = time.time() - tp
        plain_nu = ps["node_updates"]
    value = len(names) / wall
    line = {
        "metric": "station fields/s served on the full 401x401x161 grid, fields device-resident up to a budget "
                  "then spilled to pinned host memory, bit-identical to reference",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 stencils / f32 fields",
        "data": "synthetic (seeded, config 5 recipe)",
        "config": {"workload": f"{len(names)} of the 1200 stations on 401x401x161 with a 30-degree dipping +8 % slab "
                               "(config 5)", "field_budget_fields": args.field_budget,
                   "session_hbm_gb": args.session_gb},
        "fields": {"device_resident": resident, "spilled_to_host": spilled, "solved_into_host": direct,
                   "bytes_each": field_bytes},
        "latency_ms": {"p50": m["p50_ms"], "p99": m["p99_ms"], "max": m["max_ms"]},
        "solve_ms": {"p50": m["solve_p50_ms"], "p99": m["solve_p99_ms"]},
        "node_updates_per_s": m["node_updates"] / wall, "failed": failed, "hbm_peak_bytes": m["hbm_peak"],
        "plain": {"station": names[kp], "s_per_station": plain_s, "node_updates": plain_nu,
                  "node_updates_per_s": plain_nu / plain_s,
                  "served_node_updates_over_plain": (m["node_updates"] / wall) / (plain_nu / plain_s),
                  "note": "stations here differ by up to 4x in sweeps, so node updates/s compare the forms"},
        "parity": {"pinned_stations_bit_identical_to_reference": same,
                   "against": "SHA-256 of the reference binary's time files for a seeded sample"},
        "gpu_launches": m["grid_launches"] + 1,
    }
    print(json.dumps(line), flush=True)
    shutil.rmtree(case_dir, ignore_errors=True)



def run_config4(args):
    """--config 4: served P and S solves.  Requests (station window, phase) drawn from 800 windows
    (61..301 x 61..301 x 61..121 over the 401x401x161 model, seed 4) arrive as a seeded Poisson stream
    (args.rate per second); S = P/1.73 with an independent 2 % perturbation; every 100 requests both
    models are replaced by a 1 % smooth perturbation of themselves, as an inversion iteration would.
    Reports throughput, latency percentiles and, for a sample of requests, bit equality with the same
    station solved alone against the model version it was served with.  Prints one JSON line."""
    import numpy as np
    import torch
    from fdtomoc_gb300 import build, lib, workloads as W
    from fdtomoc_gb300.formats import write_par
    g, vp, _ = W.config(3)
    vs = (vp / 1.73 * (1.0 + 0.02 * W.smooth_noise(vp.shape, (g.h, 0.556, 0.509), 10.0, 41))).astype(np.float32)
    rng = np.random.default_rng(4)
    wins = []
    for i in range(800):
        wx, wy, wz = int(rng.integers(61, 302)), int(rng.integers(61, 302)), int(rng.integers(61, 122))
        ox, oy = int(rng.integers(0, 401 - wx + 1)), int(rng.integers(0, 401 - wy + 1))
        wins.append(dict(name=f"R{i:04d}", nx=wx, ny=wy, nz=wz, ox=ox, oy=oy, fx=float(rng.uniform(2, wx - 3)),
                         fy=float(rng.uniform(2, wy - 3)), elev=float(rng.uniform(0, 2))))
    case_dir = tempfile.mkdtemp(prefix="fdbench_c4_")
    build.build()
    stations = []
    for w in wins:
        pf = os.path.join(case_dir, w["name"] + ".par")
        write_par(pf, W.window_par(g, w, os.path.join(case_dir, "vp.mod"), w["name"] + ".ptimes"))
        st = lib.station_from_par("par=" + pf)[0]
        st.ox, st.oy, st.oz = w["ox"], w["oy"], 0
        stations.append(st)
    n = args.serve_requests
    picks = [(int(rng.integers(0, 800)), int(rng.integers(0, 2))) for _ in range(n)]
    gaps = rng.exponential(1.0 / args.rate, n)
    # the model versions, made before the clock starts
    versions = {0: [vp], 1: [vs]}
    for q in range(100, n, 100):
        for m_ in (0, 1):
            pert = W.smooth_noise(vp.shape, (g.h, 0.556, 0.509), 10.0, 1000 + q + m_)
            versions[m_].append((versions[m_][-1] * (1.0 + 0.01 * pert)).astype(np.float32))
    outs = [torch.empty(stations[k].shape, dtype=torch.float32, device="cuda") for k, _ in picks]
    meta = []
    with lib.Server(0, hbm_bytes=120 << 30) as sv:
        sv.set_model(0, vp)
        sv.set_model(1, vs)
        cur = {0: 1, 1: 1}
        t0 = time.time()
        due = t0
        for q, (k, ph) in enumerate(picks):
            if q > 0 and q % 100 == 0:
                for m_ in (0, 1):
                    sv.set_model(m_, versions[m_][cur[m_]])
                    cur[m_] += 1
            due += gaps[q]
            d = due - time.time()
            if d > 0:
                time.sleep(d)
            sv.submit(stations[k], ph, outs[q], tag=q)
            meta.append((k, ph, cur[ph]))
        sv.drain(3600000)
        wall = time.time() - t0
        res = sv.poll(n + 8)
        m = sv.metrics()
    bad = sum(1 for r in res if r["status"] != 0)
    # a sample re-solved alone against the model version each was served with
    sample = [int(q) for q in np.random.default_rng(44).choice(n, 6, replace=False)]
    same = 0
    with lib.Context(0) as ctx:
        for q in sample:
            k, ph, ver = meta[q]
            v = versions[ph][ver - 1]
            (t,), _ = ctx.solve_host([stations[k]], v)
            same += int(np.array_equal(t.view(np.uint32), outs[q].cpu().numpy().view(np.uint32)))
    line = {
        "metric": "station fields/s served (P and S, Poisson arrivals), bit-identical to reference",
        "value": n / wall, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 stencils / f32 fields",
        "data": "synthetic (seeded, config 4 recipe, scaled rate)",
        "config": {"workload": f"{n} requests over 800 windows 61..301 x 61..301 x 61..121 (401x401x161 model), "
                               f"P and S, Poisson {args.rate}/s, models replaced every 100 requests (config 4)",
                   "rate_per_s": args.rate, "model_updates": cur[0] - 1},
        "latency_ms": {"p50": m["p50_ms"], "p90": m["p90_ms"], "p99": m["p99_ms"], "max": m["max_ms"]},
        "solve_ms": {"p50": m["solve_p50_ms"], "p99": m["solve_p99_ms"]},
        "node_updates_per_s": m["node_updates"] / wall, "failed": bad, "hbm_peak_bytes": m["hbm_peak"],
        "parity": {"sampled_requests_equal_alone": f"{same}/{len(sample)}"},
        "gpu_launches": m["grid_launches"],
    }
    print(json.dumps(line), flush=True)
    shutil.rmtree(case_dir, ignore_errors=True)


def run_gpu(args):
    rank, world, local = dist_env()
    n = args.stations
    case_dir = tempfile.mkdtemp(prefix=f"fdbench_r{rank}_")
    g, v, sts = workload(rank, n, args.config)
    write_case(case_dir, g, v, sts)
    names = [s["name"] for s in sts]

    # CPU baseline first (before any CUDA call in this process), rank 0 at N=1 only
    cpu = None
    ncores = os.cpu_count() or 1
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sample = names[:min(ncores, n)]
        wall, nu_cpu, cpu_out = cpu_solve(case_dir, sample, ncores)
        cpu = dict(value=len(sample) / wall, unit=UNIT, cores=min(ncores, len(sample)), kind="port",
                   sample=f"{len(sample)} of the {n} stations, one oracle process per core (oracle FAST mode: "
                          f"exact pruned restatement, faster than the reference binary), {wall:.1f} s wall",
                   node_updates_per_s=nu_cpu / wall)

    import numpy as np
    import torch
    from fdtomoc_gb300 import build, lib

    build.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stations = [lib.station_from_par("par=" + os.path.join(case_dir, nm + ".par"))[0] for nm in names]
    ctx = lib.Context(local)
    stream = torch.cuda.Stream()
    vel_d = torch.from_numpy(v.reshape(-1)).cuda()
    slow = torch.empty_like(vel_d)
    with torch.cuda.stream(stream):
        ctx.velocity_to_slowness(vel_d.data_ptr(), slow.data_ptr(), v.size, stream.cuda_stream)
    stream.synchronize()
    fields = [torch.empty(s.shape, dtype=torch.float32, device="cuda") for s in stations]
    tptr = [f.data_ptr() for f in fields]

    def step():
        return ctx.solve_device(stations, slow.data_ptr(), g.nx, g.nx * g.ny, tptr, stream_ptr=stream.cuda_stream)

    for _ in range(args.warmup):
        stats = step()

    # parity against the CPU oracle on the stations it solved
    parity = None
    if cpu is not None:
        nd, maxd = 0, 0.0
        for nm, f in zip(names[:cpu["cores"]], fields):
            ref = np.fromfile(os.path.join(case_dir, "cpu_out", nm + ".ptimes"), dtype="<f4", offset=232)
            got = f.cpu().numpy().reshape(-1)
            nd += int((ref != got).sum())
            maxd = max(maxd, float(np.abs(ref.astype(np.float64) - got).max()))
        parity = {"stations_checked": cpu["cores"], "nodes_differing": nd, "max_abs_dt_s": maxd,
                  "tolerance_s": 1e-4, "bit_identical": nd == 0}

    # timed region
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    all_stats = []
    for _ in range(args.steps):
        all_stats.append(step())
    ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    total_stations = n * world
    value = total_stations * args.steps / (ms / 1e3)
    nu_step = sum(s["node_updates"] for s in all_stats[-1])
    lat = sorted((s["t_end_ns"] - min(x["t_start_ns"] for x in all_stats[-1])) / 1e6 for s in all_stats[-1])
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]

    # plain form: one station per launch
    t0 = time.time()
    ev0.record(stream)
    ctx.solve_device(stations[:1], slow.data_ptr(), g.nx, g.nx * g.ny, tptr[:1], stream_ptr=stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    plain_ms = ev0.elapsed_time(ev1)

    # end to end through the host-buffer entry point: pinned velocity in, all fields out
    vel_h = torch.from_numpy(v.reshape(-1).copy()).pin_memory()
    outs = [torch.empty(s.shape, dtype=torch.float32).pin_memory() for s in stations]
    import ctypes as C
    lib_ = lib.load()
    arr = (lib.Station * n)(*stations)
    outp = (C.POINTER(C.c_float) * n)(*[C.cast(o.data_ptr(), C.POINTER(C.c_float)) for o in outs])
    e2e_steps = max(1, min(args.steps, 2))
    rc = lib_.fdgpu_solve_host(ctx.ptr, n, arr, C.cast(vel_h.data_ptr(), C.POINTER(C.c_float)), g.nx, g.ny, g.nz,
                               outp, None, None)   # warm-up: allocates the context's host-path buffers
    if rc != 0:
        raise RuntimeError(f"fdgpu_solve_host failed: {rc}")
    torch.cuda.synchronize()
    t0 = time.time()
    for _ in range(e2e_steps):
        rc = lib_.fdgpu_solve_host(ctx.ptr, n, arr, C.cast(vel_h.data_ptr(), C.POINTER(C.c_float)), g.nx, g.ny,
                                   g.nz, outp, None, None)
        if rc != 0:
            raise RuntimeError(f"fdgpu_solve_host failed: {rc}")
    e2e_s = (time.time() - t0) / e2e_steps
    e2e = {"value": total_stations / e2e_s if world == 1 else None, "unit": UNIT,
           "h2d_bytes_per_step": int(v.size * 4), "d2h_bytes_per_step": int(sum(o.numel() * 4 for o in outs))}
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e["value"] = total_stations / float(t.item())

    locating = locate_leg(args, lib, ctx, g, fields, stream) if args.locate_events > 0 else None
    modelling = c2f_leg(args, lib, ctx, stream) if not args.no_c2f else None
    tracing = ray_leg(args, lib, ctx, g, sts, fields, stream) if args.ray_events > 0 else None
    # the serving session's long-running grid waits on its host thread; under a profiler that
    # serialises launches the launching call would not return while the grid waits, so the leg is
    # left out there
    profiled = under_profiler()
    serving = serve_leg(args, lib, stations, v, fields) if args.serve_requests > 0 and not profiled else None

    # roofline of the solve kernel (one launch per step): algorithmic bytes 12 B per node update
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = ALGO_BYTES_PER_NODE_UPDATE * nu_step / (ms_step / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "fd_solve_traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath))
        traffic = tj["dram_bytes_per_node_update"] * nu_step
    # FP64 pipe roofline: FP64 instructions per stencil evaluation (static counts of the evaluators,
    # divisions 5, square roots 8) x evaluations, against the FP64 rate measured live on this GPU
    st_sum = [sum(s["stencils"][k] for s in all_stats[-1]) for k in range(5)]
    fp64_ops = 116 * st_sum[0] + 70 * st_sum[1] + 69 * st_sum[2] + 25 * st_sum[3] + 6 * st_sum[4]
    fp64_peak = ctx.probe_fp64_gops()
    fp64 = {"achieved_gops": fp64_ops / (ms_step / 1e3) / 1e9, "peak_gops": fp64_peak,
            "frac": fp64_ops / (ms_step / 1e3) / 1e9 / fp64_peak, "peak_kind": "measured (FP64 add/mul/fma chain probe)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 stencils / f32 fields", "data": f"synthetic (seeded, config {args.config} recipe)",
            "config": {"workload": CONFIG_NAME if args.config == 2 else CONFIG1_NAME, "stations_per_gpu": n, "grid": [g.nx, g.ny, g.nz],
                       "l2": ("inputs larger than L2 (64 fields x 13 MB + 13 MB model)" if args.config == 2
                              else "small case: inputs fit in L2"), "parallelism": f"stations x{world}"},
            "node_updates_per_s": nu_step * world / (ms_step / 1e3),
            "latency_ms": {"p50": p50, "p99": p99, "what": "station completion time within a batch"},
            "plain": {"ms_per_station": plain_ms, "fields_per_s": 1e3 / plain_ms,
                      "batched_over_plain": value / world / (1e3 / plain_ms)},
            "e2e": e2e,
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "note": "the path is FP64- and dependency-latency-bound, not HBM-bound"},
            "fp64": fp64,
            "parity": parity,
            "clocks": clocks,
            "sweeps": [s["sweeps"] for s in all_stats[-1]][:8],
        }
        if serving is not None:
            line["serving"] = serving
        if locating is not None:
            line["locate"] = locating
        if modelling is not None:
            line["c2f"] = modelling
        if tracing is not None:
            line["rays"] = tracing
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    ctx.close()
    shutil.rmtree(case_dir, ignore_errors=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------------------------------------
# reference arm: the oracle on the host cores


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n = args.stations
    ncores = os.cpu_count() or 1
    case_dir = tempfile.mkdtemp(prefix="fdbench_ref_")
    g, v, sts = workload(0, n, args.config)
    write_case(case_dir, g, v, sts)
    names = [s["name"] for s in sts]
    sample = names[:min(ncores, n)]
    for _ in range(args.warmup):
        cpu_solve(case_dir, sample, ncores)
    walls, nus = [], []
    for k in range(args.steps):
        wall, nu, _ = cpu_solve(case_dir, sample, ncores)
        walls.append(wall)
        nus.append(nu)
    tot = sum(walls)
    value = len(sample) * args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 stencils / f32 fields", "data": f"synthetic (seeded, config {args.config} recipe)",
        "config": {"workload": CONFIG_NAME if args.config == 2 else CONFIG1_NAME, "stations_per_gpu": n, "grid": [g.nx, g.ny, g.nz],
                   "parallelism": f"{len(sample)} processes x 1 thread"},
        "node_updates_per_s": sum(nus) / tot,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(sample), "kind": "port",
                         "sample": f"{len(sample)} of the {n} stations per step, one oracle process per core "
                                   "(oracle FAST mode, exact)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    shutil.rmtree(case_dir, ignore_errors=True)


def main():
    args = parse()
    if args.profile_legs:
        profile_legs(args)
    elif args.config == 3 and args.impl == "reference":
        run_reference_config3(args)
    elif args.config == 3:
        run_config3(args)
    elif args.config == 4 and args.impl != "reference":
        run_config4(args)
    elif args.config == 5 and args.impl != "reference":
        run_config5(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
