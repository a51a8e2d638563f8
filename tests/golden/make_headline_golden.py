"""Pin the benchmark workloads against the reference binary: every station of the 64-station
201x201x81 workload (config 2) and every one of the 500 uneven windows over the 401x401x161 model
(config 3); with --config5, a seeded sample of 8 of the 1200 stations on the full 401x401x161 grid
with the dipping slab (config 5).

Run where the reference sources are present (oracle/Makefile builds the reference's own sphfd from
them into oracle/_ref/sphfd_ref; the source root is taken from $FDTOMOC_REFERENCE):

    python tests/golden/make_headline_golden.py [--jobs 8]

For each solve it runs the reference binary and the oracle (its exact pruned mode, the one the CPU
baselines time) on the same par file, one process per job slot, and records

  data_sha256   SHA-256 of the reference's time file without its 232-byte header, i.e. of the
                nx*ny*nz float32 travel times as they sit in memory (the GPU tests hash their
                fields the same way);
  file_sha256   SHA-256 of the whole reference time file (header included);
  sweeps        the reference's sweep count (1 + restarts, from its stderr);
  node_updates  the oracle's node updates (one face-point evaluation each), the unit the CPU baseline
                of the benchmark extrapolates with;
  oracle_equal  whether the oracle's time file equals the reference's byte for byte.

The models are regenerated from their seeds by fdtomoc_gb300.workloads; the SHA-256 of each model's
float32 values is stored too, so a machine whose generator produced different bits is detected
before any field is compared.  Each config-3 window is cut from the model into its own velocity
file, because sphfd reads the first nx*ny*nz values of its file; the GPU reads the same window in
place at (ox, oy, 0).

Writes tests/golden/headline_reference.json (resumable: finished solves are kept in
headline_reference.partial.json until the run completes).
"""
import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "sphfd_ref")
ORACLE_BIN = os.path.join(ROOT, "oracle", "sphfd_oracle")
OUT = os.path.join(HERE, "headline_reference.json")
PARTIAL = os.path.join(HERE, "headline_reference.partial.json")


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def model_sha(v) -> str:
    import numpy as np
    return sha(np.ascontiguousarray(v, dtype="<f4").tobytes())


def jobs_for(tmp):
    """(key, par file, write-inputs callable, nodes) for every solve; window inputs are written
    lazily, just before their first solve."""
    import numpy as np
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_grid, write_par
    out = []
    g2, v2, sts = W.config(2)
    d2 = os.path.join(tmp, "c2")
    os.makedirs(d2, exist_ok=True)
    vf2 = os.path.join(d2, "vp.mod")
    write_grid(vf2, W.head_for(g2), v2)
    for st in sts:
        pf = os.path.join(d2, st["name"] + ".par")
        write_par(pf, W.par_for(g2, st, vf2, st["name"] + ".ptimes"))
        out.append((("config2", st["name"]), pf, None, g2.nx * g2.ny * g2.nz))
    g3, v3, _ = W.config(3)
    d3 = os.path.join(tmp, "c3")
    os.makedirs(d3, exist_ok=True)
    for w in W.config3_windows():
        wg = W.Grid(w["nx"], w["ny"], w["nz"], g3.dlon, g3.dlat, g3.h, x0=g3.x0 + w["ox"] * g3.dlon,
                    y0=g3.y0 - w["oy"] * g3.dlat, z0=g3.z0)
        wf = os.path.join(d3, w["name"] + ".mod")
        pf = os.path.join(d3, w["name"] + ".par")
        write_par(pf, W.window_par(g3, w, wf, w["name"] + ".ptimes"))

        def make(w=w, wg=wg, wf=wf):
            write_grid(wf, W.head_for(wg), np.ascontiguousarray(v3[:w["nz"], w["oy"]:w["oy"] + w["ny"],
                                                                   w["ox"]:w["ox"] + w["nx"]]))
        out.append((("config3", w["name"]), pf, make, w["nx"] * w["ny"] * w["nz"]))
    return out, {"config2": model_sha(v2), "config3": model_sha(v3)}


def launch(exe, parfile, outdir, env=None):
    os.makedirs(outdir, exist_ok=True)
    d = os.path.dirname(parfile)
    base = os.path.basename(outdir)
    pl = os.path.join(d, f"pl_{base}")
    with open(pl, "w") as f:
        f.write("par=" + parfile + "\n")
    spec = os.path.join(d, f"spec_{base}")
    with open(spec, "w") as f:
        f.write(f"parlist {pl}\ntimedir {outdir}\n")
    p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                         text=True, env=dict(os.environ, OMP_NUM_THREADS="1", **(env or {})))
    p.stdin.write(spec + "\n")
    p.stdin.close()
    return p


def sweeps_of(log):
    return 1 + log.count("RESTART at") - log.count("RESTART CANCELLED")


CONFIG5_SAMPLE = 8   # config-5 stations pinned (a seeded sample of the 1200: full-grid solves are long)


def config5_sample():
    """The seeded sample of config-5 stations that is pinned: their indices among the 1200."""
    import numpy as np
    return sorted(int(k) for k in np.random.default_rng(55).choice(1200, CONFIG5_SAMPLE, replace=False))


def main_config5(jobs):
    """Add the config-5 sample (401x401x161 with the dipping slab) to headline_reference.json."""
    import numpy as np
    from fdtomoc_gb300 import workloads as W
    from fdtomoc_gb300.formats import write_grid, write_par
    out = json.load(open(OUT))
    tmp = tempfile.mkdtemp(prefix="headline5_")
    g, v, sts = W.config(5)
    vf = os.path.join(tmp, "vp.mod")
    write_grid(vf, W.head_for(g), v)
    picks = config5_sample()
    running, res = [], {}
    pending = []
    for k in picks:
        st = sts[k]
        pf = os.path.join(tmp, st["name"] + ".par")
        write_par(pf, W.par_for(g, st, vf, st["name"] + ".ptimes"))
        pending += [(st["name"], "ref", pf), (st["name"], "oracle", pf)]
    t_start = time.time()
    while pending or running:
        while pending and len(running) < jobs:
            name, kind, pf = pending.pop(0)
            outdir = os.path.join(tmp, f"{name}_{kind}")
            exe = REF_BIN if kind == "ref" else ORACLE_BIN
            running.append((name, kind, launch(exe, pf, outdir, None if kind == "ref" else {"FDO_MODE": "fast"}),
                            outdir, time.time()))
        time.sleep(0.2)
        still = []
        for name, kind, p, outdir, t0 in running:
            if p.poll() is None:
                still.append((name, kind, p, outdir, t0))
                continue
            log = p.stderr.read()
            if p.returncode != 0:
                raise RuntimeError(f"{kind} failed on {name}: {log[-2000:]}")
            b = open(os.path.join(outdir, name + ".ptimes"), "rb").read()
            shutil.rmtree(outdir)
            res.setdefault(name, {})[kind] = (b, log, time.time() - t0)
            print(f"[{time.time() - t_start:7.0f} s] config5/{name} {kind} done", flush=True)
        running = still
    out["models"]["config5"] = model_sha(v)
    out["config5"] = {}
    for name, h in res.items():
        rb, rlog, rt = h["ref"]
        ob, olog, ot = h["oracle"]
        nu = 0
        for tok in olog.split():
            if tok.startswith("node_updates="):
                nu = int(tok.split("=")[1])
        out["config5"][name] = {"data_sha256": sha(rb[232:]), "file_sha256": sha(rb), "sweeps": sweeps_of(rlog),
                                "node_updates": nu, "oracle_equal": rb == ob, "ref_s": round(rt, 2),
                                "oracle_s": round(ot, 2)}
    json.dump(out, open(OUT, "w"), indent=0, sort_keys=True)
    shutil.rmtree(tmp, ignore_errors=True)
    print(json.dumps({k: (v["sweeps"], v["oracle_equal"]) for k, v in out["config5"].items()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--config5", action="store_true",
                    help="add the pinned sample of config-5 stations to an existing headline_reference.json")
    args = ap.parse_args()
    if args.config5:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "sphfd_oracle"], check=True)
        return main_config5(args.jobs)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "sphfd_oracle"], check=True)
    assert os.path.exists(REF_BIN), "reference binary not built (are the reference sources present?)"
    tmp = tempfile.mkdtemp(prefix="headline_")
    todo, models = jobs_for(tmp)
    done = {}
    if os.path.exists(PARTIAL):
        part = json.load(open(PARTIAL))
        if part.get("models") == models:
            done = part["solves"]
    # largest first, so that the last job slots do not wait on one long solve
    todo = [t for t in todo if "/".join(t[0]) not in done]
    todo.sort(key=lambda t: -t[3])
    pending = []
    for key, pf, make, _ in todo:
        pending.append((key, "ref", pf, make))
        pending.append((key, "oracle", pf, None))
    running, half = [], {}
    t_start = time.time()
    while pending or running:
        while pending and len(running) < args.jobs:
            key, kind, pf, make = pending.pop(0)
            if make is not None:
                make()
            outdir = os.path.join(os.path.dirname(pf), f"{key[1]}_{kind}")
            exe = REF_BIN if kind == "ref" else ORACLE_BIN
            env = None if kind == "ref" else {"FDO_MODE": "fast"}
            running.append((key, kind, launch(exe, pf, outdir, env), outdir, time.time(), pf))
        time.sleep(0.05)
        still = []
        for key, kind, p, outdir, t0, pf in running:
            if p.poll() is None:
                still.append((key, kind, p, outdir, t0, pf))
                continue
            log = p.stderr.read()
            if p.returncode != 0:
                raise RuntimeError(f"{kind} failed on {key}: {log[-2000:]}")
            b = open(os.path.join(outdir, key[1] + ".ptimes"), "rb").read()
            shutil.rmtree(outdir)
            k = "/".join(key)
            h = half.setdefault(k, {})
            h[kind] = (b, log, time.time() - t0)
            if "ref" in h and "oracle" in h:
                rb, rlog, rt = h["ref"]
                ob, olog, ot = h["oracle"]
                nu = 0
                for tok in olog.split():
                    if tok.startswith("node_updates="):
                        nu = int(tok.split("=")[1])
                done[k] = {"data_sha256": sha(rb[232:]), "file_sha256": sha(rb), "sweeps": sweeps_of(rlog),
                           "node_updates": nu, "oracle_equal": rb == ob, "ref_s": round(rt, 2),
                           "oracle_s": round(ot, 2)}
                del half[k]
                if key[0] == "config3":
                    wf = os.path.join(os.path.dirname(pf), key[1] + ".mod")
                    if os.path.exists(wf):
                        os.remove(wf)
                json.dump({"models": models, "solves": done}, open(PARTIAL, "w"))
                print(f"[{time.time() - t_start:7.0f} s] {k}: sweeps {done[k]['sweeps']}, {nu} node updates, "
                      f"ref {rt:.1f} s, oracle {ot:.1f} s, oracle equal {rb == ob}", flush=True)
        running = still
    out = {"models": models, "config2": {}, "config3": {}}
    for k, v in sorted(done.items()):
        c, name = k.split("/")
        out[c][name] = v
    json.dump(out, open(OUT, "w"), indent=0, sort_keys=True)
    os.remove(PARTIAL)
    shutil.rmtree(tmp, ignore_errors=True)
    bad = [k for k, v in done.items() if not v["oracle_equal"]]
    print(json.dumps({"solves": len(done), "oracle_differs": bad}))


if __name__ == "__main__":
    main()
