#!/usr/bin/env python3
"""Golden digests for c2f: run the reference's own c2f (compiled from its sources by
oracle/Makefile into oracle/_ref/) on the seeded coarse models of c2f_cases.py and record the SHA-256
of its three output files' data.  Run here, where the reference sources exist:

    make -C oracle ref && python tests/golden/make_c2f_golden.py
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import c2f_cases as CC  # noqa: E402


def data_digest(path):
    return hashlib.sha256(open(path, "rb").read()[232:]).hexdigest()


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "c2f_ref")
    if not os.path.exists(exe):
        raise SystemExit("build the reference first: make -C oracle ref")
    out = {}
    for seed in CC.SEEDS:
        p = CC.make_case(seed)
        work = tempfile.mkdtemp(prefix=f"c2f{seed}_")
        spec = CC.write_reference_inputs(p, work)
        r = subprocess.run([exe], input=f"{spec}\n{spec}\n", text=True, capture_output=True, cwd=work, timeout=300)
        if r.returncode != 0:
            raise SystemExit(f"reference c2f failed on seed {seed}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        out[str(seed)] = dict(case=p, dims=CC.dims(p), fine=data_digest(os.path.join(work, "fine")),
                              pvel=data_digest(os.path.join(work, "fine.pvel")),
                              svel=data_digest(os.path.join(work, "fine.svel")))
        print(seed, CC.dims(p))
        shutil.rmtree(work, ignore_errors=True)
    with open(CC.golden_path(), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
