#!/usr/bin/env python3
"""Golden fixtures for sphfdloc followed by sphrayderv: run the reference's own two programs (compiled
from their sources by oracle/Makefile into oracle/_ref/) on the cases of chain_cases.py and keep their
ten output files.  Run here, where the reference sources exist:

    make -C oracle ref && python tests/golden/make_chain_golden.py

Writes tests/golden/chain_<seed>/{case.json, fhd.txt, dat.txt, sum.txt, out.txt, dtds.bin, res.bin,
dtdh.txt, book.txt, scle.txt, hit.txt}.
"""
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

import chain_cases as CC  # noqa: E402
import loc_cases as LC  # noqa: E402


def main():
    loc = os.path.join(ROOT, "oracle", "_ref", "sphfdloc_ref")
    ray = os.path.join(ROOT, "oracle", "_ref", "sphrayderv_ref")
    if not (os.path.exists(loc) and os.path.exists(ray)):
        raise SystemExit("build the reference first: make -C oracle ref")
    for seed in CC.SEEDS:
        p = LC.make_case(seed)
        work = tempfile.mkdtemp(prefix=f"chain{seed}_")
        spec = CC.write_inputs(p, work)
        for exe in (loc, ray):
            r = subprocess.run([exe], input=spec + "\n", text=True, capture_output=True, cwd=work, timeout=300)
            if r.returncode != 0:
                raise SystemExit(f"{os.path.basename(exe)} failed on seed {seed}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        d = CC.golden_dir(seed)
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "case.json"), "w") as fh:
            json.dump(p, fh, indent=1)
        for name in CC.LOC_FILES.values():
            shutil.copy(os.path.join(work, "out", name), os.path.join(d, name))
        for name in CC.RAY_FILES.values():
            shutil.copy(os.path.join(work, "ray", name), os.path.join(d, name))
        with open(os.path.join(work, "ray", "book.txt")) as fh:
            print(seed, "book:", fh.read().split("\n")[:-1])
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
