#!/usr/bin/env python3
"""Golden fixtures for the location path: run the reference's own sphfdloc (compiled from its
sources by oracle/Makefile into oracle/_ref/) on the seeded cases of loc_cases.py and keep its four
output files.  Run here, where the reference sources exist:

    make -C oracle ref && python tests/golden/make_loc_golden.py

Writes tests/golden/loc_<seed>/{case.json, ref_fhd.txt, ref_dat.txt, ref_sum.txt, ref_out.txt}.
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

import loc_cases as LC  # noqa: E402


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "sphfdloc_ref")
    if not os.path.exists(exe):
        raise SystemExit("build the reference first: make -C oracle ref")
    for seed in LC.SEEDS:
        p = LC.make_case(seed)
        work = tempfile.mkdtemp(prefix=f"loc{seed}_")
        spec = LC.write_reference_inputs(p, work)
        r = subprocess.run([exe], input=spec + "\n", text=True, capture_output=True, cwd=work, timeout=600)
        if r.returncode != 0:
            raise SystemExit(f"reference sphfdloc failed on seed {seed}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        d = LC.golden_dir(seed)
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump(p, f, indent=1)
        for k, name in (("fhd", "fhd.txt"), ("dat", "dat.txt"), ("sum", "sum.txt"), ("out", "out.txt")):
            shutil.copy(os.path.join(work, "out", name), os.path.join(d, f"ref_{k}.txt"))
        print(seed, "events", len(p["events"]), "accepted", open(os.path.join(d, "ref_fhd.txt")).read().count("\n"))
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
