#!/usr/bin/env python3
"""Golden fixtures for sphrayderv: run the reference's own sphrayderv (compiled from its sources by
oracle/Makefile into oracle/_ref/) on the seeded cases of ray_cases.py and keep its six output files.
Run here, where the reference sources exist:

    make -C oracle ref && python tests/golden/make_ray_golden.py

Writes tests/golden/ray_<seed>/{case.json, dtds.bin, res.bin, dtdh.txt, book.txt, scle.txt, hit.txt}.
The inputs (time fields included) are rebuilt from case.json by ray_cases.write_inputs.
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import ray_cases as RC  # noqa: E402


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "sphrayderv_ref")
    if not os.path.exists(exe):
        raise SystemExit("build the reference first: make -C oracle ref")
    for seed in RC.SEEDS + RC.EXTRA_SEEDS:
        p = RC.make_case(seed)
        work = tempfile.mkdtemp(prefix=f"ray{seed}_")
        spec = RC.write_inputs(p, work)
        r = subprocess.run([exe], input=spec + "\n", text=True, capture_output=True, cwd=work, timeout=600)
        if r.returncode != 0:
            raise SystemExit(f"reference sphrayderv failed on seed {seed}:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        d = RC.golden_dir(seed)
        os.makedirs(d, exist_ok=True)
        RC.save_case_json(p, d)
        for name in RC.OUT_FILES.values():
            shutil.copy(os.path.join(work, "out", name), os.path.join(d, name))
        with open(os.path.join(work, "out", "book.txt")) as fh:
            print(seed, "grid", p["nx"], p["ny"], p["nz"], "book:", fh.read().split("\n")[:-1])
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
