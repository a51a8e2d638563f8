"""Golden outputs of the reference's make_par_file (src/make_par_file.c), for the par-file writer
fdtomoc_gb300.parfiles.

Run where the reference sources are present (oracle/Makefile builds make_par_file from them into
oracle/_ref/make_par_file_ref):

    python tests/golden/make_parfile_golden.py

For each case of PARFILE_CASES (a spec and a station list) the reference binary runs in an empty
directory; every file it writes there (<sta>.par, <sta>.spar, runsphfd01.sh) is stored, as text,
in tests/golden/parfiles_reference.json.
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from cases import PARFILE_CASES  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "make_par_file_ref")


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    out = {}
    for name, case in PARFILE_CASES.items():
        with tempfile.TemporaryDirectory() as d:
            spec, sta = os.path.join(d, "in.spec"), os.path.join(d, "in.sta")
            open(spec, "w").write(case["spec"])
            open(sta, "w").write(case["stations"])
            work = os.path.join(d, "work")
            os.makedirs(work)
            subprocess.run([REF_BIN, spec, sta], cwd=work, check=True, capture_output=True)
            out[name] = {f: open(os.path.join(work, f)).read() for f in sorted(os.listdir(work))}
    json.dump(out, open(os.path.join(HERE, "parfiles_reference.json"), "w"), indent=1, sort_keys=True)
    print({k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
