"""Generate the golden fixtures of the parity tests from the reference itself.

Run where the reference sources are present (their root from $FDTOMOC_REFERENCE; oracle/Makefile
builds the reference's own sphfd from them into oracle/_ref/sphfd_ref):

    python tests/golden/make_golden.py

Writes:
  m001.npz          the reference's golden pair for station M001 (verification/cmod): the velocity
                    file (header + P field) and M001.ptimes, with the three CR bytes that the
                    reference's `.gitattributes` ("* text eol=lf") stripped from the binary file
                    restored at data offsets 103421, 131353, 181824; checked against a fresh run of the
                    reference binary.
  reference_outputs.json
                    SHA-256 of the reference binary's time file for seeded cases (cases.py), for
                    solves from a supplied start (srctype 2 and 3, fill=1; cases.start_case) and for
                    config 1 (fdtomoc_gb300.workloads), with their sweep counts; for byte-swapped
                    models and times (swab 1/2/3, cases.write_swab_case); and for one iteration's
                    P and S par files in make_par_file's dialect, solved through the reference's
                    parlist driver (cases.ps_station_case).
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
REF = os.environ.get("FDTOMOC_REFERENCE", "/root/reference")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "sphfd_ref")
M001_PAR = dict(fxs="121.37915", fys="23.12651", fzs="-0.198", nx="41.000000", ny="41.000000", nz="31.000000",
                x0="120.9", y0="23.8", z0="-4.0", h="2.0", timefile="M001.ptimes", reverse="50")
CR_OFFSETS = [103421, 131353, 181824]
SEEDS = [0, 1, 2, 4, 5, 6, 8, 9, 10, 11, 13, 17, 21, 33, 47, 58, 77, 91, 123, 250]


def run_reference(parfile, outdir):
    os.makedirs(outdir, exist_ok=True)
    d = os.path.dirname(parfile)
    with open(os.path.join(d, "parlist_ref"), "w") as f:
        f.write("par=" + parfile + "\n")
    spec = os.path.join(d, "spec_ref")
    with open(spec, "w") as f:
        f.write(f"parlist {os.path.join(d, 'parlist_ref')}\ntimedir {outdir}\n")
    r = subprocess.run([REF_BIN], input=spec + "\n", capture_output=True, text=True)
    return r.stderr


def sweeps_of(log):
    return 1 + log.count("RESTART at") - log.count("RESTART CANCELLED")


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    assert os.path.exists(REF_BIN), "reference binary not built"
    from fdtomoc_gb300.formats import write_par
    from cases import random_case, write_random_case
    tmp = tempfile.mkdtemp()
    # M001
    vel = open(os.path.join(REF, "verification/cmod/tempvel"), "rb").read()
    raw = open(os.path.join(REF, "verification/cmod/M001.ptimes"), "rb").read()
    hdr, data = raw[:232], bytearray(raw[232:])
    for off in CR_OFFSETS:
        assert data[off] == 0x0A
        data[off:off] = b"\r"
    expected = hdr + bytes(data)
    nxyz = 41 * 41 * 31
    vel_p = vel[:232 + 4 * nxyz]
    vf = os.path.join(tmp, "m001.vel")
    open(vf, "wb").write(vel_p)
    pf = os.path.join(tmp, "M001.par")
    write_par(pf, dict(M001_PAR, velfile=vf))
    run_reference(pf, os.path.join(tmp, "m001_out"))
    got = open(os.path.join(tmp, "m001_out", "M001.ptimes"), "rb").read()
    assert got == expected, "reference binary does not reproduce the repaired golden file"
    np.savez_compressed(os.path.join(HERE, "m001.npz"), velocity_file=np.frombuffer(vel_p, np.uint8),
                        expected=np.frombuffer(expected, np.uint8))
    out = {"m001": {"sha256": hashlib.sha256(expected).hexdigest(), "par": M001_PAR}}
    # seeded cases
    cases = {}
    for s in SEEDS:
        d = os.path.join(tmp, f"c{s}")
        pf = write_random_case(random_case(s), d)
        log = run_reference(pf, os.path.join(d, "out"))
        b = open(os.path.join(d, "out", "case.ptimes"), "rb").read()
        cases[str(s)] = {"sha256": hashlib.sha256(b).hexdigest(), "sweeps": sweeps_of(log), "bytes": len(b)}
    out["cases"] = cases
    # solves from a supplied start (srctype 2, srctype 3, fill=1)
    from cases import START_KINDS, START_SEEDS, start_case, write_start_case
    starts = {}
    for s in START_SEEDS:
        for kind in START_KINDS:
            d = os.path.join(tmp, f"s{s}_{kind}")
            pf = write_start_case(start_case(s, kind), d)
            log = run_reference(pf, os.path.join(d, "out"))
            b = open(os.path.join(d, "out", "case.ptimes"), "rb").read()
            # srctype 2/3: the reference writes its uninitialised source point into the header's
            # fxs/fys/fzs (bytes 120-143), so those cases are compared with the three doubles zeroed
            masked = b[:120] + bytes(24) + b[144:]
            starts[f"{s}_{kind}"] = {"sha256": hashlib.sha256(b).hexdigest(),
                                     "sha256_source_zeroed": hashlib.sha256(masked).hexdigest(),
                                     "sweeps": sweeps_of(log), "bytes": len(b)}
    out["start_cases"] = starts
    # config 1
    from fdtomoc_gb300 import workloads as W
    g, v, sts = W.config(1)
    d = os.path.join(tmp, "cfg1")
    W.write_case(d, g, v, sts)
    log = run_reference(os.path.join(d, "S0000.par"), os.path.join(d, "ref"))
    b = open(os.path.join(d, "ref", "S0000.ptimes"), "rb").read()
    out["config1_S0000"] = {"sha256": hashlib.sha256(b).hexdigest(), "sweeps": sweeps_of(log)}
    # byte-swapped models and times
    from cases import SWAB_SEEDS, ps_station_case, write_swab_case
    swabs = {}
    for s in SWAB_SEEDS:
        for sw in (1, 2, 3):
            d = os.path.join(tmp, f"w{s}_{sw}")
            pf = write_swab_case(random_case(s), d, sw)
            run_reference(pf, os.path.join(d, "out"))
            b = open(os.path.join(d, "out", "case.ptimes"), "rb").read()
            swabs[f"{s}_{sw}"] = {"sha256": hashlib.sha256(b).hexdigest(), "bytes": len(b)}
    out["swab_cases"] = swabs
    # one iteration's P and S par files (make_par_file's dialect) through the reference's parlist driver
    d = os.path.join(tmp, "ps")
    paths, _, _ = ps_station_case(d)
    with open(os.path.join(d, "parlist_ref"), "w") as f:
        f.write("".join("par=" + p + "\n" for p in paths))
    spec = os.path.join(d, "spec_ref")
    with open(spec, "w") as f:
        f.write(f"parlist {os.path.join(d, 'parlist_ref')}\ntimedir {os.path.join(d, 'out')}\n")
    os.makedirs(os.path.join(d, "out"))
    subprocess.run([REF_BIN], input=spec + "\n", capture_output=True, text=True, check=True)
    out["ps_stations"] = {f: hashlib.sha256(open(os.path.join(d, "out", f), "rb").read()).hexdigest()
                          for f in sorted(os.listdir(os.path.join(d, "out")))}
    json.dump(out, open(os.path.join(HERE, "reference_outputs.json"), "w"), indent=1)
    print(json.dumps({k: (v if k != "cases" else len(v)) for k, v in out.items()}))


if __name__ == "__main__":
    main()
