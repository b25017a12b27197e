#!/usr/bin/env python3
"""Golden outputs of the reference CUDA binary, run on a GB300.

Step 1 (here, where the reference tree is present):
    python tests/golden/make_ref_golden.py stage
  copies the reference sources into oracle/_ref/src (git-ignored; never
  committed), writes the input files of every case below into
  oracle/_ref/runs/<tag>/ (input file, betas, LUT from the reference's own
  create_LUT.c or, where it refuses the temperature set, from the oracle's
  restatement of its arithmetic) and a driver script oracle/_ref/runs/run_all.sh.

Step 2 (on the GPU host, from the repository root):
    bash oracle/_ref/runs/run_all.sh
  builds one reference executable per case with plain nvcc/g++ lines
  (oracle/Makefile, target ref-cuda; not the reference's own Makefile), runs
  it, and copies each output tree to <OUT>/<tag>/, OUT being the folder that
  the GPU host hands back (EA_REFGOLD_OUT, relative to the repository root).

Step 3 (here):
    python tests/golden/make_ref_golden.py collect
  turns <OUT>/ into tests/golden/ref_<tag>.npz: every output file
  of every (sample, replica) -- whole when small, SHA-256 otherwise.
"""
import hashlib
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")
RUNS = os.path.join(ORACLE, "_ref", "runs")
# EA_REF: the reference's PROGRAM folder (required where the reference is read)
REF = os.environ.get("EA_REF", "")
# EA_REFGOLD_OUT: folder, relative to the repository root, that the GPU host
# hands back with the reference outputs (required by stage and collect)
OUT = os.environ.get("EA_REFGOLD_OUT", "")
MASTERS = (81985529216486895, 1147797409030816545, 1229782938247303441, 6148914691236517205)

# tag: L, Lz, BC, cluster, lut-set, isample, nbits, list_samples, nbin, itmax, houfr, mesfr, ptfr, resume_nbin
CASES = {
    "r1_L8_Lz8_PBC_nocl": (8, 8, "PBC", 0, "T08_16_N4", 3, 2, None, 3, 4, 1, 2, 2, 5),
    "r2_L8_Lz16_OBC": (8, 16, "OBC", 1, "T07_16_N6", 0, 3, [1, 4, 7], 2, 4, 2, 2, 1, 3),
    "r3_L8_Lz16_WEAK": (8, 16, "WEAK", 1, "T07_16_N6", 11, 2, None, 2, 2, 3, 1, 1, 0),
    "r4_L16_Lz24_STRONG": (16, 24, "STRONG", 1, "T07_16_N8", 5, 2, None, 2, 2, 1, 2, 3, 0),
    "r5_L16_Lz48_OBC_NB40": (16, 48, "OBC", 1, "shipped_N40", 0, 1, None, 1, 2, 2, 2, 1, 0),
    "r6_L24_Lz192_OBC_NB32": (24, 192, "OBC", 1, "T06_16_N32", 2, 2, None, 1, 1, 5, 1, 1, 0),
}
# timing runs of the reference binary (same geometry as bench.py): tag, nbits, nbin, itmax, houfr
TIMING = {"t1_L24_Lz192_OBC_NB32_ns31": (31, 3, 100, 5)}


def case_inputs(tag, dirpath):
    """Write the input files of case `tag` into dirpath (LUT rebuilt from the
    committed thresholds and checked against the generator's file digest)."""
    sys.path.insert(0, os.path.dirname(HERE))
    import refflow
    if tag in CASES:
        L, Lz, BC, cl, lutname, isample, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, resume = CASES[tag]
    else:
        (nbits, nbin, itmax, houfr), (L, Lz, lutname, lst, mesfr, ptfr) = TIMING[tag], (24, 192, "T06_16_N32", None, 1, 1)
    d = np.load(os.path.join(HERE, "lut_%s.npz" % lutname))
    assert hashlib.sha256(refflow.lut_bytes(d["betas"], d["cum"])).digest() == d["file_sha256"].tobytes()
    refflow.write_case_inputs(dirpath, L, Lz, d["betas"], d["cum"], nbits, lst, nbin, itmax, houfr, mesfr, ptfr,
                              MASTERS)
    return len(d["betas"])


def stage():
    if not REF or not os.path.isdir(REF):
        sys.exit("set EA_REF to the reference's PROGRAM folder")
    if not OUT:
        sys.exit("set EA_REFGOLD_OUT to the folder the GPU host hands back")
    shutil.rmtree(RUNS, ignore_errors=True)
    subprocess.run(["make", "-s", "-C", ORACLE, "ref-stage", "REF=" + REF], check=True)
    lines = ["#!/bin/bash", "# builds and runs the reference binary for every golden case (GPU host)",
             "set -u", "cd \"$(dirname \"$0\")/../../..\"", "R=$PWD", "mkdir -p %s" % OUT,
             "nvidia-smi -L > %s/gpu.txt 2>&1" % OUT, "builds=()"]
    runs = []
    for tag, (L, Lz, BC, cl, lutname, isample, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, resume) in CASES.items():
        nb = case_inputs(tag, os.path.join(RUNS, tag))
        cfg = "%d,%d,%d,%s" % (L, Lz, nb, BC)
        exe = "oracle/_ref/bin/EA_L%d_Lz%d_NB%d_%s%s" % (L, Lz, nb, BC, "" if cl else "_NOCL")
        lines.append("make -s -C oracle ref-cuda CFG=%s CLUSTER=%d > %s/build_%s.log 2>&1 &" % (cfg, cl, OUT, tag))
        args = "%d %d betas input.in LUT 0 0%s" % (isample, nbits, " list" if lst else "")
        runs.append((tag, exe, args, resume))
    for tag, (nbits, nbin, itmax, houfr) in TIMING.items():
        nb = case_inputs(tag, os.path.join(RUNS, tag))
        runs.append((tag, "oracle/_ref/bin/EA_L24_Lz192_NB%d_OBC" % nb, "0 %d betas input.in LUT 0 0" % nbits, 0))
    lines.append("wait")
    for tag, exe, args, resume in runs:
        lines.append("( cd oracle/_ref/runs/%s && \"$R/%s\" %s > run.log 2>&1 ; echo rc=$? >> run.log )" % (tag, exe, args))
        if resume:
            lines.append("( cd oracle/_ref/runs/%s && sed -i '2s/.*/%d/;9s/.*/0/' input.in && \"$R/%s\" %s > resume.log 2>&1 ; echo rc=$? >> resume.log )" % (tag, resume, exe, args))
        lines.append("mkdir -p %s/%s && cp -r oracle/_ref/runs/%s/. %s/%s/ && rm -f %s/%s/LUT" % (OUT, tag, tag, OUT, tag, OUT, tag))
    with open(os.path.join(RUNS, "run_all.sh"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print("staged", len(runs), "cases in", RUNS)


def collect():
    if not OUT:
        sys.exit("set EA_REFGOLD_OUT to the folder the GPU host handed back")
    src = os.path.join(ROOT, OUT)
    for tag in CASES:
        base = os.path.join(src, tag)
        if not os.path.isdir(base):
            print("missing", tag)
            continue
        out = {}
        for dp, _, files in os.walk(base):
            for fn in sorted(files):
                rel = os.path.relpath(os.path.join(dp, fn), base)
                # `conf` is a hard link to the newest conf.%06d (io.c:73-86)
                if fn in ("LUT", "conf") or fn.startswith(("running", "time.log")):
                    continue
                raw = open(os.path.join(dp, fn), "rb").read()
                key = rel.replace("/", "|")
                if len(raw) <= 65536:
                    out["file:" + key] = np.frombuffer(raw, np.uint8).copy()
                else:
                    out["sha256:" + key] = np.frombuffer(hashlib.sha256(raw).digest(), np.uint8)
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % tag), **out)
        print("wrote ref_%s.npz (%d files)" % (tag, len(out)))


if __name__ == "__main__":
    {"stage": stage, "collect": collect}[sys.argv[1]]()
