#!/usr/bin/env python3
"""Generate host-side golden fixtures from the reference's own code.

Runs only where the reference tree is present (it reads the reference sources
in the folder EA_REF names, the reference's PROGRAM folder, through
oracle/Makefile).  For each geometry below
it compiles the reference host code (random_generator.cu, ini.c, io.c, upd.c,
med.c) with oracle/ref_host_harness.cpp, runs it with fixed master seeds and
stores what it computed in tests/golden/host_<TAG>.npz.  It also compiles the
reference LUT generator (input/create_LUT.c) and stores the cumulative
thresholds of each temperature set in tests/golden/lut_<name>.npz.

Small arrays are stored whole; arrays above 64 KiB are stored as SHA-256
digests (key "sha256:<name>").
"""
import hashlib
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")
# EA_REF: the reference's PROGRAM folder (required where the reference is read)
REF = os.environ.get("EA_REF", "")

MASTERS = (81985529216486895, 1147797409030816545, 1229782938247303441, 6148914691236517205)

# name, L, Lz, NB, BC, nbits, beta-set name
CONFIGS = [
    ("L8_Lz8_NB4_PBC", 8, 8, 4, "PBC", 2, "T08_16_N4"),
    ("L8_Lz16_NB6_OBC", 8, 16, 6, "OBC", 3, "T07_16_N6"),
    ("L8_Lz16_NB6_WEAK", 8, 16, 6, "WEAK", 2, "T07_16_N6"),
    ("L16_Lz24_NB8_STRONG", 16, 24, 8, "STRONG", 2, "T07_16_N8"),
    ("L16_Lz48_NB40_OBC", 16, 48, 40, "OBC", 1, "shipped_N40"),
    ("L24_Lz192_NB32_OBC", 24, 192, 32, "OBC", 1, "T06_16_N32"),
]

# temperature sets of the mixed-geometry (batched vs plain) and serving workloads
EXTRA_LUTS = ["T07_16_N16", "T07_16_N24", "T07_16_N32", "T07_16_N8", "T07_16_N12", "T08_16_N12"]


def beta_set(name):
    """Temperatures uniform in [Tmin, Tmax]; betas written descending with 13 decimals."""
    if name == "shipped_N40":
        with open(os.path.join(REF, "input", "betas_T07_T20_N40")) as f:
            return np.array([float(x) for x in f.read().split()])
    t = name.split("_")
    tmin, tmax, n = int(t[0][1:]) / 10.0, int(t[1]) / 10.0, int(t[2][1:])
    T = np.linspace(tmin, tmax, n)
    return np.array([float("%.13f" % (1.0 / x)) for x in T])


def write_betas(path, betas):
    with open(path, "w") as f:
        for b in betas:
            f.write("%.17g\n" % b)


def parse_dump(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        n, = struct.unpack_from("<I", data, p); p += 4
        name = data[p:p + n].decode(); p += n
        b, = struct.unpack_from("<Q", data, p); p += 8
        out[name] = data[p:p + b]; p += b
    return out


def store(d, name, raw, dtype):
    if len(raw) > 65536:
        d["sha256:" + name] = np.frombuffer(hashlib.sha256(raw).digest(), np.uint8)
    else:
        d[name] = np.frombuffer(raw, dtype).copy()


def lut_fixture(name, betas, work):
    nb = len(betas)
    bfile = os.path.join(work, "betas_" + name)
    if name == "shipped_N40":
        bfile = os.path.join(REF, "input", "betas_T07_T20_N40")
    else:
        write_betas(bfile, betas)
    subprocess.run(["make", "-s", "-C", ORACLE, "ref-lut", "CFG=8,8,%d,PBC" % nb, "REF=" + REF], check=True)
    exe = os.path.join(ORACLE, "_ref", "create_LUT_NB%d" % nb)
    res = subprocess.run([exe, bfile], cwd=work, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    refused = res.returncode != 0
    if refused:
        # create_LUT.c:87-217 aborts when a byte value has probability < 2^-64
        # (empty interval); the thresholds themselves are still defined, so the
        # oracle's restatement of prepara_LUT (create_LUT.c:265-388) builds them.
        sys.path.insert(0, os.path.dirname(HERE))
        import oracle_py
        raw = np.asarray(betas, np.float64).tobytes()
        for b in betas:
            cum, umb, pre = oracle_py.lut_beta(float(b))
            raw += umb.tobytes() + pre.tobytes()
    else:
        raw = open(os.path.join(work, "LUT_for_PRNG_nbits12_NB%d.bin" % nb), "rb").read()
    b = np.frombuffer(raw[:8 * nb], np.float64)
    per = (128 + 512) * 16
    cum = np.zeros((nb, 256), np.uint64)
    for i in range(nb):
        u = np.frombuffer(raw[8 * nb + i * per: 8 * nb + i * per + 2048], np.uint32).reshape(256, 2)
        cum[i] = (u[:, 0].astype(np.uint64) << np.uint64(32)) | u[:, 1].astype(np.uint64)
    d = {"betas": b.copy(), "cum": cum, "file_sha256": np.frombuffer(hashlib.sha256(raw).digest(), np.uint8),
         "ref_generator_refused": np.array([int(refused)], np.int32)}
    if name == "shipped_N40":
        shipped = open(os.path.join(REF, "input", "LUT_for_PRNG_nbits12_NB40.bin"), "rb").read()
        d["matches_shipped_file"] = np.array([int(shipped == raw)], np.int32)
    # the pre-search words of the first temperature, to pin the file layout
    d["prebusqueda0"] = np.frombuffer(raw[8 * nb + 2048: 8 * nb + per], np.uint32).copy()
    np.savez_compressed(os.path.join(HERE, "lut_%s.npz" % name), **d)
    return b


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("set EA_REF to the reference's PROGRAM folder")
    work = tempfile.mkdtemp(prefix="eagold_")
    if sys.argv[1:] == ["luts"]:
        for name in EXTRA_LUTS:
            lut_fixture(name, beta_set(name), work)
        return
    done_luts = {}
    for tag, L, Lz, NB, BC, nbits, bset in CONFIGS:
        if bset not in done_luts:
            done_luts[bset] = lut_fixture(bset, beta_set(bset), work)
        betas = done_luts[bset]
        subprocess.run(["make", "-s", "-C", ORACLE, "ref-host", "CFG=%d,%d,%d,%s" % (L, Lz, NB, BC), "REF=" + REF], check=True)
        exe = os.path.join(ORACLE, "_ref", "host_" + tag, "harness")
        rundir = os.path.join(work, tag)
        os.makedirs(rundir, exist_ok=True)
        bfile = os.path.join(rundir, "betas")
        write_betas(bfile, betas)
        dump = os.path.join(rundir, "dump.bin")
        # cwd=rundir: create_sample_path (io.c:573) formats `dir` into itself, which
        # drops the prefix with glibc, so the sample tree lands in the cwd.
        subprocess.run([exe, rundir, str(nbits)] + [str(m) for m in MASTERS] + [bfile, dump], check=True,
                       stdout=subprocess.DEVNULL, cwd=rundir)
        raw = parse_dump(dump)
        d = {"geom": np.array([L, Lz, NB, 8, nbits, {"PBC": 0, "OBC": 1, "WEAK": 2, "STRONG": 3}[BC]], np.int32),
             "masters": np.array(MASTERS, np.uint64), "betas": betas}
        for k, v in raw.items():
            if k == "geom":
                continue
            if k.startswith(("seeds", "even", "odd", "Jw", "ctr", "pt_state", "prc", "xo", "rc", "pt")) and not k.startswith(("pt_energies", "pt_perm", "pt_acc")):
                dt = np.uint32 if k.startswith(("ctr", "keys")) else np.uint64
                if k.startswith(("prc", "rc", "pt", "pt_state")):
                    dt = np.uint8
            elif k.startswith(("J6", "rot", "pt_perm")):
                dt = np.uint8
            elif k.startswith(("pt_acc",)):
                dt = np.float64
            else:
                dt = np.int32 if not k.startswith(("bianchi", "neri", "keys")) else np.uint32
            store(d, k, v, dt)
        np.savez_compressed(os.path.join(HERE, "host_%s.npz" % tag), **d)
        print("wrote host_%s.npz (%d entries)" % (tag, len(d)))


if __name__ == "__main__":
    main()
