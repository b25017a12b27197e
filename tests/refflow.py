"""The reference driver's flow (PROGRAM/src/main.cu:10-283, io.c) on top of the
CPU oracle, writing the reference's output tree: couplings.bin, seeds.in,
master_seeds.in, conf.%06d (+ conf hard link), evol.txt, aceptancePT.txt and
history_b.dat.  Test infrastructure: it pins the oracle against the output
files of the reference binary (tests/golden/ref_*.npz) and is the model the
command-line driver of the library is checked against.

New runs (flag 1) and restarts from conf (flag 0) are covered; run
management (locks, signals, changenbin.in, time budget) is not.
"""
import ctypes as C
import os
import struct

import numpy as np

import oracle_py as O

MAXNSAMPLES = 32


def read_input(path):
    """read_input (io.c:399-436): directory line, nine ints, four 64-bit seeds."""
    lines = open(path).read().splitlines()
    d = {"dir": lines[0].split()[0]}
    names = ["nbin", "itcut", "itmax", "houfr", "mesfr", "ptfr", "nbetas", "flag", "l"]
    for i, n in enumerate(names):
        d[n] = int(lines[1 + i].split()[0])
    for i, n in enumerate(["seed_J", "seed_u", "seed_MC", "seed_Cluster"]):
        d[n] = int(lines[10 + i].split()[0])
    d["L"], d["Lz"] = d["l"] & 0xFFFF, d["l"] >> 16
    return d


def read_betas(path, nb):
    return np.array([float(x) for x in open(path).read().split()[:nb]])


def read_lut(path, nb):
    raw = open(path, "rb").read()
    b = np.frombuffer(raw[:8 * nb], np.float64)
    per = (128 + 512) * 16
    cum = np.zeros((nb, 256), np.uint64)
    for i in range(nb):
        u = np.frombuffer(raw[8 * nb + i * per: 8 * nb + i * per + 2048], np.uint32).reshape(256, 2)
        cum[i] = (u[:, 0].astype(np.uint64) << np.uint64(32)) | u[:, 1].astype(np.uint64)
    return b, cum


def sdata(d, seed_J, seed_u, seed_MC, seed_C):
    """s_data as written in conf files (header.h:86-100): 9 int32, padding, 4 uint64."""
    return struct.pack("<9i4x4Q", d["nbin"], d["itcut"], d["itmax"], d["houfr"], d["mesfr"], d["ptfr"],
                       d["nbetas"], d["flag"], d["l"], seed_J, seed_u, seed_MC, seed_C)


def frec_trw(itmax):
    for f in range(1, itmax + 1):
        if itmax % f == 0 and itmax // f <= 512:
            return f, itmax // f
    return 1, itmax


def janus_pack(g, uu_r):
    """Janus_packing_for_write (io.c:242-261): clone-major, bit site & 7 of byte site >> 3."""
    bits = uu_r.reshape(g.NB, g.V // 8, 8).astype(np.uint8)
    return np.packbits(bits, axis=2, bitorder="little").reshape(-1).tobytes()


def janus_unpack(g, raw):
    b = np.frombuffer(raw, np.uint8).reshape(g.NB, g.V // 8, 1)
    return np.unpackbits(b, axis=2, bitorder="little").reshape(-1).astype(np.uint8)


def fmt_g(x):
    return "%g" % x


def run(workdir, isample, nbits, betas_path, input_path, lut_path, list_path=None, bc=None, cluster=True):
    """Run the reference flow with the oracle inside `workdir` (as the cwd of the
    reference binary).  Returns the sample directory."""
    d = read_input(input_path)
    L, Lz, NB, NR = d["L"], d["Lz"], d["nbetas"], 8
    betas = read_betas(betas_path, NB)
    lb, cum = read_lut(lut_path, NB)
    assert np.all(np.abs(lb - betas) <= 1e-14)
    lst = list(range(nbits)) if not list_path else [int(x) for x in open(list_path).read().split()[:nbits]]
    base = os.path.join(workdir, "I%03d" % isample)   # see create_sample_path, io.c:573
    os.makedirs(base, exist_ok=True)
    dirs = [os.path.join(base, "BIT%03d" % s) for s in lst]
    rdirs = [[os.path.join(dirs[i], "R%02d" % r) for r in range(NR)] for i in range(nbits)]
    for i in range(nbits):
        for r in range(NR):
            os.makedirs(rdirs[i][r], exist_ok=True)
    there_is_conf = os.path.exists(os.path.join(rdirs[0][0], "conf"))
    if d["flag"] == 2:
        d["flag"] = 0 if there_is_conf else 1
    masters = (d["seed_J"], d["seed_u"], d["seed_MC"], d["seed_Cluster"])
    sim = O.Sim(L, Lz, betas, cum, nbits=nbits, NR=NR, bc=bc, masters=masters, list_samples=lst, itmax=d["itmax"])
    g = sim.g
    countJ0 = sim.countJ
    for i in range(nbits):
        with open(os.path.join(dirs[i], "couplings.bin"), "wb") as f:
            f.write(sim.J6[i].tobytes())
    if d["flag"] == 1:
        with open(os.path.join(base, "master_seeds.in"), "w") as f:
            f.write("%d %d %d %d\n" % masters)
        for i in range(nbits):
            with open(os.path.join(dirs[i], "seeds.in"), "w") as f:
                f.write("%d %d" % (sim.sd.seeds_J[i], sim.sd.seeds_u[i]))
                for r in range(NR):
                    f.write(" %d" % sim.sd.seeds_MC[r])
                f.write(" %d" % d["seed_Cluster"])
                f.write(" %d\n" % countJ0[i])
    else:
        # read_conf (io.c:105-240)
        uu = np.zeros((nbits, NR, NB * g.V), np.uint8)
        for i in range(nbits):
            for r in range(NR):
                raw = open(os.path.join(rdirs[i][r], "conf"), "rb").read()
                p = 0
                hdr = struct.unpack_from("<9i4x4Q", raw, p); p += 72
                d["itcut"] = hdr[1]
                p += 8 * NB
                sim.pt[i * NR + r] = O.HQ.from_buffer_copy(raw[p:p + 2080]); p += 2080
                sim.prc[r] = O.HQ.from_buffer_copy(raw[p:p + 2080]); p += 2080
                sim.rc = O.HQ.from_buffer_copy(raw[p:p + 2080]); p += 2080
                sim.xo[r] = O.XO.from_buffer_copy(raw[p:p + 48]); p += 48
                sim.cuda_rng_offset, = struct.unpack_from("<Q", raw, p); p += 8
                sim.wctb[i, r] = np.frombuffer(raw[p:p + NB], np.uint8); p += NB
                sim.wbtc[i, r][sim.wctb[i, r]] = np.arange(NB, dtype=np.uint8)
                uu[i, r] = janus_unpack(g, raw[p:p + NB * g.V // 8])
        for i in range(nbits):
            ev, od = O.pack_spins(g, uu[i].reshape(-1))
            sim.spins[i, 0] = ev
            sim.spins[i, 1] = od
    # iter restarts without the houfr factor (main.cu:139)
    it = 2 * d["itcut"] * d["itmax"] * d["mesfr"] * d["ptfr"]
    frec, maxit = frec_trw(d["itmax"])
    for ibin in range(d["itcut"], d["nbin"]):
        it = sim.run_bin(d["itmax"], d["houfr"], d["mesfr"], d["ptfr"], it, jobid=isample, cluster=cluster)
        avg = sim.avgE / d["itmax"]
        for i in range(nbits):
            for r in range(NR):
                # opened for append (io.c:377): writes land at the end of the file
                with open(os.path.join(rdirs[i][r], "history_b.dat"), "ab") as f:
                    f.write(sim.hist[i, r].tobytes())
                with open(os.path.join(rdirs[i][r], "evol.txt"), "a") as f:
                    f.write("%d " % ibin + "".join("%14.10g " % v for v in avg[i, r]) + "\n")
                with open(os.path.join(rdirs[i][r], "aceptancePT.txt"), "a") as f:
                    f.write("#%d\n" % ibin)
                    for b in range(NB - 1):
                        att = sim.att[i, r, b]
                        f.write("%s %s %s %s\n" % (fmt_g(betas[b]), fmt_g(sim.acc[i, r, b] / att),
                                                   fmt_g(sim.accraw[i, r, b] / att), fmt_g(att)))
        d["itcut"] += 1
        uu = [O.unpack_spins(g, sim.spins[i, 0], sim.spins[i, 1]).reshape(NR, NB * g.V) for i in range(nbits)]
        for i in range(nbits):
            for r in range(NR):
                raw = sdata(d, int(sim.sd.seeds_J[i]), int(sim.sd.seeds_u[i]), int(sim.sd.seeds_MC[r]), d["seed_Cluster"])
                raw += betas.astype(np.float64).tobytes()
                raw += O.as_bytes(sim.pt[i * NR + r]) + O.as_bytes(sim.prc[r]) + O.as_bytes(sim.rc)
                raw += O.as_bytes(sim.xo[r]) + struct.pack("<Q", sim.cuda_rng_offset)
                raw += sim.wctb[i, r].tobytes()
                raw += janus_pack(g, uu[i][r])
                raw += np.array([sim.E[i, r, c] for c in sim.wctb[i, r]], np.int32).tobytes()
                name = os.path.join(rdirs[i][r], "conf.%06d" % d["itcut"])
                with open(name, "wb") as f:
                    f.write(raw)
                link = os.path.join(rdirs[i][r], "conf")
                if os.path.exists(link):
                    os.remove(link)
                os.link(name, link)
    return base


def lut_bytes(betas, cum, nbits_pre=12):
    """LUT file (create_LUT.c:402-417) from the cumulative thresholds: betas, then per
    beta 128 uint4 of thresholds and the pre-search table (create_LUT.c:320-376)."""
    out = np.asarray(betas, np.float64).tobytes()
    npre = 1 << nbits_pre
    tail = np.uint64((1 << (64 - nbits_pre)) - 1)
    for c in np.asarray(cum, np.uint64):
        out += np.stack([(c >> np.uint64(32)).astype(np.uint32), (c & np.uint64(0xFFFFFFFF)).astype(np.uint32)],
                        axis=1).reshape(-1).tobytes()
        t = np.arange(npre, dtype=np.uint64) << np.uint64(64 - nbits_pre)
        tmin = np.minimum(np.searchsorted(c, t, side="right"), 255).astype(np.uint32)
        tmax = np.minimum(np.searchsorted(c, t | tail, side="right"), 255).astype(np.uint32)
        pairs = (tmin | (tmax << 8)).astype(np.uint16)
        out += pairs.tobytes()
    return out


def write_case_inputs(dirpath, L, Lz, betas, cum, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, masters, flag=1):
    """The input files the reference reads: input.in, betas, LUT and the optional sample list."""
    os.makedirs(dirpath, exist_ok=True)
    with open(os.path.join(dirpath, "LUT"), "wb") as f:
        f.write(lut_bytes(betas, cum))
    with open(os.path.join(dirpath, "betas"), "w") as f:
        for b in betas:
            f.write("%.17g\n" % b)
    with open(os.path.join(dirpath, "input.in"), "w") as f:
        f.write("./\n")
        for v in (nbin, 0, itmax, houfr, mesfr, ptfr, len(betas), flag, (Lz << 16) | L):
            f.write("%d\n" % v)
        for m in masters:
            f.write("%d\n" % m)
    if lst:
        with open(os.path.join(dirpath, "list"), "w") as f:
            f.write("\n".join(str(x) for x in lst) + "\n")


def set_resume(dirpath, nbin):
    """The restart the golden runs make: nbin raised, flag 0 (backup)."""
    p = os.path.join(dirpath, "input.in")
    lines = open(p).read().splitlines()
    lines[1] = str(nbin)
    lines[8] = "0"
    open(p, "w").write("\n".join(lines) + "\n")
