"""ctypes view of the CPU oracle (oracle/libea_oracle.so).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's
reference leg use this module.  It builds the oracle on first use.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "libea_oracle.so")

PBC, OBC, OBC_WEAK, OBC_STRONG = 0, 1, 2, 3
BC_NAMES = {"PBC": PBC, "OBC": OBC, "WEAK": OBC_WEAK, "STRONG": OBC_STRONG}


class HQ(C.Structure):
    _fields_ = [("ira", C.c_uint64 * 256), ("PR", C.c_uint64), ("zseed", C.c_uint64),
                ("final", C.c_uint64), ("ip", C.c_uint8), ("ip1", C.c_uint8), ("ip2", C.c_uint8),
                ("ip3", C.c_uint8), ("padding", C.c_uint8 * 4)]


class XO(C.Structure):
    _fields_ = [("s", C.c_uint64 * 4), ("t", C.c_uint64), ("final", C.c_uint64)]


class Geom(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("L", "Lz", "NB", "NR", "nbits", "bc", "msc_l", "msc_lz",
                                        "msc_s", "msc_v", "half", "V")]


class Seeds(C.Structure):
    _fields_ = [("seeds_J", C.c_uint64 * 32), ("seeds_u", C.c_uint64 * 32),
                ("seeds_MC", C.c_uint64 * 64), ("seed_cluster", C.c_uint64)]


class RunCfg(C.Structure):
    _fields_ = [("nbin", C.c_int), ("itcut", C.c_int), ("itmax", C.c_int), ("houfr", C.c_int),
                ("mesfr", C.c_int), ("ptfr", C.c_int), ("jobid", C.c_uint32), ("cluster", C.c_int),
                ("nclust", C.c_int), ("nthreads", C.c_int), ("cluster_exact", C.c_int)]


P = C.c_void_p


class State(C.Structure):
    _fields_ = [("g", Geom), ("spins", P), ("Jw", P), ("wctb", P), ("wbtc", P), ("E", P),
                ("acc", P), ("att", P), ("accraw", P), ("avgE", P), ("hist", P), ("prc", P),
                ("xo", P), ("keys", P), ("pt", P), ("rc", HQ), ("cuda_rng_offset", C.c_uint64),
                ("seed_cluster", C.c_uint64), ("betas", P), ("cum", P), ("frec_trw", C.c_int),
                ("maxit_trw", C.c_int), ("curand_gen", P)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(ORACLE_DIR, f) for f in ("ea_oracle.c", "sp_oracle.c", "ea_oracle.h")]
        if (not os.path.exists(LIB_PATH)) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(f) for f in srcs):
            subprocess.run(["make", "-s", "-C", ORACLE_DIR, "libea_oracle.so"], check=True)
        _lib = C.CDLL(LIB_PATH)
        _lib.or_hq_next.restype = C.c_uint64
        _lib.or_xo_next.restype = C.c_uint64
        _lib.or_geom_init.restype = C.c_int
        _lib.or_init_couplings.restype = C.c_int
        _lib.or_scalar_energy.restype = C.c_int
        _lib.or_lut_search.restype = C.c_int
        _lib.or_lut_beta.restype = C.c_int
        _lib.or_run_bin.restype = C.c_int
    return _lib


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def geom(L, Lz, NB, NR=8, nbits=1, bc=OBC):
    g = Geom()
    if lib().or_geom_init(C.byref(g), L, Lz, NB, NR, nbits, bc) != 0:
        raise ValueError("L and Lz must be multiples of 8")
    return g


def hq_array(n):
    return (HQ * n)()


def as_bytes(obj):
    return bytes(memoryview(obj).cast("B"))


def init_run(g, masters, list_samples=None):
    """Seeds and generator states of a new run (flag 1), as the reference builds them."""
    L = lib()
    nb = g.nbits
    ls = np.arange(nb, dtype=np.int32) if list_samples is None else np.asarray(list_samples, np.int32)
    sd = Seeds()
    L.or_generate_seed_vectors(C.c_uint64(masters[0]), C.c_uint64(masters[1]), C.c_uint64(masters[2]),
                               ptr(ls), nb, g.NR, C.byref(sd))
    sd.seed_cluster = masters[3]
    prc = hq_array(g.NR)
    xo = (XO * g.NR)()
    keys = np.zeros(g.NR, np.uint32)
    pt = hq_array(nb * g.NR)
    rc = HQ()
    L.or_init_random(C.byref(sd), ptr(ls), nb, g.NR, prc, xo, ptr(keys), pt, C.byref(rc))
    return sd, prc, xo, keys, pt, rc


def tables(g):
    neig = np.zeros(12 * g.half, np.int32)
    rot = np.zeros(2 * g.half, np.uint8)
    bi = np.zeros(g.half, np.uint32)
    ne = np.zeros(g.half, np.uint32)
    lib().or_tables(C.byref(g), ptr(neig), ptr(rot), ptr(bi), ptr(ne))
    return neig, rot, bi, ne


def init_spins(g, seed_u):
    uu = np.zeros(g.NR * g.NB * g.V, np.uint8)
    lib().or_init_spins(C.byref(g), C.c_uint64(seed_u), ptr(uu))
    return uu


def pack_spins(g, uu):
    n = g.NB * g.half * g.NR
    ev = np.zeros(n, np.uint64)
    od = np.zeros(n, np.uint64)
    lib().or_pack_spins(C.byref(g), ptr(uu), ptr(ev), ptr(od))
    return ev, od


def unpack_spins(g, ev, od):
    uu = np.zeros(g.NR * g.NB * g.V, np.uint8)
    lib().or_unpack_spins(C.byref(g), ptr(np.ascontiguousarray(ev)), ptr(np.ascontiguousarray(od)), ptr(uu))
    return uu


def init_couplings(g, seed_J):
    J6 = np.zeros(6 * g.V, np.uint8)
    cnt = lib().or_init_couplings(C.byref(g), C.c_uint64(seed_J), ptr(J6))
    return J6, cnt


def pack_couplings(g, J6):
    Jw = np.zeros(12 * g.half, np.uint64)
    lib().or_pack_couplings(C.byref(g), ptr(J6), ptr(Jw))
    return Jw


def lut_beta(beta, nbits_pre=12):
    cum = np.zeros(256, np.uint64)
    umb = np.zeros(512, np.uint32)
    pre = np.zeros((1 << nbits_pre) // 2, np.uint32)
    if lib().or_lut_beta(C.c_double(beta), nbits_pre, ptr(cum), ptr(umb), ptr(pre)) != 0:
        raise RuntimeError("quad precision unavailable in this oracle build")
    return cum, umb, pre


def fill_bits(prc, xo, NR, it, jobid):
    ctr = np.zeros(4 * NR, np.uint32)
    lib().or_fill_bits(prc, xo, NR, C.c_uint64(it), C.c_uint32(jobid), ptr(ctr))
    return ctr


class Sim:
    """Whole-run oracle state in the reference layout (one process of the reference)."""

    def __init__(self, L, Lz, betas, cum, nbits=1, NR=8, bc=OBC, masters=(1, 2, 3, 4),
                 list_samples=None, itmax=1):
        self.g = geom(L, Lz, len(betas), NR, nbits, bc)
        g = self.g
        self.betas = np.ascontiguousarray(betas, np.float64)
        self.cum = np.ascontiguousarray(cum, np.uint64).reshape(-1)
        self.sd, self.prc, self.xo, self.keys, self.pt, self.rc = init_run(g, masters, list_samples)
        NB, half = g.NB, g.half
        self.spins = np.zeros((nbits, 2, NB * half * NR), np.uint64)
        self.J6 = np.zeros((nbits, 6 * g.V), np.uint8)
        self.Jw = np.zeros((nbits, 12 * half), np.uint64)
        self.countJ = []
        for s in range(nbits):
            uu = init_spins(g, self.sd.seeds_u[s])
            ev, od = pack_spins(g, uu)
            self.spins[s, 0] = ev
            self.spins[s, 1] = od
            J6, cnt = init_couplings(g, self.sd.seeds_J[s])
            self.J6[s] = J6
            self.countJ.append(cnt)
            self.Jw[s] = pack_couplings(g, J6)
        self.wctb = np.tile(np.arange(NB, dtype=np.uint8), (nbits, NR, 1)).copy()
        self.wbtc = self.wctb.copy()
        self.E = np.zeros((nbits, NR, NB), np.int32)
        self.acc = np.zeros((nbits, NR, NB - 1))
        self.att = np.zeros_like(self.acc)
        self.accraw = np.zeros_like(self.acc)
        self.avgE = np.zeros((nbits, NR, NB))
        for f in range(1, itmax + 1):
            if itmax % f == 0 and itmax // f <= 512:
                self.frec_trw, self.maxit_trw = f, itmax // f
                break
        self.hist = np.zeros((nbits, NR, self.maxit_trw, NB), np.uint8)
        self.cuda_rng_offset = 0
        self.curand_gen = None

    def __del__(self):
        try:
            if self.curand_gen:
                st = self.state()
                lib().or_state_release(C.byref(st))
        except Exception:
            pass

    def state(self):
        st = State()
        st.g = self.g
        for name in ("spins", "Jw", "wctb", "wbtc", "E", "acc", "att", "accraw", "avgE", "hist", "keys",
                     "betas", "cum"):
            setattr(st, name, ptr(getattr(self, name)))
        st.prc = C.cast(self.prc, C.c_void_p)
        st.xo = C.cast(self.xo, C.c_void_p)
        st.pt = C.cast(self.pt, C.c_void_p)
        st.rc = self.rc
        st.cuda_rng_offset = self.cuda_rng_offset
        st.seed_cluster = self.sd.seed_cluster
        st.frec_trw = self.frec_trw
        st.maxit_trw = self.maxit_trw
        st.curand_gen = self.curand_gen
        return st

    def run_bin(self, itmax, houfr, mesfr, ptfr, iter0, jobid=0, cluster=True, nclust=None,
                nthreads=0, cluster_exact=False):
        st = self.state()
        cfg = RunCfg(1, 0, itmax, houfr, mesfr, ptfr, jobid, int(cluster),
                     nclust if nclust is not None else int(np.floor(self.g.NB * 0.5 + 0.5)), nthreads,
                     int(cluster_exact))
        it = C.c_uint64(iter0)
        rc = lib().or_run_bin(C.byref(st), C.byref(cfg), C.byref(it))
        if rc != 0:
            raise RuntimeError("oracle run failed %d" % rc)
        self.rc = st.rc
        self.cuda_rng_offset = st.cuda_rng_offset
        self.curand_gen = st.curand_gen
        return it.value

    def half_sweep(self, ctr, parity, nthreads=0):
        lib().or_half_sweep(C.byref(self.g), ptr(self.spins), ptr(self.Jw), ptr(self.wbtc), ptr(ctr),
                            ptr(self.keys), ptr(self.cum), parity, nthreads)

    def energy(self):
        E = np.zeros((self.g.nbits, self.g.NR, self.g.NB), np.int32)
        lib().or_energy(C.byref(self.g), ptr(self.spins), ptr(self.Jw), ptr(E))
        return E


def curand_host(seed, offset, n):
    out = np.zeros(n, np.float64)
    if lib().or_curand_host(C.c_uint64(seed), C.c_uint64(offset), C.c_uint64(n), ptr(out)) != 0:
        raise RuntimeError("cuRAND host generator failed")
    return out


# ---------------------------------------------------------------------------
# Sample-packed layout (oracle/sp_oracle.c)
# ---------------------------------------------------------------------------
_exp_tables = {}


def sp_exp_table(betas):
    """exp(pt) of every tempering exponent that can change a decision, with
    the host libm, per beta pair (offsets) -- dE = -2, -4, ... down to pt = -50."""
    key = np.ascontiguousarray(betas, np.float64).tobytes()
    if key in _exp_tables:
        return _exp_tables[key]
    vals, off = [], []
    for i in range(len(betas) - 1):
        off.append(len(vals))
        j = 1
        while True:
            dE = float(-2 * j)
            pt = -(float(betas[i + 1]) - float(betas[i])) * dE
            if not pt < 0 or pt < -50.0 or j > (1 << 22):
                break
            vals.append(math.exp(pt))
            j += 1
    off.append(len(vals))
    _exp_tables[key] = (np.array(vals, np.float64), np.array(off, np.int32))
    return _exp_tables[key]


def sp_pass(V, NR, NB, nw, nb, sites, ctr, keys, cum, J, S):
    lib().or_sp_pass(V, NR, NB, nw, ptr(nb), ptr(sites), len(sites), ptr(ctr), ptr(keys), ptr(cum), ptr(J), ptr(S))


def sp_energy(V, NR, NB, nw, nb, J, S):
    U2 = np.zeros((nw, 64, NR, NB), np.int32)
    lib().or_sp_energy(V, NR, NB, nw, ptr(nb), ptr(J), ptr(S), ptr(U2))
    return U2


def sp_pt(V, NR, NB, nw, betas, step, seed, U2, perm, acc, S):
    """One tempering step (in place on perm, acc and S); returns E, masks."""
    tab, off = sp_exp_table(betas)
    E = np.zeros((nw, 64, NR, NB), np.int32)
    masks = np.zeros((nw, NR, NB - 1), np.uint64)
    b = np.ascontiguousarray(betas, np.float64)
    lib().or_sp_pt(V, NR, NB, nw, ptr(b), ptr(tab), ptr(off), C.c_uint64(step), C.c_uint64(seed), ptr(U2), ptr(E),
                   ptr(perm), ptr(acc), ptr(masks), ptr(S))
    return E, masks


def sp_dos(V, nb, J, w, lane):
    h = np.zeros(6 * V + 1, np.uint64)
    lib().or_sp_dos(V, ptr(nb), ptr(J), w, lane, ptr(h))
    return h


def sp_cluster(V, NR, NB, nw, nb, nclust, g, r1, r2, move, key, S):
    lib().or_sp_cluster(V, NR, NB, nw, ptr(nb), nclust, g, r1, r2, C.c_uint64(move), C.c_uint64(key), ptr(S))
