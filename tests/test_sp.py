"""Sample-packed layout (ea_sp_*): 64 disorder samples per word, tubes of any
L >= 2 and Lz >= 2.

CPU: the bond graph (slots, fake bonds of the open planes, mates, colouring),
the couplings' symmetry, and the oracle's density of states against a plain
enumeration.  GPU: colour passes, energies, tempering steps and whole runs
bit for bit against the oracle (oracle/sp_oracle.c); the density of states
against the oracle; and the Monte Carlo <E>(T) at 3x3x3 against exact
enumeration of all 2^27 configurations, within its statistical error."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_py as O
from conftest import ROOT

import importlib.util

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)

GOLD = os.path.join(ROOT, "tests", "golden")
SEEDS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def lut(name):
    d = np.load(os.path.join(GOLD, "lut_%s.npz" % name))
    return d["betas"], d["cum"]


GEOMS = [(2, 2, eagb.EA_PBC), (3, 3, eagb.EA_PBC), (3, 3, eagb.EA_OBC), (4, 5, eagb.EA_PBC), (5, 7, eagb.EA_OBC),
         (6, 24, eagb.EA_PBC), (12, 48, eagb.EA_OBC), (7, 4, eagb.EA_OBC), (9, 2, eagb.EA_OBC), (2, 3, eagb.EA_OBC),
         (8, 16, eagb.EA_OBC)]


@pytest.mark.parametrize("L,Lz,bc", GEOMS)
def test_graph(L, Lz, bc):
    nb, mate, col, ncol = eagb.sp_graph(L, Lz, bc)
    V = L * L * Lz
    h = np.arange(6 * V)
    m = mate.reshape(-1)
    assert np.array_equal(m[m], h)                      # mates form an involution
    assert np.array_equal(nb.reshape(-1)[m], h // 6)    # the mate sits at the neighbour
    assert np.all(col[nb] != col[:, None])             # proper colouring (no self bonds)
    bip = L % 2 == 0 and (bc == eagb.EA_OBC or Lz % 2 == 0)
    assert ncol == (2 if bip else 3)
    x, y, z = np.arange(V) % L, (np.arange(V) // L) % L, np.arange(V) // (L * L)
    site = lambda xx, yy, zz: xx % L + L * (yy % L + L * (zz % Lz))
    assert np.array_equal(nb[:, 0], site(x + 1, y, z)) and np.array_equal(nb[:, 3], site(x - 1, y, z))
    assert np.array_equal(nb[:, 1], site(x, y + 1, z)) and np.array_equal(nb[:, 4], site(x, y - 1, z))
    inner_up = (bc == eagb.EA_PBC) | (z < Lz - 1)
    inner_dn = (bc == eagb.EA_PBC) | (z > 0)
    assert np.array_equal(nb[inner_up, 2], site(x, y, z + 1)[inner_up])
    assert np.array_equal(nb[inner_dn, 5], site(x, y, z - 1)[inner_dn])
    if bc == eagb.EA_OBC:
        top, bot = z == Lz - 1, z == 0
        if L % 2 == 0:
            # the reference's pairing: +y for even x+y+z, -y for odd
            even = (x + y + z) % 2 == 0
            want = np.where(even, site(x, y + 1, z), site(x, y - 1, z))
            assert np.array_equal(nb[top, 2], want[top]) and np.array_equal(nb[bot, 5], want[bot])
        else:
            corner = (x == L - 1) & (y == L - 1)
            assert np.array_equal(nb[top & corner, 2], site(x, y, 0)[top & corner])
            assert np.array_equal(nb[bot & corner, 5], site(x, y, Lz - 1)[bot & corner])


def test_colour_counts_all_small_tubes():
    """Every tube with L, Lz in 2..13 under PBC and OBC takes 2 colours when
    bipartite and 3 otherwise (the greedy fallback is never needed), and
    each colouring is proper."""
    for L in range(2, 14):
        for Lz in range(2, 14):
            for bc in (eagb.EA_PBC, eagb.EA_OBC):
                nb, mate, col, ncol = eagb.sp_graph(L, Lz, bc)
                bip = L % 2 == 0 and (bc == eagb.EA_OBC or Lz % 2 == 0)
                assert ncol == (2 if bip else 3), (L, Lz, bc, ncol)
                assert np.all(col[nb] != col[:, None])


@pytest.mark.parametrize("ln", ["T06_16_N32", "T07_16_N24", "T08_16_N12"])
def test_presearch11_brackets_every_key(ln):
    """The 11-bit pre-search of the per-item pass: entry t is the byte of
    the bucket's smallest key (the first n with key < cum[n]), the padding
    is 255, and every key's byte lies between its bucket's entry and the
    next one -- at the bucket edges and for random keys."""
    betas, cum = lut(ln)
    rng = np.random.default_rng(5)

    def byte(R):  # the reference's search: first n with R < cum[n], at most 255
        return np.minimum(np.searchsorted(c, R, side="right"), 255)

    for c in np.asarray(cum, np.uint64)[::7]:
        pre = eagb.sp_presearch11(c)
        edges = np.arange(2048, dtype=np.uint64) << np.uint64(53)
        assert np.array_equal(pre[:2048], byte(edges))
        assert np.all(pre[2048:] == 255)
        R = np.concatenate([rng.integers(0, 2**64, 200000, dtype=np.uint64, endpoint=False),
                            edges, edges + np.uint64((1 << 53) - 1), c[:255], c[:255] - np.uint64(1)])
        t = (R >> np.uint64(53)).astype(np.int64)
        b = byte(R)
        assert np.all(pre[t] <= b) and np.all(b <= pre[t + 1])
    with pytest.raises(RuntimeError):
        bad = np.array(c, np.uint64)
        bad[255] = 1
        eagb.sp_presearch11(bad)


def test_couplings_and_spins():
    g = eagb.SpGeom(5, 7, 4, 3, 2, eagb.EA_OBC)
    nb, mate, col, ncol = eagb.sp_graph(5, 7, eagb.EA_OBC)
    J, S = eagb.sp_host_init(g, 11, 22)
    Jf = J.reshape(2, -1)
    assert np.array_equal(Jf[:, mate.reshape(-1)], Jf)  # both ends of a bond hold the same word
    assert J.shape == (2, 5 * 5 * 7, 6) and S.shape == (2, 5 * 5 * 7, 3, 4)
    # couplings are +-J with p = 1/2 per bit
    bits = np.unpackbits(Jf.view(np.uint8)).mean()
    assert abs(bits - 0.5) < 0.01
    J2, S2 = eagb.sp_host_init(g, 11, 22)
    assert np.array_equal(J, J2) and np.array_equal(S, S2)
    # the streams themselves are pinned: words may be generated in any order
    # or in parallel, never differently
    import hashlib
    g5 = eagb.SpGeom(5, 7, 4, 3, 5, eagb.EA_OBC)
    J5, S5 = eagb.sp_host_init(g5, 11, 22)
    assert hashlib.sha256(J5.tobytes()).hexdigest()[:32] == "6b126edd8f1b964dcf3b91481282f69d"
    assert hashlib.sha256(S5.tobytes()).hexdigest()[:32] == "a92dd8c263255d4ffc91f5dad7cc45d7"


def test_job_bytes_cover_the_arrays():
    """What admission charges for a sample-packed job covers its spins,
    couplings and, with cluster moves, the overlap words (and the global
    labelling scratch of lattices above 32768 sites)."""
    betas, _ = lut("T07_16_N24")
    for L, Lz, nw, NR in [(12, 48, 4, 4), (7, 9, 1, 2), (20, 96, 2, 2)]:
        g = eagb.SpGeom(L, Lz, 24, NR, nw, eagb.EA_OBC)
        V = L * L * Lz
        plain = eagb.sp_job_bytes(g, eagb.Cadence(2, 10, 1, 1, 0, 0), betas)
        clus = eagb.sp_job_bytes(g, eagb.Cadence(2, 10, 1, 1, 1, 0), betas)
        base = nw * V * NR * 24 * 8 + nw * V * 48
        assert plain >= base
        assert clus >= base + nw * 12 * V * 8 + (nw * 12 * 8 * 7 * V if V > 32768 else 0)
    # a job small enough for the resident kernel is charged its random words
    # (16 MB per launch here) when its bins have no cluster moves
    g = eagb.SpGeom(6, 24, 12, 2, 1, eagb.EA_PBC)
    plain = eagb.sp_job_bytes(g, eagb.Cadence(512, 1, 1, 1, 0, 0), betas[:12])
    clus = eagb.sp_job_bytes(g, eagb.Cadence(512, 1, 1, 1, 1, 0), betas[:12])
    assert plain - clus >= 33 * 24 * 864 * 24 - 864 * 6 * 8
    with pytest.raises(eagb.EAError):
        eagb.sp_job_bytes(eagb.SpGeom(1, 4, 24, 2, 1, eagb.EA_PBC))


def brute_dos(nb, J, lane):
    """Plain enumeration from the definition: E = 3V - (unsatisfied half-edges)."""
    V = nb.shape[0]
    c = np.arange(1 << (V - 1), dtype=np.int64) << 1
    spins = (c[:, None] >> np.arange(V)) & 1
    jb = ((J[0] >> np.uint64(lane)) & np.uint64(1)).astype(np.int64)
    U2 = np.zeros(len(c), np.int64)
    for d in range(6):
        U2 += (spins ^ spins[:, nb[:, d]] ^ jb[:, d][None, :]).sum(1)
    return np.bincount(6 * V - U2, minlength=6 * V + 1).astype(np.uint64)


@pytest.mark.parametrize("L,Lz,bc", [(2, 2, eagb.EA_PBC), (2, 3, eagb.EA_OBC), (2, 4, eagb.EA_PBC)])
def test_oracle_dos_small(L, Lz, bc):
    nb, mate, col, ncol = eagb.sp_graph(L, Lz, bc)
    g = eagb.SpGeom(L, Lz, 2, 1, 1, bc)
    J, _ = eagb.sp_host_init(g, 5, 6)
    V = L * L * Lz
    for lane in (0, 17, 63):
        h = O.sp_dos(V, nb, J, 0, lane)
        assert np.array_equal(h, brute_dos(nb, J, lane))
        assert h.sum() == 1 << (V - 1)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def oracle_gens(gen, NR):
    prc = (O.HQ * NR).from_buffer_copy(bytes(memoryview(gen.prc).cast("B"))[:C.sizeof(O.HQ) * NR])
    xo = (O.XO * NR).from_buffer_copy(bytes(memoryview(gen.xo).cast("B"))[:C.sizeof(O.XO) * NR])
    keys = np.array(list(gen.keys)[:NR], np.uint32)
    return prc, xo, keys


class OracleSP:
    """The oracle's copy of a job: passes, energies, tempering."""

    def __init__(self, job, jobid):
        g = job.g
        self.L, self.Lz, self.NR, self.NB, self.nw = g.L, g.Lz, g.nrep, g.nbetas, g.nwords
        self.V = job.V
        self.nb, _, self.col, self.ncol = eagb.sp_graph(g.L, g.Lz, g.bc)
        self.J, S0 = eagb.sp_host_init(g, SEEDS[0], SEEDS[1])
        self.S = job.get_spins()
        assert np.array_equal(self.S, S0)
        self.prc, self.xo, self.keys = oracle_gens(job.get_generators(), self.NR)
        self.betas, self.cum = job.betas, job.cum
        self.sites = [np.nonzero(self.col == c)[0].astype(np.int32) for c in range(self.ncol)]
        self.it, self.step, self.jobid = 0, 0, jobid
        gen = job.get_generators()
        self.rc = O.HQ.from_buffer_copy(bytes(memoryview(gen.rc).cast("B")))
        self.move = 0
        self.perm = np.tile(np.arange(self.NB, dtype=np.uint8), (self.nw, 64, self.NR, 1))
        self.acc = np.zeros((self.nw, 64, self.NR, self.NB - 1), np.uint32)

    def sweeps(self, n):
        for _ in range(n):
            for c in range(self.ncol):
                ctr = O.fill_bits(self.prc, self.xo, self.NR, self.it, self.jobid)
                O.sp_pass(self.V, self.NR, self.NB, self.nw, self.nb, self.sites[c], ctr, self.keys, self.cum,
                          self.J, self.S)
                self.it += 1

    def energy(self):
        return O.sp_energy(self.V, self.NR, self.NB, self.nw, self.nb, self.J, self.S)

    def pt(self):
        U2 = self.energy()
        E, M = O.sp_pt(self.V, self.NR, self.NB, self.nw, self.betas, self.step, SEEDS[3], U2, self.perm,
                       self.acc, self.S)
        self.step += 1
        return E, M

    def houdayer(self, nclust=0):
        """Replica pairs drawn from random_c as main.cu:408-421 draws them, then
        the cluster flips of each group."""
        if nclust <= 0:
            nclust = int(np.floor(0.5 * self.NB + 0.5))
        self.move += 1
        ng = 2 if self.NR >= 4 else 1
        h = self.NR // ng
        for g in range(ng):
            idx = list(range(g * h, g * h + h))
            for k in range(h - 1):
                f = O.lib().or_hq_next(C.byref(self.rc))
                q = k + ((f >> 32) % (h - k))
                idx[k], idx[q] = idx[q], idx[k]
            O.sp_cluster(self.V, self.NR, self.NB, self.nw, self.nb, nclust, g, idx[0], idx[1], self.move,
                         SEEDS[3] ^ 0xC2B2AE3585EBCA6B, self.S)


def new_job(L, Lz, bc, lutname, NR, nw, jobid=3):
    # "name:k" takes the first k temperatures of a set (odd NB runs the
    # pass's one-slot-per-lane path, even NB the two-slot one)
    name, _, k = lutname.partition(":")
    betas, cum = lut(name)
    if k:
        betas, cum = betas[:int(k)], cum[:int(k)]
    job = eagb.SpJob(L, Lz, betas, cum, nrep=NR, nwords=nw, bc=bc, seeds=SEEDS, jobid=jobid)
    job.cum = np.ascontiguousarray(cum, np.uint64)
    return job


CASES = [(6, 8, eagb.EA_PBC, "T08_16_N4", 2, 2), (5, 7, eagb.EA_OBC, "T07_16_N6", 3, 1),
         (6, 6, eagb.EA_OBC, "T07_16_N6:5", 3, 2), (7, 4, eagb.EA_PBC, "T07_16_N8:7", 2, 1),
         (3, 3, eagb.EA_PBC, "T07_16_N8", 2, 1), (12, 16, eagb.EA_OBC, "T07_16_N12", 4, 1),
         (8, 16, eagb.EA_OBC, "T07_16_N24", 2, 3)]


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [None, 0, 4])
@pytest.mark.parametrize("L,Lz,bc,ln,NR,nw", CASES)
def test_sweeps_energy_tempering_match_oracle(L, Lz, bc, ln, NR, nw, tile):
    """tile None: the job's default form (the per-item pass for one word,
    tiles for more); 0: the per-item pass (one thread per site, replica and
    slot); 4: tiles of 4 sites staging their random words in SMEM."""
    job = new_job(L, Lz, bc, ln, NR, nw)
    if tile is not None:
        job.set_tile(tile)
        assert job.info()[1] == tile
    orc = OracleSP(job, 3)
    job.sweeps(2)
    orc.sweeps(2)
    assert np.array_equal(job.get_spins(), orc.S)
    assert np.array_equal(job.energy(), orc.energy())
    for _ in range(2):
        job.parallel_tempering()
        E, M = orc.pt()
        gE, gperm, gacc, gM = job.tempering()
        assert np.array_equal(gE, E)
        assert np.array_equal(gM, M)
        assert np.array_equal(gperm, orc.perm)
        assert np.array_equal(gacc, orc.acc)
        assert np.array_equal(job.get_spins(), orc.S)
        job.sweeps(1)
        orc.sweeps(1)
    assert job.counter() == (orc.it, orc.step)
    # the swaps did move configurations: some lane changed slot
    assert orc.acc.sum() > 0
    job.close()


@pytest.mark.gpu
# lattices of the four labelling paths: up to 8900 sites all 8 samples per
# pass (odd and even L, PBC and OBC), up to 10500 4 samples per pass, up to
# 32768 one sample at a time in SMEM, above in slabs of z planes joined by a
# union across the slab faces (odd L OBC: corner fake bonds between the two
# open planes; even L PBC: the z wrap)
@pytest.mark.parametrize("L,Lz,bc,NR,nw", [(5, 6, eagb.EA_OBC, 4, 2), (3, 3, eagb.EA_PBC, 2, 1), (4, 8, eagb.EA_OBC, 8, 1),
                                           (2, 5, eagb.EA_OBC, 2, 1), (10, 96, eagb.EA_OBC, 2, 1),
                                           (11, 90, eagb.EA_PBC, 2, 1), (19, 96, eagb.EA_OBC, 2, 1),
                                           (16, 130, eagb.EA_PBC, 4, 1)])
def test_houdayer_matches_oracle(L, Lz, bc, NR, nw):
    job = new_job(L, Lz, bc, "T07_16_N6", NR, nw)
    orc = OracleSP(job, 3)
    for _ in range(3):
        job.sweeps(1)
        orc.sweeps(1)
        job.parallel_tempering()
        orc.pt()
        before = job.energy()
        job.houdayer(3)
        orc.houdayer(3)
        assert np.array_equal(job.get_spins(), orc.S)
        after = job.energy()
        # each move conserves E(r1) + E(r2) of every sample and slot: the sum
        # over replicas is unchanged
        assert np.array_equal(before.sum(2), after.sum(2))
    # clusters did flip
    assert not np.array_equal(before, after)
    job.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", [False, True])
def test_run_bin_matches_oracle(cluster):
    job = new_job(5, 6, eagb.EA_PBC, "T07_16_N6", 4, 2)
    orc = OracleSP(job, 3)
    itmax, houfr, mesfr, ptfr = 3, 2, 2, 2
    avg = job.run_bin(itmax, houfr, mesfr, ptfr, cluster=cluster, nclust=0)
    tot = np.zeros((2, 64, 4, 6))
    for it in range(itmax):
        for im in range(mesfr):
            for ih in range(houfr):
                orc.sweeps(ptfr)
                orc.pt()
            if cluster:
                orc.houdayer(0)
        tot += 3 * orc.V - orc.energy()
    assert np.array_equal(job.get_spins(), orc.S)
    assert np.array_equal(avg, tot / itmax)
    job.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [eagb.EA_PBC, eagb.EA_OBC])
def test_exact_dos_matches_oracle(bc):
    job = new_job(3, 3, bc, "T07_16_N8", 2, 1)
    dos, mean = job.exact()
    V = 27
    assert np.all(dos.sum(1) == 1 << (V - 1))
    nb, _, _, _ = eagb.sp_graph(3, 3, bc)
    J, _ = eagb.sp_host_init(job.g, SEEDS[0], SEEDS[1])
    for lane in (0, 41):
        assert np.array_equal(dos[lane], O.sp_dos(V, nb, J, 0, lane))
    # <E>(beta) from the histogram, recomputed on the host
    E = np.arange(-3 * V, 3 * V + 1)
    for lane in (0, 41):
        g = dos[lane].astype(np.float64)
        for k, b in enumerate(job.betas):
            w = g * np.exp(b * (E - E[g > 0].max()))
            assert abs((w * E).sum() / w.sum() - mean[lane, k]) < 1e-9 * V
    job.close()


@pytest.mark.gpu
@pytest.mark.parametrize("bc,cluster", [(eagb.EA_PBC, False), (eagb.EA_OBC, False), (eagb.EA_PBC, True),
                                        (eagb.EA_OBC, True)])
def test_monte_carlo_matches_exact_enumeration(bc, cluster):
    """3x3x3, 64 samples, 8 temperatures in [0.7, 1.6], tempering every sweep
    (2 replicas), or with a Houdayer move every 5 sweeps (4 replicas): the
    time average of E per sample and temperature agrees with exact
    enumeration within the statistical error of the blocks."""
    job = new_job(3, 3, bc, "T07_16_N8", 4 if cluster else 2, 1)
    NR = job.g.nrep
    _, exact = job.exact()
    cad = dict(houfr=5, mesfr=1, ptfr=1, cluster=cluster)
    job.run_bin(800, **cad)   # equilibration
    nblk = 20
    blocks = np.stack([job.run_bin(300, **cad) for _ in range(nblk)])     # [blk, 1, 64, NR, NB]
    est = blocks[:, 0].transpose(0, 2, 1, 3).reshape(nblk * NR, 64, -1)  # blocks x replicas
    mean = est.mean(0)
    err = est.std(0, ddof=1) / np.sqrt(est.shape[0])
    z = (mean - exact) / np.maximum(err, 1e-12)
    assert np.abs(z).max() < 6.0, np.abs(z).max()
    assert 0.5 < (z ** 2).mean() < 2.0, (z ** 2).mean()
    job.close()


BATCH = [(3, 3, eagb.EA_PBC, "T07_16_N8", 2, 1), (5, 7, eagb.EA_OBC, "T07_16_N6", 4, 2),
         (8, 16, eagb.EA_OBC, "T07_16_N24", 2, 1), (6, 12, eagb.EA_PBC, "T08_16_N4", 4, 3),
         (19, 96, eagb.EA_OBC, "T08_16_N4", 2, 1)]


@pytest.mark.gpu
def test_batch_equals_jobs_alone():
    """A batch of sample-packed jobs of different L (odd and even, 2 and 3
    colours), Lz, boundary, replica, temperature and word counts, one
    lattice above the SMEM labelling limit: every job ends as if run alone."""
    alone = [new_job(*c, jobid=40 + k) for k, c in enumerate(BATCH)]
    batched = [new_job(*c, jobid=40 + k) for k, c in enumerate(BATCH)]
    batch = eagb.SpBatch(batched)
    for itmax, houfr, mesfr, ptfr, cl in [(2, 2, 1, 1, True), (3, 1, 2, 2, False), (1, 3, 1, 1, True)]:
        batch.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        for a, b in zip(alone, batched):
            avg = a.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
            assert np.array_equal(avg, b.bin_results())
    batch.sync()
    for a, b in zip(alone, batched):
        assert np.array_equal(a.get_spins(), b.get_spins())
        assert all(np.array_equal(x, y) for x, y in zip(a.tempering(), b.tempering()))
        assert a.counter() == b.counter()
    batch.close()
    for j in alone + batched:
        j.close()


@pytest.mark.gpu
def test_large_batch_classes_equal_jobs_alone():
    """Above 256 jobs a batch groups jobs into classes of equal NB and lattice
    size (one launch per kernel kind for a whole class): 260 small jobs of
    five geometries still end as if run alone."""
    geoms = [(2, 2, eagb.EA_PBC, "T08_16_N4", 2, 1), (3, 3, eagb.EA_OBC, "T07_16_N6", 4, 1),
             (2, 4, eagb.EA_OBC, "T07_16_N6", 2, 1), (4, 2, eagb.EA_PBC, "T08_16_N4", 4, 1),
             (3, 5, eagb.EA_PBC, "T07_16_N8", 2, 1)]
    cases = [geoms[k % len(geoms)] for k in range(260)]
    alone = [new_job(*c, jobid=k) for k, c in enumerate(cases)]
    batched = [new_job(*c, jobid=k) for k, c in enumerate(cases)]
    batch = eagb.SpBatch(batched)
    batch.run_bin(2, 2, 1, 1, cluster=True)
    for a in alone:
        a.run_bin(2, 2, 1, 1, cluster=True)
    batch.sync()
    for a, b in zip(alone, batched):
        assert np.array_equal(a.get_spins(), b.get_spins())
        assert np.array_equal(a.bin_results(), b.bin_results())
    batch.close()
    for j in alone + batched:
        j.close()


def oracle_bin(orc, itmax, houfr, mesfr, ptfr, cluster, nclust=0):
    """One bin of the cadence on the oracle: sweeps, tempering every ptfr
    sweeps, a move every houfr tempering steps, the energy measured after
    each of the itmax iterations; returns the averages."""
    tot = np.zeros((orc.nw, 64, orc.NR, orc.NB))
    for it in range(itmax):
        for im in range(mesfr):
            for ih in range(houfr):
                orc.sweeps(ptfr)
                orc.pt()
            if cluster:
                orc.houdayer(nclust)
        tot += 3 * orc.V - orc.energy()
    return tot / itmax


# the sample-packed configurations the bench times, at the size it times them:
# L=6, Lz=24, PBC, NT=12 in [0.8, 1.6], NR=2, one word (64 samples), a bin
# of 512 sweeps with tempering after each (no cluster moves); and L=12,
# Lz=48, OBC, NT=24 in [0.7, 1.6], NR=4, 64 words (4096 samples), a bin of 10
# sweeps with tempering after each and a Houdayer move on the colder half --
# the 16-byte two-slot pass, the tile width, the energy chunking and the
# 4-samples-per-pass labelling of 6912-site lattices as the bench runs them;
# and the large tube as written (L=24, Lz=192, OBC, NT=32 in [0.6, 1.6],
# NR=4, one word, a move every 5 sweeps): slab labelling.  One-word jobs
# take the per-item pass by default; they also run with the tiles their
# heuristic chooses (8 and 32 sites).
TIMED = [(6, 24, eagb.EA_PBC, "T08_16_N12", 2, 1, (512, 1, 1, 1, False), None),
         (12, 48, eagb.EA_OBC, "T07_16_N24", 4, 1, (10, 10, 1, 1, True), None),
         (12, 48, eagb.EA_OBC, "T07_16_N24", 4, 1, (10, 10, 1, 1, True), 8),
         (12, 48, eagb.EA_OBC, "T07_16_N24", 4, 64, (1, 10, 1, 1, True), None),
         (24, 192, eagb.EA_OBC, "T06_16_N32", 4, 1, (1, 5, 1, 1, True), None),
         (24, 192, eagb.EA_OBC, "T06_16_N32", 4, 1, (1, 5, 1, 1, True), 32)]


@pytest.mark.gpu
@pytest.mark.parametrize("L,Lz,bc,ln,NR,nw,cad,tile", TIMED)
def test_timed_configurations_match_oracle(L, Lz, bc, ln, NR, nw, cad, tile):
    itmax, houfr, mesfr, ptfr, cl = cad
    job = new_job(L, Lz, bc, ln, NR, nw, jobid=0)
    if tile is not None:
        job.set_tile(tile)
    orc = OracleSP(job, 0)
    avg = job.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl, nclust=0)
    want = oracle_bin(orc, itmax, houfr, mesfr, ptfr, cl)
    assert np.array_equal(job.get_spins(), orc.S)
    assert np.array_equal(avg, want)
    gE, gperm, gacc, gM = job.tempering()
    assert np.array_equal(gperm, orc.perm) and np.array_equal(gacc, orc.acc)
    assert job.counter() == (orc.it, orc.step)
    assert orc.acc.sum() > 0
    job.close()


# jobs of 2 and 3 colours, 1..3 words, 2..5 replicas, with and without moves
BINS = [(6, 8, eagb.EA_PBC, "T08_16_N4", 2, 2, (3, 2, 1, 2, False)),
        (5, 7, eagb.EA_OBC, "T07_16_N6", 4, 1, (2, 2, 2, 1, True)),
        (7, 4, eagb.EA_PBC, "T07_16_N8:7", 5, 3, (2, 3, 1, 1, True)),
        (12, 16, eagb.EA_OBC, "T07_16_N12", 4, 2, (2, 5, 1, 1, True))]


@pytest.mark.gpu
@pytest.mark.parametrize("L,Lz,bc,ln,NR,nw,cad", BINS)
def test_persistent_bin_kernel_equals_graph(L, Lz, bc, ln, NR, nw, cad):
    """The persistent bin kernel (one cooperative launch per bin) and the
    graph of per-phase launches give the same words, averages, tempering
    state and counters, bin after bin; and both equal the oracle."""
    itmax, houfr, mesfr, ptfr, cl = cad
    a, b = new_job(L, Lz, bc, ln, NR, nw, jobid=11), new_job(L, Lz, bc, ln, NR, nw, jobid=11)
    a.set_bin_kernel(eagb.EA_BIN_GRAPH)
    b.set_bin_kernel(eagb.EA_BIN_PERSISTENT)
    orc = OracleSP(a, 11)
    for _ in range(2):
        va = a.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        vb = b.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        want = oracle_bin(orc, itmax, houfr, mesfr, ptfr, cl)
        assert np.array_equal(va, want) and np.array_equal(vb, want)
    assert np.array_equal(a.get_spins(), b.get_spins())
    assert np.array_equal(b.get_spins(), orc.S)
    assert all(np.array_equal(x, y) for x, y in zip(a.tempering(), b.tempering()))
    assert a.counter() == b.counter() == (orc.it, orc.step)
    a.close()
    b.close()


# bins without cluster moves: 2 and 3 colours (L=3 and L=7 PBC), 1..3 words,
# 2..5 replicas, one CTA per z plane up to 16 CTAs of several planes; the
# first is the L=6, Lz=24 job of the timed configurations with 40 sweeps,
# two launches of 33 and 7 sweeps (16 MB of random words per launch)
RESIDENT = [(6, 24, eagb.EA_PBC, "T08_16_N12", 2, 1, (40, 1, 1, 1, False)),
            (6, 8, eagb.EA_PBC, "T08_16_N4", 2, 2, (3, 2, 1, 2, False)),
            (5, 7, eagb.EA_OBC, "T07_16_N6", 4, 1, (2, 2, 2, 1, False)),
            (7, 4, eagb.EA_PBC, "T07_16_N8:7", 5, 3, (2, 3, 1, 1, False)),
            (3, 3, eagb.EA_PBC, "T07_16_N8", 2, 1, (3, 1, 1, 3, False)),
            (12, 16, eagb.EA_OBC, "T07_16_N12", 4, 2, (2, 5, 1, 1, False)),
            (4, 40, eagb.EA_OBC, "T07_16_N6:5", 1, 1, (4, 1, 2, 1, False)),
            # cluster moves between resident launches of houfr x ptfr >= 4 sweeps
            (6, 8, eagb.EA_PBC, "T08_16_N4", 4, 1, (3, 5, 1, 1, True)),
            (5, 7, eagb.EA_OBC, "T07_16_N6", 4, 1, (2, 4, 2, 1, True)),
            (7, 4, eagb.EA_PBC, "T07_16_N8:7", 5, 3, (2, 2, 1, 2, True)),
            (12, 16, eagb.EA_OBC, "T07_16_N12", 4, 2, (2, 10, 1, 1, True)),
            (6, 12, eagb.EA_OBC, "T07_16_N6", 2, 1, (3, 4, 1, 1, True))]


@pytest.mark.gpu
@pytest.mark.parametrize("L,Lz,bc,ln,NR,nw,cad", RESIDENT)
def test_resident_bin_kernel_equals_graph(L, Lz, bc, ln, NR, nw, cad):
    """The resident bin kernel (counters, random words, then one cluster
    holding the words in distributed shared memory; with cluster moves, one
    launch per block of sweeps and the moves between them) and the graph of
    per-phase launches give the same words, averages, tempering state,
    counters and generator states, bin after bin; and both equal the
    oracle."""
    itmax, houfr, mesfr, ptfr, cl = cad
    a, b = new_job(L, Lz, bc, ln, NR, nw, jobid=13), new_job(L, Lz, bc, ln, NR, nw, jobid=13)
    a.set_bin_kernel(eagb.EA_BIN_GRAPH)
    b.set_bin_kernel(eagb.EA_BIN_RESIDENT)
    orc = OracleSP(a, 13)
    assert b.bin_kernel_for(itmax, houfr, mesfr, ptfr, cluster=cl) == eagb.EA_BIN_RESIDENT
    for _ in range(2):
        va = a.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        vb = b.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        want = oracle_bin(orc, itmax, houfr, mesfr, ptfr, cl)
        assert np.array_equal(va, want) and np.array_equal(vb, want)
    assert np.array_equal(a.get_spins(), b.get_spins())
    assert np.array_equal(b.get_spins(), orc.S)
    assert all(np.array_equal(x, y) for x, y in zip(a.tempering(), b.tempering()))
    assert a.counter() == b.counter() == (orc.it, orc.step)
    ga, gb = a.get_generators(), b.get_generators()
    assert bytes(ga) == bytes(gb)
    assert np.array_equal(a.energy(), b.energy())
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("L,Lz,bc,ln,NR,nw", [(12, 48, eagb.EA_OBC, "T07_16_N24", 4, 2),
                                              (7, 4, eagb.EA_PBC, "T07_16_N8:7", 5, 3)])
def test_autotuned_job_equals_untuned(L, Lz, bc, ln, NR, nw):
    """The autotuner leaves the job's state as it was, and the job with the
    tuned tile width, energy chunking and labelling block size gives the same
    words, averages, tempering state and counters as the untuned one, with and
    without cluster moves (graph path) -- and both equal the oracle."""
    a, b = new_job(L, Lz, bc, ln, NR, nw, jobid=15), new_job(L, Lz, bc, ln, NR, nw, jobid=15)
    a.set_bin_kernel(eagb.EA_BIN_GRAPH)
    b.set_bin_kernel(eagb.EA_BIN_GRAPH)
    S0, c0 = b.get_spins(), b.counter()
    kt, ec, ct = b.autotune()
    assert kt >= 0 and ec >= 1 and ct in (256, 512, 1024)
    assert np.array_equal(b.get_spins(), S0) and b.counter() == c0
    orc = OracleSP(a, 15)
    for cl in (True, False):
        va = a.run_bin(2, 2, 1, 1, cluster=cl)
        vb = b.run_bin(2, 2, 1, 1, cluster=cl)
        assert np.array_equal(va, vb)
        assert np.array_equal(va, oracle_bin(orc, 2, 2, 1, 1, cl))
    assert np.array_equal(a.get_spins(), b.get_spins())
    assert all(np.array_equal(x, y) for x, y in zip(a.tempering(), b.tempering()))
    assert a.counter() == b.counter()
    a.close()
    b.close()


@pytest.mark.gpu
def test_resident_then_graph_and_moves_continue_alike():
    """A resident bin followed by a bin with cluster moves (the graph) and
    another resident bin ends where the graph alone ends; the explicit
    resident mode refuses a bin with moves."""
    a = new_job(12, 16, eagb.EA_OBC, "T07_16_N12", 4, 1, jobid=14)
    b = new_job(12, 16, eagb.EA_OBC, "T07_16_N12", 4, 1, jobid=14)
    a.set_bin_kernel(eagb.EA_BIN_GRAPH)
    for cl in (False, True, False):
        va = a.run_bin(3, 2, 1, 1, cluster=cl)
        vb = b.run_bin(3, 2, 1, 1, cluster=cl)
        assert np.array_equal(va, vb)
    assert np.array_equal(a.get_spins(), b.get_spins())
    assert a.counter() == b.counter()
    b.set_bin_kernel(eagb.EA_BIN_RESIDENT)
    with pytest.raises(RuntimeError):
        b.run_bin(1, 1, 1, 1, cluster=True)
    a.close()
    b.close()


@pytest.mark.gpu
def test_persistent_batch_equals_graph_batch():
    """A batch of mixed jobs run by the persistent bin kernel (one work list
    of every job) ends as the same batch run by per-class graph branches."""
    geoms = BATCH + [(12, 16, eagb.EA_OBC, "T07_16_N12", 4, 2), (3, 5, eagb.EA_PBC, "T07_16_N8", 2, 1)]
    ga = [new_job(*c, jobid=60 + k) for k, c in enumerate(geoms)]
    gb = [new_job(*c, jobid=60 + k) for k, c in enumerate(geoms)]
    A, B = eagb.SpBatch(ga), eagb.SpBatch(gb)
    A.set_bin_kernel(eagb.EA_BIN_GRAPH)
    B.set_bin_kernel(eagb.EA_BIN_PERSISTENT)
    for itmax, houfr, mesfr, ptfr, cl in [(2, 2, 1, 1, True), (3, 1, 2, 2, False)]:
        A.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        B.run_bin(itmax, houfr, mesfr, ptfr, cluster=cl)
        A.sync()
        B.sync()
        for x, y in zip(ga, gb):
            assert np.array_equal(x.bin_results(), y.bin_results())
    for x, y in zip(ga, gb):
        assert np.array_equal(x.get_spins(), y.get_spins())
        assert x.counter() == y.counter()
    A.close()
    B.close()
    for j in ga + gb:
        j.close()
