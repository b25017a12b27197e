"""GPU parity: the CUDA path (through the C ABI of libeagb.so) against the CPU
oracle on the same seeded inputs.  Integer and byte results must be bit-exact;
the FP64 tempering statistics must be identical too (same operations, same
order, exp() values from the host's libm)."""
import os

import numpy as np
import pytest

import oracle_py as O
from conftest import ROOT

import importlib.util

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(ROOT, "tests", "golden")

# name: L, Lz, lut, bc, nsamples
CASES = {
    "L8_Lz8_PBC": (8, 8, "T08_16_N4", O.PBC, 2),
    "L8_Lz16_OBC": (8, 16, "T07_16_N6", O.OBC, 3),
    "L8_Lz16_WEAK": (8, 16, "T07_16_N6", O.OBC_WEAK, 2),
    "L16_Lz24_STRONG": (16, 24, "T07_16_N8", O.OBC_STRONG, 2),
    "L16_Lz48_OBC_NB40": (16, 48, "shipped_N40", O.OBC, 1),
}
MASTERS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)


def lut(name):
    d = np.load(os.path.join(GOLD, "lut_%s.npz" % name))
    return d["betas"], d["cum"]


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def make(case, jobid=3, iter0=0):
    L, Lz, ln, bc, ns = CASES[case]
    betas, cum = lut(ln)
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, bc=bc, masters=MASTERS, iter0=iter0, jobid=jobid)
    sim = O.Sim(L, Lz, betas, cum, nbits=ns, bc=bc, masters=MASTERS, itmax=4)
    return job, sim


def assert_same_state(job, sim):
    for s in range(sim.g.nbits):
        ev, od = job.get_spins(s)
        assert np.array_equal(ev, sim.spins[s, 0]), "even spins, sample %d" % s
        assert np.array_equal(od, sim.spins[s, 1]), "odd spins, sample %d" % s
    wctb, wbtc = job.get_permutations()
    assert np.array_equal(wctb, sim.wctb)
    assert np.array_equal(wbtc, sim.wbtc)
    gen, pt = job.get_generators()
    NR = sim.g.NR
    assert O.as_bytes(gen.prc)[:NR * 2080] == O.as_bytes(sim.prc)
    assert O.as_bytes(gen.xo)[:NR * 48] == O.as_bytes(sim.xo)
    assert O.as_bytes(pt) == O.as_bytes(sim.pt)
    assert O.as_bytes(gen.rc) == O.as_bytes(sim.rc)


def test_curand_device_matches_host():
    for seed, off, n in ((0x5555666677778888, 0, 4096), (12345, 1000003, 5000), (7, 2 ** 33 + 11, 777)):
        d = eagb.curand_uniforms(seed, off, n)
        h = O.curand_host(seed, off, n)
        assert np.array_equal(d, h)
    # a fresh generator at offset n does not continue one that produced n numbers:
    # the reference keeps one generator per process and only uses the offset on restart
    a = O.curand_host(99, 0, 8000)
    b = eagb.curand_uniforms(99, 4000, 4000)
    assert not np.array_equal(a[4000:], b)


@pytest.mark.parametrize("case", list(CASES))
def test_half_sweeps_and_energy(case):
    job, sim = make(case, jobid=7, iter0=10)
    it = 10
    for sweep in range(3):
        for p in (0, 1):
            ctr = O.fill_bits(sim.prc, sim.xo, sim.g.NR, it, 7)
            sim.half_sweep(ctr, p)
            it += 1
    job.monte_carlo(3)
    assert job.get_counter() == it
    for s in range(sim.g.nbits):
        ev, od = job.get_spins(s)
        assert np.array_equal(ev, sim.spins[s, 0]) and np.array_equal(od, sim.spins[s, 1])
    assert np.array_equal(job.measure_energy(), sim.energy())
    job.close()


@pytest.mark.parametrize("case", list(CASES))
def test_tempering_after_sweeps(case):
    job, sim = make(case)
    it = 0
    for rnd in range(4):
        for p in (0, 1):
            ctr = O.fill_bits(sim.prc, sim.xo, sim.g.NR, it, 3)
            sim.half_sweep(ctr, p)
            it += 1
        E = sim.energy()
        for s in range(sim.g.nbits):
            for r in range(sim.g.NR):
                O.lib().or_parallel_tempering(O.C.byref(sim.pt[s * sim.g.NR + r]), O.ptr(sim.wctb[s, r]),
                                              O.ptr(sim.wbtc[s, r]), O.ptr(np.ascontiguousarray(E[s, r])),
                                              O.ptr(sim.betas), sim.g.NB, O.ptr(sim.acc[s, r]),
                                              O.ptr(sim.att[s, r]), O.ptr(sim.accraw[s, r]))
        job.monte_carlo(1)          # energies fused into the odd half-sweep
        job.parallel_tempering()
    assert_same_state(job, sim)
    acc, att, raw = job.get_pt_stats()
    assert np.array_equal(att, sim.att) and np.array_equal(raw, sim.accraw)
    assert np.array_equal(acc, sim.acc)
    job.close()


@pytest.mark.parametrize("case", list(CASES))
def test_full_bins(case):
    job, sim = make(case, jobid=21, iter0=0)
    it = 0
    for b in range(2):
        avg, hist = job.run_bin(itmax=4, houfr=2, mesfr=2, ptfr=1 + b, cluster=sim.g.NR >= 4)
        it = sim.run_bin(itmax=4, houfr=2, mesfr=2, ptfr=1 + b, iter0=it, jobid=21)
        assert np.array_equal(avg, sim.avgE)
        assert np.array_equal(hist, sim.hist)
    assert_same_state(job, sim)
    assert job.get_counter() == it
    acc, att, raw = job.get_pt_stats()
    assert np.array_equal(raw, sim.accraw) and np.array_equal(acc, sim.acc)
    gen, _ = job.get_generators()
    assert gen.cuda_rng_offset == sim.cuda_rng_offset
    job.close()


def _move_pairs(job):
    """The two replica pairs the next Houdayer move draws from random_c
    (main.cu:408-421), replayed on a copy of the job's generator."""
    gen, _ = job.get_generators()
    rc = O.HQ.from_buffer_copy(bytes(memoryview(gen.rc).cast("B")))
    out = []
    for g in range(2):
        r1, r2 = O.C.c_int(), O.C.c_int()
        O.lib().or_houdayer_pair(O.C.byref(rc), job.g.nrep, g, O.C.byref(r1), O.C.byref(r2))
        out.append((r1.value, r2.value))
    return out


@pytest.mark.parametrize("L,Lz,lutname,ns,rule", [(16, 24, "T07_16_N8", 4, "reference"),
                                                  (24, 16, "T07_16_N8", 8, "exact")])
def test_houdayer_conserves_pair_energy(L, Lz, lutname, ns, rule):
    """One Houdayer move flips each cluster of equal overlap in both replicas
    of a pair, so E(r1) + E(r2) of every (sample, temperature < nclust,
    group) is unchanged, every other energy is untouched, and some energies
    do change.  Under the reference's bond rule this holds when L is a power
    of two; at L = 24 the reference tests site 0's x-wrap bond against
    x = 15 (HoudayerXEA.cu:96), which can split a cluster (rarely: only when
    no other path joins its two pieces) -- with EA_CLUSTER_EXACT it holds for
    every L.  (The reference rule at L = 24 is pinned against the oracle by
    the whole-bin tests.)"""
    betas, cum = lut(lutname)
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, bc=O.OBC, masters=MASTERS, iter0=0, jobid=3)
    if rule == "exact":
        eagb._ck(eagb.lib().ea_set_cluster_rule(job.ctx, 1))
    job.monte_carlo(3)
    job.parallel_tempering()
    E0 = job.measure_energy()
    wctb, _ = job.get_permutations()
    pairs = _move_pairs(job)
    job.houdayer()
    E1 = job.measure_energy()
    NB, NR = job.g.nbetas, job.g.nrep
    nclust = int(np.floor(0.5 * NB + 0.5))
    moved = np.zeros(E0.shape, bool)
    bad = 0
    for r1, r2 in pairs:
        for s in range(ns):
            for b in range(nclust):
                c1, c2 = wctb[s, r1, b], wctb[s, r2, b]
                before = int(E0[s, r1, c1]) + int(E0[s, r2, c2])
                after = int(E1[s, r1, c1]) + int(E1[s, r2, c2])
                bad += before != after
                moved[s, r1, c1] = moved[s, r2, c2] = True
    assert np.array_equal(E0[~moved], E1[~moved]), "an energy outside the moved pairs changed"
    assert not np.array_equal(E0, E1), "no cluster flipped"
    assert bad == 0, "%d pair sums changed" % bad
    job.close()


def test_cluster_exact_rule_bin_matches_oracle():
    """EA_CLUSTER_EXACT at L = 24 (where it differs from the reference rule):
    a whole bin with cluster moves equals the oracle run with the exact rule."""
    betas, cum = lut("T07_16_N8")
    job = eagb.new_job(24, 16, betas, cum, nsamples=3, bc=O.OBC, masters=MASTERS, iter0=0, jobid=6)
    eagb._ck(eagb.lib().ea_set_cluster_rule(job.ctx, 1))
    sim = O.Sim(24, 16, betas, cum, nbits=3, bc=O.OBC, masters=MASTERS, itmax=3)
    it = 0
    for _ in range(2):
        avg, hist = job.run_bin(itmax=3, houfr=2, mesfr=1, ptfr=1, cluster=True)
        it = sim.run_bin(itmax=3, houfr=2, mesfr=1, ptfr=1, iter0=it, jobid=6, cluster_exact=True)
        assert np.array_equal(avg, sim.avgE)
        assert np.array_equal(hist, sim.hist)
    assert_same_state(job, sim)
    job.close()


def test_headline_bin_31_samples():
    """The timed configuration itself: L=24, Lz=192, OBC, NB=32 (T in
    [0.6, 1.6]), NR=8, 31 samples -- every (sample, clone) stride of the
    sweep tile and the cluster kernels at full size, the generator on its SM
    partition -- one step of the timed cadence (5 x (sweep, energy, PT), one
    Houdayer move, the energy measurement) against the oracle."""
    betas, cum = lut("T06_16_N32")
    job = eagb.new_job(24, 192, betas, cum, nsamples=31, bc=O.OBC, masters=MASTERS, iter0=0, jobid=0)
    sim = O.Sim(24, 192, betas, cum, nbits=31, bc=O.OBC, masters=MASTERS, itmax=1)
    avg, hist = job.run_bin(itmax=1, houfr=5, mesfr=1, ptfr=1, cluster=True)
    assert job.rng_sms() == 32
    sim.run_bin(itmax=1, houfr=5, mesfr=1, ptfr=1, iter0=0, jobid=0)
    assert np.array_equal(avg, sim.avgE)
    assert np.array_equal(hist, sim.hist)
    assert_same_state(job, sim)
    acc, att, raw = job.get_pt_stats()
    assert np.array_equal(raw, sim.accraw) and np.array_equal(acc, sim.acc)
    job.close()


def test_large_tube_bin():
    """L=24, Lz=192, NB=32 (T in [0.6,1.6]), OBC, two samples: one short bin."""
    betas, cum = lut("T06_16_N32")
    job = eagb.new_job(24, 192, betas, cum, nsamples=2, bc=O.OBC, masters=MASTERS, iter0=0, jobid=1)
    sim = O.Sim(24, 192, betas, cum, nbits=2, bc=O.OBC, masters=MASTERS, itmax=1)
    avg, hist = job.run_bin(itmax=1, houfr=2, mesfr=1, ptfr=1, cluster=True)
    sim.run_bin(itmax=1, houfr=2, mesfr=1, ptfr=1, iter0=0, jobid=1)
    assert np.array_equal(avg, sim.avgE)
    assert_same_state(job, sim)
    job.close()


def test_uniforms_drawn_ahead_continue_across_calls():
    """The next move's uniforms are drawn ahead on the generator stream: asynchronous
    bins, a generator read-back and a re-upload of the same state in between must
    leave the sequence as the reference process's single generator draws it."""
    job, sim = make("L8_Lz16_OBC", jobid=9, iter0=0)
    it = 0
    job.run_cycles(itmax=2, houfr=1, mesfr=1, ptfr=1)
    it = sim.run_bin(itmax=2, houfr=1, mesfr=1, ptfr=1, iter0=it, jobid=9)
    gen, pt = job.get_generators()
    assert gen.cuda_rng_offset == sim.cuda_rng_offset
    job.set_generators(gen, pt)
    avg, hist = job.run_bin(itmax=3, houfr=1, mesfr=2, ptfr=1, cluster=True)
    it = sim.run_bin(itmax=3, houfr=1, mesfr=2, ptfr=1, iter0=it, jobid=9)
    assert np.array_equal(avg, sim.avgE)
    assert_same_state(job, sim)
    gen, _ = job.get_generators()
    assert gen.cuda_rng_offset == sim.cuda_rng_offset
    job.close()


@pytest.mark.parametrize("nsm", [0, 32, 48])
def test_sm_split_leaves_results_unchanged(nsm):
    """The generator's SM partition changes only where kernels run."""
    betas, cum = lut("T06_16_N32")
    job = eagb.new_job(24, 192, betas, cum, nsamples=2, bc=O.OBC, masters=MASTERS, iter0=0, jobid=4)
    job.set_rng_sms(nsm)
    sim = O.Sim(24, 192, betas, cum, nbits=2, bc=O.OBC, masters=MASTERS, itmax=2)
    avg, hist = job.run_bin(itmax=2, houfr=1, mesfr=1, ptfr=1, cluster=True)
    sim.run_bin(itmax=2, houfr=1, mesfr=1, ptfr=1, iter0=0, jobid=4)
    assert np.array_equal(avg, sim.avgE)
    assert_same_state(job, sim)
    with pytest.raises(eagb.EAError):
        job.set_rng_sms(16)      # only before the first cluster move
    job.close()
