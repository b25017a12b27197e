"""Batched persistent form: a batch of jobs of different L, Lz, boundary
condition, temperature count and sample count, advanced by one launch per step
for all of them, must leave every job exactly as the same job run alone
(words, energies, tempering statistics, histories, generator states)."""
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
MASTERS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)

# L, Lz, lut, bc, nsamples
MIX = [
    (8, 8, "T08_16_N4", O.PBC, 2),
    (8, 16, "T07_16_N6", O.OBC, 3),
    (8, 16, "T07_16_N6", O.OBC_WEAK, 2),
    (16, 24, "T07_16_N8", O.OBC_STRONG, 2),
    (16, 48, "shipped_N40", O.OBC, 1),
    (24, 24, "T06_16_N32", O.PBC, 1),
    (8, 32, "T07_16_N8", O.PBC, 4),
]


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def lut(name):
    d = np.load(os.path.join(GOLD, "lut_%s.npz" % name))
    return d["betas"], d["cum"]


def make_jobs():
    jobs = []
    for k, (L, Lz, ln, bc, ns) in enumerate(MIX):
        betas, cum = lut(ln)
        m = tuple(x ^ (k * 0x9E3779B97F4A7C15 & 0xFFFFFFFFFFFFFFFF) for x in MASTERS)
        jobs.append(eagb.new_job(L, Lz, betas, cum, nsamples=ns, bc=bc, masters=m, iter0=0, jobid=10 + k))
    return jobs


def assert_same(a, b):
    for s in range(a.g.nsamples):
        ea, oa = a.get_spins(s)
        eb, ob = b.get_spins(s)
        assert np.array_equal(ea, eb) and np.array_equal(oa, ob), "sample %d" % s
    assert all(np.array_equal(x, y) for x, y in zip(a.get_permutations(), b.get_permutations()))
    assert all(np.array_equal(x, y) for x, y in zip(a.get_pt_stats(), b.get_pt_stats()))
    ga, pa = a.get_generators()
    gb, pb = b.get_generators()
    assert O.as_bytes(ga) == O.as_bytes(gb)
    assert O.as_bytes(pa) == O.as_bytes(pb)
    assert a.get_counter() == b.get_counter()
    assert np.array_equal(a.measure_energy(), b.measure_energy())


CADENCES = [(3, 2, 2, 1), (2, 1, 1, 2), (2, 2, 1, 0)]


@pytest.mark.parametrize("tile", [0, 1])
def test_batch_equals_jobs_alone(tile):
    alone, batched = make_jobs(), make_jobs()
    batch = eagb.Batch(batched, tile=tile)
    if tile:
        assert batch.tile() == tile
    for itmax, houfr, mesfr, ptfr in CADENCES:
        batch.run_bin(itmax=itmax, houfr=houfr, mesfr=mesfr, ptfr=ptfr, cluster=True)
        for a, b in zip(alone, batched):
            avg, hist = a.run_bin(itmax=itmax, houfr=houfr, mesfr=mesfr, ptfr=ptfr, cluster=True)
            bavg, bhist = b.bin_results()
            assert np.array_equal(avg, bavg)
            assert np.array_equal(hist, bhist)
    batch.sync()
    for a, b in zip(alone, batched):
        assert_same(a, b)
    batch.close()
    for j in alone + batched:
        j.close()


def test_batch_matches_oracle():
    """One member of a mixed batch against the CPU oracle, two bins."""
    jobs = make_jobs()
    batch = eagb.Batch(jobs)
    L, Lz, ln, bc, ns = MIX[1]
    betas, cum = lut(ln)
    m = tuple(x ^ (1 * 0x9E3779B97F4A7C15 & 0xFFFFFFFFFFFFFFFF) for x in MASTERS)
    sim = O.Sim(L, Lz, betas, cum, nbits=ns, bc=bc, masters=m, itmax=3)
    it = 0
    for b in range(2):
        batch.run_bin(itmax=3, houfr=2, mesfr=1, ptfr=1 + b, cluster=True)
        it = sim.run_bin(itmax=3, houfr=2, mesfr=1, ptfr=1 + b, iter0=it, jobid=11)
        avg, hist = jobs[1].bin_results()
        assert np.array_equal(avg, sim.avgE)
        assert np.array_equal(hist, sim.hist)
    for s in range(ns):
        ev, od = jobs[1].get_spins(s)
        assert np.array_equal(ev, sim.spins[s, 0]) and np.array_equal(od, sim.spins[s, 1])
    batch.close()
    for j in jobs:
        j.close()


def test_upload_spins_async():
    """ea_upload_spins_async: one copy of every sample's spins, read back as
    ea_get_spins returns them."""
    import ctypes as C
    L, Lz, ln, bc, ns = MIX[3]
    betas, cum = lut(ln)
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, bc=bc, masters=MASTERS, iter0=0, jobid=3)
    rng = np.random.default_rng(5)
    nw = len(job.get_spins(0)[0])
    allw = rng.integers(0, 2 ** 63, size=(ns, 2, nw), dtype=np.int64).view(np.uint64)
    eagb._ck(eagb.lib().ea_upload_spins_async(job.ctx, eagb.P(allw)))
    job.sync()
    for s in range(ns):
        ev, od = job.get_spins(s)
        assert np.array_equal(ev, allw[s, 0]) and np.array_equal(od, allw[s, 1])
    # staged: the job's spins change only at the commit, after the kernels
    # enqueued before it (here a measurement of the previous state)
    other = rng.integers(0, 2 ** 63, size=(ns, 2, nw), dtype=np.int64).view(np.uint64)
    E0 = job.measure_energy()
    eagb._ck(eagb.lib().ea_stage_spins_async(job.ctx, eagb.P(other)))
    assert np.array_equal(job.measure_energy(), E0)
    assert np.array_equal(job.get_spins(0)[0], allw[0, 0])
    eagb._ck(eagb.lib().ea_commit_staged_spins(job.ctx))
    job.sync()
    for s in range(ns):
        ev, od = job.get_spins(s)
        assert np.array_equal(ev, other[s, 0]) and np.array_equal(od, other[s, 1])
    assert eagb.lib().ea_commit_staged_spins(job.ctx) == -4  # EA_ERR_STATE: nothing staged
    job.close()
