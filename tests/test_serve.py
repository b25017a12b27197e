"""Serving: continuous batching of simulation jobs (ea_server_*).

Jobs arrive while others run, wait for HBM budget and slots, share batched
launches with whatever else is running, and leave when their bins are done.
Each job's result must be exactly the result of the same job run alone
(ea_run_bin, bin after bin): words, energy averages, histories, swaps,
generator states and counters."""
import os
import time

import numpy as np
import pytest

import oracle_py as O
from conftest import ROOT

import importlib.util

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)

GOLD = os.path.join(ROOT, "tests", "golden")
MASTERS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)

# L, Lz, lut, bc, nsamples, NR, nbins, cadence (itmax, houfr, mesfr, ptfr, cluster)
JOBS = [
    (8, 16, "T07_16_N6", O.OBC, 3, 4, 3, (2, 2, 1, 1, 1)),
    (16, 48, "T07_16_N16", O.PBC, 2, 4, 2, (2, 2, 1, 1, 1)),
    (8, 32, "T07_16_N8", O.OBC_WEAK, 4, 4, 4, (2, 2, 1, 1, 1)),
    (16, 32, "T07_16_N24", O.OBC, 1, 4, 1, (2, 2, 1, 1, 1)),
    (8, 8, "T08_16_N4", O.PBC, 2, 8, 3, (1, 1, 2, 2, 0)),
    (24, 24, "T06_16_N32", O.PBC, 1, 4, 2, (2, 2, 1, 1, 1)),
    (8, 24, "T07_16_N12", O.OBC_STRONG, 2, 8, 2, (1, 1, 2, 2, 0)),
]


def lut(name):
    d = np.load(os.path.join(GOLD, "lut_%s.npz" % name))
    return d["betas"], d["cum"]


def masters(k):
    return tuple((x ^ ((k + 1) * 0x9E3779B97F4A7C15)) & 0xFFFFFFFFFFFFFFFF for x in MASTERS)


def run_alone(k):
    L, Lz, ln, bc, ns, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = JOBS[k]
    betas, cum = lut(ln)
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, NR=NR, bc=bc, masters=masters(k), iter0=0, jobid=100 + k)
    job.set_rng_sms(0)
    for _ in range(nbins):
        avg, hist = job.run_bin(itmax=itmax, houfr=houfr, mesfr=mesfr, ptfr=ptfr, cluster=bool(cl))
    return job, avg, hist


def submit(srv, k):
    L, Lz, ln, bc, ns, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = JOBS[k]
    betas, cum = lut(ln)
    return srv.submit(L, Lz, betas, cum, ns, NR, bc, masters(k), nbins, itmax, houfr, mesfr, ptfr,
                      cluster=bool(cl), jobid=100 + k, iter0=0)


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


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def test_job_bytes_accounts_for_cluster_buffers():
    g = eagb.geom(16, 64, 24, 4, 4, eagb.EA_OBC)
    betas, _ = lut("T07_16_N24")
    plain = eagb.job_bytes(g, eagb.Cadence(4, 10, 1, 1, 0, 0), betas)
    clus = eagb.job_bytes(g, eagb.Cadence(4, 10, 1, 1, 1, 0), betas)
    V = 16 * 16 * 64
    assert clus - plain >= 4 * V * 24 * 4 * 8        # two sets of two groups of uniforms
    spins = 4 * 2 * 24 * (4 * 4 * 16 // 2) * 4 * 8  # [s][parity][clone][half][rep] words
    assert plain >= spins
    with pytest.raises(eagb.EAError):
        eagb.job_bytes(eagb.geom(12, 64, 24, 4, 4, eagb.EA_OBC))


@pytest.mark.gpu
def test_job_bytes_bounds_device_memory():
    import torch
    k = 1
    L, Lz, ln, bc, ns, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = JOBS[k]
    betas, cum = lut(ln)
    g = eagb.geom(L, Lz, len(betas), NR, ns, bc)
    need = eagb.job_bytes(g, eagb.Cadence(itmax, houfr, mesfr, ptfr, cl, 0), betas)
    # a first job loads the kernels' modules (lazy loading), which stay
    job, _, _ = run_alone(k)
    job.close()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    job, _, _ = run_alone(k)
    job.sync()
    free1, _ = torch.cuda.mem_get_info()
    job.close()
    assert free0 - free1 <= need, (free0 - free1, need)


@pytest.mark.gpu
def test_served_jobs_equal_jobs_alone():
    """Jobs submitted in two waves (the second while the first runs), under a
    budget and slot count that make some wait: every result equals the job
    run alone."""
    sizes = []
    for k in range(len(JOBS)):
        L, Lz, ln, bc, ns, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = JOBS[k]
        betas, _ = lut(ln)
        sizes.append(eagb.job_bytes(eagb.geom(L, Lz, len(betas), NR, ns, bc),
                                    eagb.Cadence(itmax, houfr, mesfr, ptfr, cl, 0), betas))
    budget = sum(sorted(sizes)[-3:])
    srv = eagb.Server(max_jobs=4, depth=2, hbm_budget=budget)
    first = [submit(srv, k) for k in range(3)]
    t_end = time.time() + 60
    while srv.info(first[0])["state"] == eagb.EA_JOB_QUEUED and time.time() < t_end:
        time.sleep(0.001)
    later = [submit(srv, k) for k in range(3, len(JOBS))]
    tickets = first + later
    infos = []
    for k, t in enumerate(tickets):
        # a finished job holds its bytes until released, so each is checked
        # and released in turn while the others run
        served = srv.wait(t, timeout=60.0)
        infos.append(srv.info(t))
        alone, avg, hist = run_alone(k)
        bavg, bhist = served.bin_results()
        assert np.array_equal(avg, bavg), "job %d" % k
        assert np.array_equal(hist, bhist), "job %d" % k
        assert_same(alone, served)
        alone.close()
        srv.release(t)
    st = srv.stats()
    srv.drain()
    srv.close()
    assert st["completed"] == len(JOBS) and st["failed"] == 0
    assert st["bytes_peak"] <= budget
    assert st["peak_running"] >= 2
    assert st["batch_changes"] >= 3
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    # continuous batching: some job of the second wave ran while a job of the
    # first wave was still running
    overlap = any(infos[j]["t_admit"] < infos[i]["t_done"] for i in range(3) for j in range(3, len(JOBS)))
    assert overlap
    for i in infos:
        assert i["t_submit"] <= i["t_admit"] <= i["t_done"]


@pytest.mark.gpu
def test_budget_and_rejection():
    L, Lz, ln, bc, ns, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = JOBS[1]
    betas, cum = lut(ln)
    need = eagb.job_bytes(eagb.geom(L, Lz, len(betas), NR, ns, bc), eagb.Cadence(itmax, houfr, mesfr, ptfr, cl, 0),
                          betas)
    srv = eagb.Server(hbm_budget=need + need // 2)   # room for one such job at a time
    with pytest.raises(eagb.EAError):
        big = eagb.geom(L, 8 * Lz, len(betas), NR, 32, bc)
        assert eagb.job_bytes(big, eagb.Cadence(itmax, houfr, mesfr, ptfr, cl, 0), betas) > need + need // 2
        srv.submit(L, 8 * Lz, betas, cum, 32, NR, bc, masters(9), 1, itmax, houfr, mesfr, ptfr, cluster=True)
    ts = [submit(srv, 1) for _ in range(3)]
    for t in ts:
        srv.wait(t, timeout=60.0)
        srv.release(t)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 3 and st["peak_running"] == 1


SP_JOBS = [
    # L, Lz, lut, bc, nwords, NR, nbins, cadence (itmax, houfr, mesfr, ptfr, cluster)
    (5, 10, "T07_16_N6", O.PBC, 1, 4, 3, (2, 2, 1, 1, 1)),
    (7, 14, "T07_16_N8", O.OBC, 2, 2, 2, (3, 1, 1, 1, 0)),
    (6, 6, "T08_16_N4", O.OBC, 1, 4, 4, (1, 3, 1, 1, 1)),
]


def sp_alone(k):
    L, Lz, ln, bc, nw, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = SP_JOBS[k]
    betas, cum = lut(ln)
    job = eagb.SpJob(L, Lz, betas, cum, nrep=NR, nwords=nw, bc=bc, seeds=masters(50 + k), jobid=200 + k)
    for _ in range(nbins):
        avg = job.run_bin(itmax, houfr, mesfr, ptfr, cluster=bool(cl))
    return job, avg


@pytest.mark.gpu
def test_served_sample_packed_jobs_equal_jobs_alone():
    """Sample-packed jobs of odd and even L served next to multispin jobs:
    each ends exactly as the same job run alone."""
    srv = eagb.Server(max_jobs=8, depth=2)
    tickets = []
    for k in range(len(SP_JOBS)):
        L, Lz, ln, bc, nw, NR, nbins, (itmax, houfr, mesfr, ptfr, cl) = SP_JOBS[k]
        betas, cum = lut(ln)
        tickets.append(srv.submit(L, Lz, betas, cum, 1, NR, bc, masters(50 + k), nbins, itmax, houfr, mesfr, ptfr,
                                  cluster=bool(cl), jobid=200 + k, layout=eagb.EA_LAYOUT_SAMPLE_PACKED, nwords=nw))
        if k == 0:
            tickets.append(submit(srv, 0))   # a multispin job in the mix
    for t in tickets:
        srv.wait(t, timeout=60.0)
    k = 0
    for t in tickets:
        if t in srv._sp_geom:
            served = srv.sp_job(t)
            alone, avg = sp_alone(k)
            assert np.array_equal(served.get_spins(), alone.get_spins()), "sample-packed job %d" % k
            assert all(np.array_equal(a, b) for a, b in zip(served.tempering(), alone.tempering()))
            assert served.counter() == alone.counter()
            alone.close()
            k += 1
        srv.release(t)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(tickets) and st["failed"] == 0
