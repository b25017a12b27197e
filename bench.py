#!/usr/bin/env python3
"""Throughput of the EA-LCD-MC hot path on one GB300 (spin updates per picosecond).

Workload (one job, reference layout): L=24, Lz=192 tube (110,592 sites), OBC
along z, NB=32 temperatures uniform in T in [0.6, 1.6], NR=8 replicas, 31
disorder samples (the most one reference process takes); Metropolis + energy + parallel tempering every sweep and a
Houdayer move on the colder half every 5 sweeps.  One step = 5 x (sweep +
energy + PT) + 1 Houdayer move = 5 * V * NR * NB * 32 spin updates.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores (the oracle's
C restatement, all threads) on a bounded sample of the same workload.
Prints one JSON line (rank 0).
"""
import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
L, LZ, NR, NS, HOUFR = 24, 192, 8, 31, 5
LUT = os.path.join(ROOT, "tests", "golden", "lut_T06_16_N32.npz")
MASTERS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)
WORKLOAD = "L24_Lz192_OBC_NB32_NR8_ns31_ptfr1_houfr5"
# DRAM bytes (read + write) of one k_sweep launch of this workload, from the
# ncu capture of one k_sweep launch of the bench (its full-set capture)
KSWEEP_DRAM_BYTES = 140.6e6
# The integer-op model of the fused sweep (the Philox4x32-10 rounds, the
# post-mix and rotation of a random word, the threshold search per byte, the
# bit-sliced update per word), in 32-bit operations: 6 Philox calls of
# 78 + 18 + 4 ops and 24 searches of 6 + 6 x (iterations) ops per random
# triple, 60 ops per updated word.
OPS_TRIPLE_BASE, OPS_PER_ITER, OPS_WORD = 6 * (78 + 18 + 4) + 24 * 6, 24 * 6, 60
# mixed-geometry workload of the batched vs plain comparison: every
# L x (Lz/L) x boundary x NT combination is one job class
# (36 geometry classes; either 36 jobs of 32 samples or 288 jobs of 4)
MIX_L, MIX_RATIO, MIX_NT, MIX_NR, MIX_HOUFR = (8, 16), (2, 4, 8), (16, 24, 32), 4, 10
MIX_WORKLOAD = "mixed_L8-16_Lz2-8L_PBC-OBC_NT16-32_NR4_ns%d_ptfr1_houfr10"


def load_eagb():
    spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def lut_search_iters(cum):
    """Expected iterations of the threshold search of one byte for a uniform
    64-bit R: the bisection between the bounds of the 8-bit pre-search
    (lut_byte in kernels_dev.cuh), weighted by the exact probability of each
    result byte within each of the 256 pre-search buckets."""
    c = [int(x) for x in np.asarray(cum, np.uint64)]

    def first_above(R):
        n = 0
        while n < 255 and not R < c[n]:
            n += 1
        return n

    tot = 0
    for t in range(256):
        lo_r, hi_r = t << 56, ((t + 1) << 56) - 1
        a0, b0 = first_above(lo_r), first_above(hi_r)
        for n in range(a0, b0 + 1):
            lo = max(c[n - 1] if n > 0 else 0, lo_r)
            hi = hi_r if n == 255 else min(c[n] - 1, hi_r)
            if hi < lo:
                continue
            a, b, d = a0, b0, 0
            while a < b:
                m = (a + b) >> 1
                d += 1
                if n <= m:
                    b = m
                else:
                    a = m + 1
            tot += (hi - lo + 1) * d
    return tot / float(1 << 64)


def lut_search_iters11(cum):
    """The same expectation for the 11-bit pre-search of the per-item pass
    (lut_byte11): bucket t = R >> 53 searches [pre[t], pre[t+1]], pre[t] the
    first byte whose threshold is above t << 53."""
    c = [int(x) for x in np.asarray(cum, np.uint64)]

    def first_above(R):
        lo, hi = 0, 255
        while lo < hi:
            m = (lo + hi) >> 1
            if R < c[m]:
                hi = m
            else:
                lo = m + 1
        return lo

    pre = [first_above(t << 53) for t in range(2048)] + [255]
    tot = 0
    for t in range(2048):
        a0, b0 = pre[t], pre[t + 1]
        if a0 == b0:
            continue
        lo_r, hi_r = t << 53, ((t + 1) << 53) - 1
        for n in range(a0, b0 + 1):
            lo = max(c[n - 1] if n > 0 else 0, lo_r)
            hi = hi_r if n == 255 else min(c[n] - 1, hi_r)
            if hi < lo:
                continue
            a, b, d = a0, b0, 0
            while a < b:
                m = (a + b) >> 1
                d += 1
                if n <= m:
                    b = m
                else:
                    a = m + 1
            tot += (hi - lo + 1) * d
    return tot / float(1 << 64)


def int_ops(cums, triples, words, iters=lut_search_iters):
    """32-bit integer operations of a launch that draws `triples` random
    triples (spread evenly over the temperatures of `cums`) and updates
    `words` spin words."""
    e = float(np.mean([iters(c) for c in cums]))
    return triples * (OPS_TRIPLE_BASE + OPS_PER_ITER * e) + words * OPS_WORD, e


_int_peak = None


def int_peak(eagb, dev):
    """Measured 32-bit integer instruction rate of this GPU (ops/s, all SMs)."""
    global _int_peak
    if _int_peak is None:
        alu, imad = C.c_double(), C.c_double()
        eagb._ck(eagb.lib().ea_probe_int32_rate(dev, C.byref(alu), C.byref(imad)))
        _int_peak = (alu.value, imad.value)
    return _int_peak


def headline_config():
    """The workload of the headline line, the same for both arms."""
    return {"workload": WORKLOAD, "L": L, "Lz": LZ, "nbetas": 32, "nrep": NR, "nsamples": NS, "bc": "OBC",
            "ptfr": 1, "houfr": HOUFR, "cluster": "Houdayer move on the colder half every 5 sweeps",
            "step": "5 x (sweep + energy + parallel tempering) + 1 Houdayer move + energy measurement",
            "l2": "flushed between steps (512 MB write)"}


class Clocks:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def cpu_cycle(nsteps, warmup=0):
    """The reference algorithm on the host cores (the oracle's C restatement,
    OpenMP over every core): the headline workload itself -- 31 samples, the
    same cadence as one GPU step (5 x (sweep + energy + FP64 parallel
    tempering) + a Houdayer move with the host cuRAND generator + the energy
    measurement) -- for `warmup` untimed and `nsteps` timed steps.  Returns
    (spin updates, seconds) of the timed steps."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_py as O
    d = np.load(LUT)
    sim = O.Sim(L, LZ, d["betas"], d["cum"], nbits=NS, NR=NR, bc=O.OBC, masters=MASTERS, itmax=1)
    it, dt = 0, 0.0
    for i in range(warmup + nsteps):
        t0 = time.perf_counter()
        it = sim.run_bin(itmax=1, houfr=HOUFR, mesfr=1, ptfr=1, iter0=it, jobid=0, cluster=True)
        if i >= warmup:
            dt += time.perf_counter() - t0
    return HOUFR * L * L * LZ * NR * len(d["betas"]) * NS * nsteps, dt


CPU_SAMPLE = ("31 samples x the full step of the GPU arm (5 sweeps with energy and FP64 tempering, a Houdayer "
              "move with host cuRAND uniforms, the energy measurement), oracle C restatement, OpenMP")


def max_over_ranks(torch, vals, device, world):
    """Each timing as the slowest rank saw it (every rank runs its own
    replica; whole-job throughput = all ranks' work / this time)."""
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t]


def run_reference(args, rank, world):
    if rank != 0:
        return
    n = os.cpu_count() or 1
    su, dt = cpu_cycle(args.steps, args.warmup)
    value = su / dt / 1e12
    line = {"metric": "spin_updates_per_ps", "value": value, "unit": "spin-updates/ps", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded couplings and spins as the reference generates them)",
            "config": headline_config(),
            "cpu_baseline": {"value": value, "unit": "spin-updates/ps", "cores": n, "kind": "port",
                             "sample": CPU_SAMPLE + "; every step of the run"},
            "e2e": {"value": value, "unit": "spin-updates/ps", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def mixed_jobs(eagb, dev, ns, copies):
    jobs = []
    for _ in range(copies):
        for L in MIX_L:
            for ratio in MIX_RATIO:
                for bc in (eagb.EA_PBC, eagb.EA_OBC):
                    for nt in MIX_NT:
                        d = np.load(os.path.join(ROOT, "tests", "golden", "lut_T07_16_N%d.npz" % nt))
                        k = len(jobs)
                        m = tuple((x ^ (0x9E3779B97F4A7C15 * (k + 1))) & 0xFFFFFFFFFFFFFFFF or 1 for x in MASTERS)
                        job = eagb.new_job(L, ratio * L, d["betas"], d["cum"], nsamples=ns, NR=MIX_NR, bc=bc,
                                           masters=m, device=dev, jobid=k)
                        job.set_rng_sms(0)
                        jobs.append(job)
    return jobs


def timed_sequential(torch, dev, jobs, enqueue_one, steps, join=None):
    """The plain form run one geometry after another: each job's bin starts
    when the previous job's bin has ended (device-side ordering through events,
    no host synchronisation); CUDA-event time in ms."""
    s0 = torch.cuda.Stream(device=dev)
    streams = [torch.cuda.ExternalStream(j.stream(), device=dev) for j in jobs]
    torch.cuda.synchronize(dev)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(s0)
    prev = t0
    for _ in range(steps):
        for j, st in zip(jobs, streams):
            st.wait_event(prev)
            enqueue_one(j)
            if join:
                join(j)
            prev = torch.cuda.Event()
            prev.record(st)
    s0.wait_event(prev)
    t1.record(s0)
    torch.cuda.synchronize(dev)
    return t0.elapsed_time(t1)


def run_mixed(args, dev, torch, eagb, ns, copies):
    """Batched persistent form vs plain form (one job per launch sequence, every
    job on its own stream, all enqueued before waiting; and the same jobs one
    geometry after another) on the same mixed workload, from twin initial
    states; one step = one bin of itmax=1 for every job.  Inputs (spins +
    uniforms) are far larger than L2."""
    su_step = 0
    plain, batched = mixed_jobs(eagb, dev, ns, copies), mixed_jobs(eagb, dev, ns, copies)
    for j in plain:
        su_step += MIX_HOUFR * j.g.L * j.g.L * j.g.Lz * MIX_NR * j.g.nbetas * ns
    batch = eagb.Batch(batched)
    s0 = torch.cuda.Stream(device=dev)
    cad = dict(itmax=1, houfr=MIX_HOUFR, mesfr=1, ptfr=1)

    def timed(jobs, enqueue, steps):
        streams = [torch.cuda.ExternalStream(j.stream(), device=dev) for j in jobs]
        torch.cuda.synchronize(dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(s0)
        for st in streams:
            st.wait_event(t0)
        for _ in range(steps):
            enqueue()
        for j, st in zip(jobs, streams):
            j.join()
            e = torch.cuda.Event()
            e.record(st)
            s0.wait_event(e)
        t1.record(s0)
        torch.cuda.synchronize(dev)
        return t0.elapsed_time(t1)

    def plain_step():
        for j in plain:
            j.run_cycles(**cad)

    def batch_step():
        batch.run_bin(**cad)

    timed(plain, plain_step, args.warmup)
    timed(batched, batch_step, args.warmup)
    ms_plain = timed(plain, plain_step, args.steps)
    ms_batch = timed(batched, batch_step, args.steps)
    same = True
    for a, b in zip(plain, batched):
        for smp in range(ns):
            ea, oa = a.get_spins(smp)
            eb, ob = b.get_spins(smp)
            same = same and np.array_equal(ea, eb) and np.array_equal(oa, ob)
        same = same and np.array_equal(a.bin_results()[0], b.bin_results()[0])
    tile = batch.tile()
    batch.close()
    # the same plain jobs, one geometry after another (after the check)
    seq_steps = max(1, args.steps // 4)
    ms_seq = timed_sequential(torch, dev, plain, lambda j: j.run_cycles(**cad), seq_steps, join=lambda j: j.join())
    for j in plain + batched:
        j.close()
    vp = su_step * args.steps / (ms_plain * 1e-3) / 1e12
    vb = su_step * args.steps / (ms_batch * 1e-3) / 1e12
    vs = su_step * seq_steps / (ms_seq * 1e-3) / 1e12
    return {"workload": MIX_WORKLOAD % ns, "jobs": len(plain), "unit": "spin-updates/ps",
            "plain_value": vp, "batched_value": vb, "speedup": vb / vp,
            "plain_sequential_value": vs, "speedup_vs_sequential": vb / vs,
            "plain_ms_per_step": ms_plain / args.steps, "batched_ms_per_step": ms_batch / args.steps,
            "spin_updates_per_step": su_step, "bit_exact_plain_vs_batched": bool(same), "tile": tile,
            "graph": "sweep/energy/tempering cycle replayed as a CUDA graph",
            "l2": "inputs larger than L2 (spins ~0.3 GB, uniforms ~9 GB)"}


# serving stream: Poisson arrivals of jobs with L in {8, 16} (the multiples of
# 8 in 6..20), Lz/L in {1,2,4,8,16}, PBC/OBC, NT in {8,12,16,24,32} over
# T in [0.7, 1.6], 8 samples, NR=4, a Houdayer move on the colder half every
# 10 sweeps; sweeps log-uniform in 2^8..2^14 (the 2^14..2^20 range scaled by
# 1/64 so that the stream lasts about half a minute), in bins of 20 sweeps
SERVE_WORKLOAD = "poisson_L8-16_LzL1-16_PBC-OBC_NT8-32_NR4_ns8_houfr10_sweeps2^8-2^14"
SERVE_NT, SERVE_NS, SERVE_NR = (8, 12, 16, 24, 32), 8, 4


def serve_stream(njobs, seed=7):
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(njobs):
        L = int(rng.choice([8, 16]))
        Lz = L * int(rng.choice([1, 2, 4, 8, 16]))
        bc = int(rng.integers(0, 2))
        nt = int(rng.choice(SERVE_NT))
        sweeps = int(round(2.0 ** rng.uniform(8, 14)))
        nbins = max(1, int(round(sweeps / 20.0)))
        jobs.append((L, Lz, bc, nt, nbins))
    return jobs


# the same stream shape with the sample-packed layout, which takes every
# L in 6..20: 64 samples per job, NR=4, sweeps log-uniform in 2^6..2^12 (the
# 2^14..2^20 range scaled by 1/256), in bins of 10 sweeps
SERVE_SP_WORKLOAD = "poisson_L6-20_LzL1-16_PBC-OBC_NT8-32_NR4_64samples_houfr10_sweeps2^6-2^12"


def serve_sp_stream(njobs, seed=9):
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(njobs):
        L = int(rng.integers(6, 21))
        Lz = L * int(rng.choice([1, 2, 4, 8, 16]))
        bc = int(rng.integers(0, 2))
        nt = int(rng.choice(SERVE_NT))
        sweeps = int(round(2.0 ** rng.uniform(6, 12)))
        jobs.append((L, Lz, bc, nt, max(1, int(round(sweeps / 10.0)))))
    return jobs


def run_serve_stream(dev, eagb, stream, sweeps_per_bin, submit_kw, su_of, capacity, util, workload, seed,
                     t_limit=600.0):
    """A Poisson stream of jobs through a server: p50/p99 completion latency
    and spin-updates/ps of the completed work."""
    import threading
    luts = {nt: np.load(os.path.join(ROOT, "tests", "golden", "lut_T07_16_N%d.npz" % nt)) for nt in SERVE_NT}
    njobs = len(stream)
    su = [su_of(*j) for j in stream]
    rate = util / (np.mean(su) / capacity)
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, size=njobs)
    srv = eagb.Server(device=dev, nb_max=32, depth=2)
    tickets = [None] * njobs
    err = []

    def producer():
        t = time.perf_counter()
        try:
            for k, (L, Lz, bc, nt, nb) in enumerate(stream):
                t += gaps[k]
                d = time.perf_counter()
                if t > d:
                    time.sleep(t - d)
                m = tuple((x ^ (0x9E3779B97F4A7C15 * (k + 1))) & 0xFFFFFFFFFFFFFFFF or 1 for x in MASTERS)
                tickets[k] = srv.submit(L, Lz, luts[nt]["betas"], luts[nt]["cum"], nbins=nb, masters=m,
                                        bc=bc, jobid=k & 0x3FFF, **submit_kw)
        except Exception as e:  # reported below
            err.append(e)

    th = threading.Thread(target=producer)
    th.start()
    # a finished job holds its bytes until released: release each as soon as
    # it is done, whatever the order
    done = [False] * njobs
    t_limit = time.perf_counter() + t_limit
    while not all(done) and time.perf_counter() < t_limit:
        for k in range(njobs):
            if done[k] or tickets[k] is None:
                continue
            st = srv.info(tickets[k])["state"]
            if st == eagb.EA_JOB_DONE:
                srv.release(tickets[k])
                done[k] = True
            elif st == eagb.EA_JOB_FAILED:
                srv.wait(tickets[k], timeout=0.0)   # raises with the job's error
        if not th.is_alive() and any(t is None for t in tickets):
            break
        time.sleep(0.0005)
    th.join()
    if err:
        raise err[0]
    st = srv.stats()
    srv.close()
    return {"workload": workload, "jobs": njobs, "arrival_rate_per_s": rate, "offered_load": util,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
            "value": st["spin_updates"] / st["span_s"] / 1e12, "unit": "spin-updates/ps",
            "span_s": st["span_s"], "completed": st["completed"], "failed": st["failed"],
            "peak_running": st["peak_running"], "bins": st["bins"], "batch_changes": st["batch_changes"],
            "hbm_budget": st["budget"], "hbm_peak": st["bytes_peak"], "gpu_busy_s": st["gpu_busy_s"],
            "host_enqueue_s": st["enqueue_s"], "host_admit_s": st["admit_s"],
            "latency_components_ms": {k: st[k + "_ms"] for k in
                                      ("queue_p50", "queue_p99", "prep_p50", "prep_p99", "start_p50", "start_p99",
                                       "run_p50", "run_p99", "gpu_p50", "gpu_p99")}}


# the serving configuration at its stated size: L uniform in 6..20, Lz/L in
# {1,2,4,8,16}, PBC/OBC, NT in {8..32}, 64 samples per job, NR=4, a Houdayer
# move every 10 sweeps, sweeps log-uniform in 2^14..2^20 (bins of 100 sweeps);
# a bounded number of jobs drawn from it (a job averages ~2e13 spin updates)
SERVE_C5_WORKLOAD = "poisson_L6-20_LzL1-16_PBC-OBC_NT8-32_NR4_64samples_houfr10_sweeps2^14-2^20"


def serve_c5_stream(njobs, seed=5):
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(njobs):
        L = int(rng.integers(6, 21))
        Lz = L * int(rng.choice([1, 2, 4, 8, 16]))
        bc = int(rng.integers(0, 2))
        nt = int(rng.choice(SERVE_NT))
        sweeps = int(round(2.0 ** rng.uniform(14, 20)))
        jobs.append((L, Lz, bc, nt, max(1, int(round(sweeps / 100.0)))))
    return jobs


def run_serve_c5(args, dev, eagb, njobs, util=0.8):
    stream = serve_c5_stream(njobs)
    kw = dict(nsamples=1, NR=SERVE_NR, itmax=10, houfr=10, mesfr=1, ptfr=1, cluster=True,
              layout=eagb.EA_LAYOUT_SAMPLE_PACKED, nwords=1)
    su_of = lambda L, Lz, bc, nt, nb: 100 * nb * L * L * Lz * SERVE_NR * nt * 64
    rec = run_serve_stream(dev, eagb, stream, 100, kw, su_of, 0.5e12, util, SERVE_C5_WORKLOAD, 17,
                           t_limit=3600.0)
    rec["jobs_drawn"] = [{"L": L, "Lz": Lz, "bc": bc, "nt": nt, "sweeps": 100 * nb} for L, Lz, bc, nt, nb in stream]
    return rec


def run_serve_sp(args, dev, eagb, njobs=100, util=0.8):
    stream = serve_sp_stream(njobs)
    kw = dict(nsamples=1, NR=SERVE_NR, itmax=1, houfr=10, mesfr=1, ptfr=1, cluster=True,
              layout=eagb.EA_LAYOUT_SAMPLE_PACKED, nwords=1)
    su_of = lambda L, Lz, bc, nt, nb: 10 * nb * L * L * Lz * SERVE_NR * nt * 64
    return run_serve_stream(dev, eagb, stream, 10, kw, su_of, 0.3e12, util, SERVE_SP_WORKLOAD, 13)


def run_serve(args, dev, eagb, njobs=240, util=0.8):
    """Continuous batching server under a Poisson stream of multispin jobs
    (batched with their class)."""
    stream = serve_stream(njobs)
    kw = dict(nsamples=SERVE_NS, NR=SERVE_NR, itmax=2, houfr=10, mesfr=1, ptfr=1, cluster=True)
    su_of = lambda L, Lz, bc, nt, nb: 20 * nb * L * L * Lz * SERVE_NR * nt * SERVE_NS
    return run_serve_stream(dev, eagb, stream, 20, kw, su_of, 0.6e12, util, SERVE_WORKLOAD, 11)


# sample-packed layout (64 samples per word): the small-tube and cluster-path
# configurations, and a wide job of 64 words (4096 samples)
SP_FORMS = {1: "graph", 2: "persistent", 3: "resident"}
SP_CASES = [
    # name, L, Lz, bc, lut, NR, nwords, cadence of one step (itmax, houfr, ptfr, cluster), steps
    ("L6_Lz24_PBC_NT12_NR2_64samples_ptfr1", 6, 24, 0, "T08_16_N12", 2, 1, (512, 1, 1, False), 8),
    ("L12_Lz48_OBC_NT24_NR4_64samples_houfr10", 12, 48, 1, "T07_16_N24", 4, 1, (10, 10, 1, True), 10),
    ("L12_Lz48_OBC_NT24_NR4_4096samples_houfr10", 12, 48, 1, "T07_16_N24", 4, 64, (2, 10, 1, True), 10),
    # the large tube as written: NR=4, 64 samples per word, Houdayer every 5 sweeps on the colder half
    ("L24_Lz192_OBC_NT32_NR4_64samples_houfr5", 24, 192, 1, "T06_16_N32", 4, 1, (1, 5, 1, True), 10),
]


def run_sp(args, dev, torch, eagb):
    """Sample-packed jobs: device-timed spin updates per ps over whole bins
    (sweeps, tempering every sweep, Houdayer moves, energy measurements)."""
    out = []
    for name, Lx, Lz, bc, ln, NR, nw, (itmax, houfr, ptfr, cl), steps in SP_CASES:
        if args.sp_case and args.sp_case not in name:
            continue
        if args.sp_case:
            steps = args.steps
        d = np.load(os.path.join(ROOT, "tests", "golden", "lut_%s.npz" % ln))
        cad = dict(itmax=itmax, houfr=houfr, mesfr=1, ptfr=ptfr, cluster=cl)

        def timed(mode):
            job = eagb.SpJob(Lx, Lz, d["betas"], d["cum"], nrep=NR, nwords=nw, bc=bc, seeds=MASTERS, device=dev)
            job.set_bin_kernel(mode)
            form = SP_FORMS[job.bin_kernel_for(**cad)]
            if form != "resident":
                tuned[:] = job.autotune()   # tile width, energy sites per thread, labelling block size
            st = torch.cuda.ExternalStream(job.stream(), device=dev)
            for _ in range(max(1, args.warmup)):
                job.run_async(**cad)
            job.sync()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(st)
            for _ in range(steps):
                job.run_async(**cad)
            t1.record(st)
            job.sync()
            ms = t0.elapsed_time(t1)
            ncol, kt = job.info()
            S = job.get_spins()
            if form != "resident":
                # the colour passes alone (counter fills + passes of 20 sweeps)
                t0.record(st)
                job.sweeps(20)
                t1.record(st)
                job.sync()
                pass_us[0] = 1e3 * t0.elapsed_time(t1) / 20
            job.close()
            return ms, form, ncol, kt, S

        tuned = [0, 0, 0]
        pass_us = [0.0]
        ms, form, ncol, kt, S = timed(eagb.EA_BIN_AUTO)
        V = Lx * Lx * Lz
        sweeps = steps * itmax * houfr * ptfr
        su = sweeps * V * NR * len(d["betas"]) * 64 * nw
        rec = {"workload": name, "value": su / (ms * 1e-3) / 1e12, "unit": "spin-updates/ps",
               "sweeps": sweeps, "ms": ms, "us_per_sweep": 1e3 * ms / sweeps, "colours": ncol, "tile": kt,
               "samples": 64 * nw, "bin_kernel": form, "l2": "job of %.1f MB" % (V * NR * len(d["betas"]) * nw * 8 / 1e6)}
        if form != "resident":
            rec["autotuned"] = {"tile": tuned[0], "energy_sites_per_thread": tuned[1], "labelling_threads": tuned[2]}
            # roofline of the colour passes of one sweep: 24 B per spin word
            # (read + write it, read it once as a neighbour) + 48 B of
            # couplings per (site, sample word); integer ops of the random
            # triples (one per site, replica and slot, shared by the words)
            # and the word updates, the search iterations of the pass's
            # pre-search (11 bits for the per-item pass, 8 for tiles)
            hbm, _ = peaks()
            ipk_alu, _ = int_peak(eagb, dev)
            words = V * NR * len(d["betas"]) * nw
            pbytes = words * 24 + V * nw * 48
            ops, e_it = int_ops(d["cum"], V * NR * len(d["betas"]), words,
                                lut_search_iters11 if kt == 0 else lut_search_iters)
            hf = pbytes / (pass_us[0] * 1e-6) / 1e9 / hbm
            inf = ops / (pass_us[0] * 1e-6) / ipk_alu
            rec["pass"] = {"form": "per-item" if kt == 0 else "tiles of %d sites" % kt,
                           "us_per_sweep": pass_us[0], "bound": "int32" if inf > hf else "hbm",
                           "frac": max(hf, inf), "hbm_frac": hf, "int_frac": inf,
                           "alg_bytes_per_sweep": pbytes, "int_ops_per_sweep": ops,
                           "search_iterations_per_byte": e_it}
        if form == "resident":
            # the same bins as a graph of per-phase launches, from the same start
            gms, _, _, _, gS = timed(eagb.EA_BIN_GRAPH)
            rec["graph"] = {"us_per_sweep": 1e3 * gms / sweeps, "value": su / (gms * 1e-3) / 1e12,
                            "bit_exact": bool(np.array_equal(S, gS))}
        out.append(rec)
    return out


# batching configuration with the sample-packed layout: every L x (Lz/L) x
# boundary x NT class of L in {8,10,12,16}, Lz/L in {2,4,8}, NT in
# {16,24,32} (72 classes) as one job; 4096 sample words (262,144 samples) in
# all, NR=2, a Houdayer move every 10 sweeps
SPMIX_L, SPMIX_RATIO, SPMIX_NT, SPMIX_WORDS, SPMIX_NR = (8, 10, 12, 16), (2, 4, 8), (16, 24, 32), 4096, 2
SPMIX_WORKLOAD = "mixed_L8-16_Lz2-8L_PBC-OBC_NT16-32_NR2_%dwords_houfr10"


def spmix_jobs(eagb, dev, nwords):
    classes = [(L, r * L, bc, nt) for L in SPMIX_L for r in SPMIX_RATIO for bc in (0, 1) for nt in SPMIX_NT]
    words = [nwords // len(classes) + (1 if k < nwords % len(classes) else 0) for k in range(len(classes))]
    jobs = []
    for k, ((L, Lz, bc, nt), nw) in enumerate(zip(classes, words)):
        d = np.load(os.path.join(ROOT, "tests", "golden", "lut_T07_16_N%d.npz" % nt))
        m = tuple((x ^ (0x9E3779B97F4A7C15 * (k + 1))) & 0xFFFFFFFFFFFFFFFF or 1 for x in MASTERS)
        jobs.append(eagb.SpJob(L, Lz, d["betas"], d["cum"], nrep=SPMIX_NR, nwords=nw, bc=bc, seeds=m, jobid=k,
                               device=dev))
    return jobs


def run_mixed_sp(args, dev, torch, eagb, nwords=SPMIX_WORDS, steps=2):
    """Sample-packed batching: one bin (10 sweeps + tempering each sweep, one
    Houdayer move, a measurement) of every class job, plain (one job per
    launch sequence, each on its own stream, all enqueued before waiting) vs
    batched (one launch per kernel kind for all 72 jobs), from twin states."""
    plain, batched = spmix_jobs(eagb, dev, nwords), spmix_jobs(eagb, dev, nwords)
    batch = eagb.SpBatch(batched)
    cad = dict(itmax=1, houfr=10, mesfr=1, ptfr=1, cluster=True)
    su_step = sum(10 * j.V * SPMIX_NR * j.g.nbetas * 64 * j.g.nwords for j in plain)
    spin_bytes = sum(8.0 * j.V * SPMIX_NR * j.g.nbetas * j.g.nwords for j in plain)
    s0 = torch.cuda.Stream(device=dev)

    def timed(streams_of, enqueue, n):
        streams = [torch.cuda.ExternalStream(h, device=dev) for h in streams_of]
        torch.cuda.synchronize(dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(s0)
        for st in streams:
            st.wait_event(t0)
        for _ in range(n):
            enqueue()
        for st in streams:
            e = torch.cuda.Event()
            e.record(st)
            s0.wait_event(e)
        t1.record(s0)
        torch.cuda.synchronize(dev)
        return t0.elapsed_time(t1)

    def plain_step():
        for j in plain:
            j.run_async(**cad)

    def batch_step():
        batch.run_bin(**cad)

    pstreams = [j.stream() for j in plain]
    bstreams = [batch.stream()]
    timed(pstreams, plain_step, 1)
    timed(bstreams, batch_step, 1)
    ms_plain = timed(pstreams, plain_step, steps)
    ms_batch = timed(bstreams, batch_step, steps)
    same = all(np.array_equal(a.get_spins(), b.get_spins()) for a, b in zip(plain, batched))
    batch.close()
    # the same plain jobs, one geometry after another (after the check)
    ms_seq = timed_sequential(torch, dev, plain, lambda j: j.run_async(**cad), steps)
    for j in plain + batched:
        j.close()
    vp = su_step * steps / (ms_plain * 1e-3) / 1e12
    vb = su_step * steps / (ms_batch * 1e-3) / 1e12
    vs = su_step * steps / (ms_seq * 1e-3) / 1e12
    return {"workload": SPMIX_WORKLOAD % nwords, "jobs": len(plain), "samples": 64 * nwords, "unit": "spin-updates/ps",
            "plain_value": vp, "batched_value": vb, "speedup": vb / vp, "plain_ms_per_step": ms_plain / steps,
            "plain_sequential_value": vs, "speedup_vs_sequential": vb / vs,
            "batched_ms_per_step": ms_batch / steps, "spin_updates_per_step": su_step,
            "bit_exact_plain_vs_batched": bool(same),
            "graph": "one bin iteration of the batch replayed as a CUDA graph",
            "l2": "spin words %.2f GB against a 129 MB L2" % (spin_bytes / 1e9)}


def run_no_cluster(args, dev, torch, eagb):
    """The headline geometry without cluster moves: one step = 5 x (sweep +
    energy + parallel tempering) + the energy measurement, so the fused sweep
    is most of the step (the cluster uniforms, which bound the full step, are
    not drawn).  Device-timed, L2 flushed between steps."""
    d = np.load(LUT)
    betas, cum = d["betas"], d["cum"]
    NB = len(betas)
    job = eagb.new_job(L, LZ, betas, cum, nsamples=NS, NR=NR, bc=eagb.EA_OBC, masters=MASTERS, device=dev, jobid=1)
    job.set_rng_sms(0)
    stream = torch.cuda.ExternalStream(job.stream(), device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)
    cad = dict(itmax=1, houfr=HOUFR, mesfr=1, ptfr=1, cluster=False)
    for _ in range(args.warmup):
        job.run_cycles(**cad)
    job.sync()
    eagb._ck(eagb.lib().ea_profile(job.ctx, 1))
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i)
            evs[i][0].record(stream)
            job.run_cycles(**cad)
            evs[i][1].record(stream)
    job.sync()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    nsw, sw_ms = C.c_int64(), C.c_double()
    eagb._ck(eagb.lib().ea_kernel_time(job.ctx, 0, C.byref(nsw), C.byref(sw_ms)))
    eagb._ck(eagb.lib().ea_profile(job.ctx, 0))
    job.close()
    su = HOUFR * L * L * LZ * NR * NB * NS * args.steps
    half = (L // 4) ** 2 * (LZ // 4) // 2
    words = NS * NB * half * NR
    launch_ms = sw_ms.value / max(1, nsw.value)
    ops, e = int_ops(cum, NB * half * NR, words)
    ipk = int_peak(eagb, dev)[0]
    hbm, _ = peaks()
    return {"workload": WORKLOAD.replace("_houfr5", "_no_cluster"), "value": su / (ms * 1e-3) / 1e12,
            "unit": "spin-updates/ps", "ms_per_step": ms / args.steps, "sweep_launch_ms": launch_ms,
            "sweep_share": sw_ms.value / ms,
            "sweep_int_frac": ops / (launch_ms * 1e-3) / ipk,
            "sweep_hbm_frac": (words * 24 + NS * 6 * half * 8) / (launch_ms * 1e-3) / 1e9 / hbm,
            "l2": "flushed between steps (512 MB write)"}


# many small sample-packed jobs: the serving configuration's distribution
# (L in 6..20, Lz/L in {1,2,4,8,16}, PBC/OBC, NT in {8..32}, 64 samples, NR=4)
# restricted to jobs of at most 2^20 spin words; one bin = 2 x (10 sweeps +
# tempering each sweep + a Houdayer move) + measurements
SPSMALL_WORKLOAD = "mixed_small_L6-20_LzL1-16_PBC-OBC_NT8-32_NR4_64samples_houfr10_%djobs"


def spsmall_jobs(eagb, dev, njobs, seed=21):
    rng = np.random.default_rng(seed)
    specs = []
    while len(specs) < njobs:
        L = int(rng.integers(6, 21))
        Lz = L * int(rng.choice([1, 2, 4, 8, 16]))
        bc = int(rng.integers(0, 2))
        nt = int(rng.choice(SERVE_NT))
        if L * L * Lz * SERVE_NR * nt <= (1 << 20):
            specs.append((L, Lz, bc, nt))
    luts = {nt: np.load(os.path.join(ROOT, "tests", "golden", "lut_T07_16_N%d.npz" % nt)) for nt in SERVE_NT}
    jobs = []
    for k, (L, Lz, bc, nt) in enumerate(specs):
        m = tuple((x ^ (0x9E3779B97F4A7C15 * (k + 1))) & 0xFFFFFFFFFFFFFFFF or 1 for x in MASTERS)
        jobs.append(eagb.SpJob(L, Lz, luts[nt]["betas"], luts[nt]["cum"], nrep=SERVE_NR, nwords=1, bc=bc, seeds=m,
                               jobid=k, device=dev))
    return jobs


def run_small_sp(args, dev, torch, eagb, njobs=64, steps=3):
    """Sample-packed batching where jobs are small: plain (each job's bin a
    graph on its own stream, all enqueued before waiting) vs batched (one
    cooperative launch of the persistent bin kernel for every job), from twin
    states; bit-exact check."""
    plain, batched, graphed = (spsmall_jobs(eagb, dev, njobs), spsmall_jobs(eagb, dev, njobs),
                               spsmall_jobs(eagb, dev, njobs))
    batch = eagb.SpBatch(batched)
    batch.set_bin_kernel(eagb.EA_BIN_PERSISTENT)
    gbatch = eagb.SpBatch(graphed)
    gbatch.set_bin_kernel(eagb.EA_BIN_GRAPH)
    cad = dict(itmax=2, houfr=10, mesfr=1, ptfr=1, cluster=True)
    su_step = sum(20 * j.V * SERVE_NR * j.g.nbetas * 64 for j in plain)
    s0 = torch.cuda.Stream(device=dev)

    def timed(streams_of, enqueue, n):
        streams = [torch.cuda.ExternalStream(h, device=dev) for h in streams_of]
        torch.cuda.synchronize(dev)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(s0)
        for st in streams:
            st.wait_event(t0)
        for _ in range(n):
            enqueue()
        for st in streams:
            e = torch.cuda.Event()
            e.record(st)
            s0.wait_event(e)
        t1.record(s0)
        torch.cuda.synchronize(dev)
        return t0.elapsed_time(t1)

    def plain_step():
        for j in plain:
            j.run_async(**cad)

    pstreams = [j.stream() for j in plain]
    bstreams = [batch.stream()]
    timed(pstreams, plain_step, 1)
    gstreams = [gbatch.stream()]
    timed(bstreams, lambda: batch.run_bin(**cad), 1)
    timed(gstreams, lambda: gbatch.run_bin(**cad), 1)
    batch.sync()
    gbatch.sync()
    ms_plain = timed(pstreams, plain_step, steps)
    ms_batch = timed(bstreams, lambda: batch.run_bin(**cad), steps)
    ms_graph = timed(gstreams, lambda: gbatch.run_bin(**cad), steps)
    batch.sync()
    gbatch.sync()
    same = all(np.array_equal(a.get_spins(), b.get_spins()) and np.array_equal(a.get_spins(), c.get_spins())
               for a, b, c in zip(plain, batched, graphed))
    same = same and all(np.array_equal(a.bin_results(), b.bin_results()) for a, b in zip(plain, batched))
    batch.close()
    gbatch.close()
    ms_seq = timed_sequential(torch, dev, plain, lambda j: j.run_async(**cad), 1)
    for j in plain + batched + graphed:
        j.close()
    vp = su_step * steps / (ms_plain * 1e-3) / 1e12
    vb = su_step * steps / (ms_batch * 1e-3) / 1e12
    vs = su_step / (ms_seq * 1e-3) / 1e12
    vg = su_step * steps / (ms_graph * 1e-3) / 1e12
    return {"workload": SPSMALL_WORKLOAD % njobs, "jobs": njobs, "unit": "spin-updates/ps",
            "plain_value": vp, "batched_value": vb, "speedup": vb / vp,
            "batched_graph_value": vg, "speedup_graph": vg / vp,
            "plain_sequential_value": vs, "speedup_vs_sequential": vb / vs,
            "plain_ms_per_step": ms_plain / steps, "batched_ms_per_step": ms_batch / steps,
            "spin_updates_per_step": su_step, "bit_exact_plain_vs_batched": bool(same),
            "form": "batched = one cooperative launch of the persistent bin kernel per bin for every job; "
                    "batched_graph = one graph launch per bin iteration, a branch per job"}


def run_ours(args, rank, world, local):
    import torch
    eagb = load_eagb()
    dev = local
    torch.cuda.set_device(dev)
    d = np.load(LUT)
    betas, cum = d["betas"], d["cum"]
    NB = len(betas)
    V = L * L * LZ
    job = eagb.new_job(L, LZ, betas, cum, nsamples=NS, NR=NR, bc=eagb.EA_OBC, masters=MASTERS, device=dev, jobid=rank)
    if args.rng_sms >= 0:
        job.set_rng_sms(args.rng_sms)
    stream = torch.cuda.ExternalStream(job.stream(), device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)   # 512 MB > L2
    su_step = HOUFR * V * NR * NB * NS

    def step():
        # one `it` of the reference cadence: houfr x (sweep, energy, PT), the
        # Houdayer move, then the energy measurement and temperature-history
        # record; enqueued without a host synchronisation
        job.run_cycles(itmax=1, houfr=HOUFR, mesfr=1, ptfr=1)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    job.sync()
    # timed region: device events on the job's stream around all K steps,
    # joined with the generator stream at the end so that every uniform drawn
    # inside the region is counted; the L2 flushes between steps are timed
    # by their own events and taken out
    t_beg, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fl = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    eagb._ck(eagb.lib().ea_profile(job.ctx, 1))
    with Clocks(dev) as clk, torch.cuda.stream(stream):
        for i in range(args.steps):
            fl[i][0].record(stream)
            flush.fill_(i)
            fl[i][1].record(stream)
            if i == 0:
                t_beg.record(stream)
            step()
        job.join()
        t_end.record(stream)
        job.sync()
    torch.cuda.synchronize(dev)
    job.check_exact()
    barrier()
    ms = t_beg.elapsed_time(t_end) - sum(a.elapsed_time(b) for a, b in fl[1:])
    nsw, sw_ms = C.c_int64(), C.c_double()
    eagb._ck(eagb.lib().ea_kernel_time(job.ctx, 0, C.byref(nsw), C.byref(sw_ms)))
    npt, pt_ms = C.c_int64(), C.c_double()
    eagb._ck(eagb.lib().ea_kernel_time(job.ctx, 1, C.byref(npt), C.byref(pt_ms)))
    ncl, cl_ms = C.c_int64(), C.c_double()
    eagb._ck(eagb.lib().ea_kernel_time(job.ctx, 2, C.byref(ncl), C.byref(cl_ms)))
    nrg, rg_ms = C.c_int64(), C.c_double()
    eagb._ck(eagb.lib().ea_kernel_time(job.ctx, 4, C.byref(nrg), C.byref(rg_ms)))
    eagb._ck(eagb.lib().ea_profile(job.ctx, 0))

    # end to end through the C ABI with host buffers: every step uploads the
    # spin state from pinned memory and reads the energies back
    half = (L // 4) ** 2 * (LZ // 4) // 2
    nw = NB * half * NR
    # the whole spin state in one pinned buffer, [sample][even, odd][word]
    pinned = torch.zeros(NS * 2 * nw, dtype=torch.int64).pin_memory()
    pv = pinned.numpy().reshape(NS, 2, nw)
    for s in range(NS):
        ev_, od_ = job.get_spins(s)
        pv[s, 0] = ev_.view(np.int64)
        pv[s, 1] = od_.view(np.int64)
    E_out = np.zeros((NS, NR, NB), np.int32)
    lib, src = eagb.lib(), C.c_void_p(pinned.data_ptr())

    def run_e2e(pipelined):
        # every step: the whole spin state from pinned memory, the step, the
        # energies read back (a host synchronisation).  Serial: one copy on
        # the job's stream ahead of the step's kernels.  Pipelined: the next
        # step's state is staged (host copy on the context's copy stream)
        # while this step runs, and moved into the spins (a device copy) once
        # this step's energies are read
        per = []
        barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        if pipelined:
            eagb._ck(lib.ea_stage_spins_async(job.ctx, src))
        for i in range(ne):
            ts = time.perf_counter()
            if pipelined:
                eagb._ck(lib.ea_commit_staged_spins(job.ctx))
            else:
                eagb._ck(lib.ea_upload_spins_async(job.ctx, src))
            step()
            if pipelined and i + 1 < ne:
                eagb._ck(lib.ea_stage_spins_async(job.ctx, src))
            eagb._ck(lib.ea_measure_energy(job.ctx, eagb.P(E_out)))
            per.append(time.perf_counter() - ts)
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        barrier()
        return el, per

    # untimed: first use of the pinned buffer and of the staging buffer
    eagb._ck(lib.ea_upload_spins_async(job.ctx, src))
    step()
    eagb._ck(lib.ea_measure_energy(job.ctx, eagb.P(E_out)))
    ne = max(2, args.steps)
    e2e_serial_s, _ = run_e2e(False)
    e2e_s, e2e_steps = run_e2e(True)

    ms, e2e_s, e2e_serial_s = max_over_ranks(torch, [ms, e2e_s, e2e_serial_s], dev, world)
    if rank != 0:
        job.close()
        return
    value = world * su_step * args.steps / (ms * 1e-3) / 1e12
    e2e = world * su_step * ne / e2e_s / 1e12
    e2e_serial = world * su_step * ne / e2e_serial_s / 1e12
    hbm, how = peaks()
    ipk_alu, ipk_imad = int_peak(eagb, dev)
    # k_sweep (one half-sweep launch): algorithmic bytes = read + write every
    # word of the updated parity, read every word of the other parity once,
    # read the couplings; algorithmic integer ops = the random triples of the
    # launch (one per temperature, half-site and replica, shared by the 31
    # samples) and the word updates
    words_parity = NS * NB * half * NR
    alg_bytes = words_parity * 8 * 3 + NS * 6 * half * 8
    sweep_ms = sw_ms.value / max(1, nsw.value)
    achieved = alg_bytes / (sweep_ms * 1e-3) / 1e9
    ops, e_iters = int_ops(cum, NB * half * NR, words_parity)
    int_achieved = ops / (sweep_ms * 1e-3)
    hbm_frac, int_frac = achieved / hbm, int_achieved / ipk_alu
    # the cluster labelling group of a move (overlap words, slab labelling,
    # face merge, compression, selection + flip), per lattice site of the
    # nclust = 16 colder temperatures, 31 samples and 2 replica groups:
    # 3/8 B of overlap bits (two replicas read, one word written), 4 B label
    # written, 4 B label read at the flip, 8 B uniform of the site's cluster
    # (counted for every site: the generator draws one per site), and the two
    # replicas' spin bits read and written (1/2 B)
    nclust = 16
    cl_sites = V * nclust * NS * 2
    cl_bytes_site = 3.0 / 8 + 4 + 4 + 8 + 0.5
    cl_move_ms = cl_ms.value / max(1, args.steps)
    cl_achieved = cl_sites * cl_bytes_site / (cl_move_ms * 1e-3) / 1e9
    roof = {"bound": "int32" if int_frac > hbm_frac else "hbm",
            "achieved": int_achieved / 1e9 if int_frac > hbm_frac else achieved,
            "peak": ipk_alu / 1e9 if int_frac > hbm_frac else hbm,
            "unit": "Gop/s" if int_frac > hbm_frac else "GB/s",
            "frac": max(hbm_frac, int_frac), "traffic": KSWEEP_DRAM_BYTES,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per k_sweep launch of this workload",
            "kernel": "k_sweep", "peak_kind": how, "launch_ms": sweep_ms, "launches": nsw.value,
            "hbm_frac": hbm_frac, "hbm_achieved_gbs": achieved, "hbm_peak_gbs": hbm, "alg_bytes_per_launch": alg_bytes,
            "int_frac": int_frac, "int_achieved_gops": int_achieved / 1e9, "int_peak_gops": ipk_alu / 1e9,
            "int_peak_source": "measured at the start of this run: independent 32-bit xor/add instruction chains "
                               "on all SMs (ea_probe_int32_rate); multiply-add chains ran at %.0f Gop/s"
                               % (ipk_imad / 1e9),
            "int_ops_per_launch": ops, "int_ops_per_spin_update": ops / (64.0 * words_parity),
            "search_iterations_per_byte": e_iters,
            "cluster": {"kernels": "k_overlap, k_cc_slab, k_cc_merge, k_cc_compress, k_flip (one move, 2 groups)",
                        "bound": "hbm", "alg_bytes_per_site": cl_bytes_site, "sites_per_move": cl_sites,
                        "move_ms": cl_move_ms, "achieved": cl_achieved, "peak": hbm, "unit": "GB/s",
                        "frac": cl_achieved / hbm, "site_labellings_per_ns": cl_sites / (cl_move_ms * 1e6),
                        "note": "labelling is bound by instruction issue and SMEM latency, not DRAM"}}
    line = {
        "metric": "spin_updates_per_ps", "value": value, "unit": "spin-updates/ps", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded couplings and spins as the reference generates them)",
        "config": headline_config(),
        "form": "plain (one job per launch)", "parallelism": "replicas" if world > 1 else "single",
        "rng_sms": job.rng_sms(),
        "e2e": {"value": e2e, "unit": "spin-updates/ps", "h2d_bytes_per_step": NS * 2 * nw * 8,
                "d2h_bytes_per_step": NS * NR * NB * 4, "steps": ne,
                "step_ms": {"min": 1e3 * min(e2e_steps), "median": 1e3 * statistics.median(e2e_steps),
                            "max": 1e3 * max(e2e_steps)},
                "form": "pipelined: each step's whole spin state is copied from pinned memory into a device "
                        "staging buffer while the previous step runs (ea_stage_spins_async) and moved into the "
                        "spins after that step's energies are read (ea_commit_staged_spins)",
                "serial_value": e2e_serial,
                "serial_form": "the copy on the job's stream ahead of the step's kernels (ea_upload_spins_async)"},
        "gpu_launches": args.steps * (HOUFR * 6 + 1 + 2 * 4 + 3),
        "roofline": roof,
        "kernel_ms": {"sweep": sw_ms.value, "pt": pt_ms.value, "cluster": cl_ms.value,
                      "uniforms_overlapped": rg_ms.value, "step_total": ms},
        "clocks": clk.summary(),
    }
    line["no_cluster"] = run_no_cluster(args, dev, torch, eagb)
    if not args.no_mixed:
        line["batched"] = [run_mixed(args, dev, torch, eagb, 4, 8), run_mixed(args, dev, torch, eagb, 32, 1),
                           run_mixed_sp(args, dev, torch, eagb), run_mixed_sp(args, dev, torch, eagb, 72, 10),
                           run_small_sp(args, dev, torch, eagb)]
    if not args.no_serve:
        line["serving"] = run_serve(args, dev, eagb)
        line["serving_sample_packed"] = run_serve_sp(args, dev, eagb)
    if not args.no_sp:
        line["sample_packed"] = run_sp(args, dev, torch, eagb)
    if not args.no_cpu:
        su, dt = cpu_cycle(2)
        line["cpu_baseline"] = {"value": su / dt / 1e12, "unit": "spin-updates/ps", "cores": os.cpu_count(),
                                "kind": "port", "sample": CPU_SAMPLE + "; 2 steps"}
    print(json.dumps(line), flush=True)
    job.close()


def main():
    # more hardware queues, so that the plain form's per-job streams and the
    # per-job cluster-uniform generators can run side by side
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the batched vs plain mixed-geometry leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving (Poisson stream) leg")
    ap.add_argument("--no-sp", action="store_true", help="skip the sample-packed legs")
    ap.add_argument("--mix-only", default="", choices=["", "plain", "batched"],
                    help="only two bins of the 36-job x 32-sample multispin mix in this form (for profilers)")
    ap.add_argument("--rng-sms", type=int, default=-1,
                    help="SMs of the cluster-uniform generator's partition for the headline job (-1: automatic)")
    ap.add_argument("--small-sp", type=int, default=0, metavar="N",
                    help="only the small sample-packed batching leg with N jobs (prints its record)")
    ap.add_argument("--serve-config5", type=int, default=0, metavar="N",
                    help="only the serving configuration at its stated size: N jobs drawn from it (prints its record)")
    ap.add_argument("--sp-case", default="", help="run only the sample-packed workloads whose name contains this "
                    "(--steps bins after --warmup; prints their JSON records)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.mix_only:
        eagb = load_eagb()
        jobs = mixed_jobs(eagb, local, 32, 1)
        cad = dict(itmax=1, houfr=MIX_HOUFR, mesfr=1, ptfr=1)
        if args.mix_only == "batched":
            batch = eagb.Batch(jobs)
            for _ in range(2):
                batch.run_bin(**cad)
            batch.sync()
            batch.close()
        else:
            for _ in range(2):
                for j in jobs:
                    j.run_cycles(**cad)
            for j in jobs:
                j.sync()
        for j in jobs:
            j.close()
    elif args.small_sp:
        import torch
        print(json.dumps(run_small_sp(args, local, torch, load_eagb(), args.small_sp)), flush=True)
    elif args.serve_config5:
        print(json.dumps(run_serve_c5(args, local, load_eagb(), args.serve_config5)), flush=True)
    elif args.sp_case:
        import torch
        print(json.dumps(run_sp(args, local, torch, load_eagb())), flush=True)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
