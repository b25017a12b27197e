"""ctypes binding of libeagb.so (include/eagb.h) for tests, bench and scripts.

The library is the product; this module only marshals numpy arrays through
the C ABI.  It refuses to run without the compiled library: there is no
Python or CPU implementation of the hot path behind it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeagb.so")

EA_PBC, EA_OBC, EA_OBC_WEAK, EA_OBC_STRONG = 0, 1, 2, 3
BC = {"PBC": EA_PBC, "OBC": EA_OBC, "WEAK": EA_OBC_WEAK, "STRONG": EA_OBC_STRONG}


class Geom(C.Structure):
    _fields_ = [("L", C.c_int32), ("Lz", C.c_int32), ("nbetas", C.c_int32), ("nrep", C.c_int32),
                ("nsamples", C.c_int32), ("bc", C.c_int32)]


class HQ(C.Structure):
    _fields_ = [("ira", C.c_uint64 * 256), ("PR", C.c_uint64), ("zseed", C.c_uint64), ("final", C.c_uint64),
                ("ip", C.c_uint8), ("ip1", C.c_uint8), ("ip2", C.c_uint8), ("ip3", C.c_uint8),
                ("padding", C.c_uint8 * 4)]


class Xoshiro(C.Structure):
    _fields_ = [("s", C.c_uint64 * 4), ("t", C.c_uint64), ("final", C.c_uint64)]


class Generators(C.Structure):
    _fields_ = [("prc", HQ * 64), ("xo", Xoshiro * 64), ("keys", C.c_uint32 * 64), ("rc", HQ),
                ("cuda_rng_offset", C.c_uint64), ("seed_cluster", C.c_uint64)]


class Cadence(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("itmax", "houfr", "mesfr", "ptfr", "cluster", "nclust")]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_jobs", C.c_int32), ("depth", C.c_int32), ("tile", C.c_int32),
                ("nb_max", C.c_int32), ("reserved", C.c_int32), ("hbm_budget", C.c_uint64)]


EA_LAYOUT_MULTISPIN, EA_LAYOUT_SAMPLE_PACKED = 0, 1
EA_BIN_AUTO, EA_BIN_GRAPH, EA_BIN_PERSISTENT, EA_BIN_RESIDENT = 0, 1, 2, 3


class Request(C.Structure):
    _fields_ = [("geom", Geom), ("betas", C.c_void_p), ("cum", C.c_void_p), ("masters", C.c_uint64 * 4),
                ("cad", Cadence), ("nbins", C.c_int32), ("jobid", C.c_uint32), ("iter0", C.c_int64),
                ("layout", C.c_int32), ("nwords", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("bins_done", C.c_int32), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("bytes", C.c_uint64), ("spin_updates", C.c_double),
                ("t_ready", C.c_double), ("t_start", C.c_double), ("gpu_s", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "admitted", "completed", "failed", "queued", "running",
                                          "bins", "batch_changes", "peak_running")] + \
               [(n, C.c_double) for n in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "spin_updates", "span_s")] + \
               [(n, C.c_uint64) for n in ("budget", "bytes_in_use", "bytes_peak")] + \
               [(n, C.c_double) for n in ("gpu_busy_s", "enqueue_s", "admit_s", "queue_p50_ms", "queue_p99_ms",
                                          "prep_p50_ms", "prep_p99_ms", "start_p50_ms", "start_p99_ms",
                                          "run_p50_ms", "run_p99_ms", "gpu_p50_ms", "gpu_p99_ms")]


EA_JOB_QUEUED, EA_JOB_RUNNING, EA_JOB_DONE, EA_JOB_FAILED, EA_JOB_RELEASED = range(5)

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libeagb.so is not built (run python ea-lcd-mc_gb300/build.py)")
        _lib = C.CDLL(LIB_PATH)
        _lib.ea_last_error.restype = C.c_char_p
    return _lib


class EAError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ea error %d: %s" % (code, msg))
        self.code = code


def _ck(rc):
    if rc != 0:
        raise EAError(rc, lib().ea_last_error().decode())


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def geom(L, Lz, NB, NR=8, nsamples=1, bc=EA_OBC):
    return Geom(L, Lz, NB, NR, nsamples, bc)


def sizes(g):
    half = (g.L // 4) * (g.L // 4) * (g.Lz // 4) // 2
    return half, g.L * g.L * g.Lz


def host_seeds(masters, nsamples, nrep=8, list_samples=None):
    sJ = np.zeros(nsamples, np.uint64)
    su = np.zeros(nsamples, np.uint64)
    sMC = np.zeros(nrep, np.uint64)
    ls = None if list_samples is None else np.ascontiguousarray(list_samples, np.int32)
    _ck(lib().ea_host_seeds(C.c_uint64(masters[0]), C.c_uint64(masters[1]), C.c_uint64(masters[2]),
                            C.c_uint64(masters[3]), None if ls is None else P(ls), nsamples, nrep, P(sJ), P(su),
                            P(sMC)))
    return sJ, su, sMC


def host_generators(seeds_MC, nsamples, seed_cluster, list_samples=None):
    nrep = len(seeds_MC)
    gen = Generators()
    pt = (HQ * (nsamples * nrep))()
    sMC = np.ascontiguousarray(seeds_MC, np.uint64)
    ls = None if list_samples is None else np.ascontiguousarray(list_samples, np.int32)
    _ck(lib().ea_host_generators(P(sMC), None if ls is None else P(ls), nsamples, nrep, C.c_uint64(seed_cluster),
                                 C.byref(gen), pt))
    return gen, pt


def host_init_spins(g, seed_u):
    half, V = sizes(g)
    n = g.nbetas * half * g.nrep
    ev = np.zeros(n, np.uint64)
    od = np.zeros(n, np.uint64)
    _ck(lib().ea_host_init_spins(C.byref(g), C.c_uint64(seed_u), P(ev), P(od)))
    return ev, od


def host_unpack_replica(g, even, odd, rep):
    """ea_host_unpack_replica: the spins of every clone of one replica as
    bytes [NB][V] (0/1), site x + L*y + L*L*z."""
    half, V = sizes(g)
    u = np.zeros((g.nbetas, V), np.uint8)
    _ck(lib().ea_host_unpack_replica(C.byref(g), P(np.ascontiguousarray(even, np.uint64)),
                                     P(np.ascontiguousarray(odd, np.uint64)), int(rep), P(u)))
    return u


def host_pack_replica(g, u, rep, even, odd):
    """ea_host_pack_replica: bytes [NB][V] into replica `rep` of the even/odd arrays."""
    _ck(lib().ea_host_pack_replica(C.byref(g), P(np.ascontiguousarray(u, np.uint8)), int(rep), P(even), P(odd)))


def host_init_couplings(g, seed_J):
    half, V = sizes(g)
    J6 = np.zeros(6 * V, np.uint8)
    Jw = np.zeros(12 * half, np.uint64)
    cnt = C.c_int32(0)
    _ck(lib().ea_host_init_couplings(C.byref(g), C.c_uint64(seed_J), P(J6), P(Jw), C.byref(cnt)))
    return J6, Jw, cnt.value


class Job:
    """One simulation job on one GPU (an ea_ctx)."""

    def __init__(self, g, device=0):
        self.g = g
        self.half, self.V = sizes(g)
        self.ctx = C.c_void_p()
        _ck(lib().ea_create(C.byref(g), device, C.byref(self.ctx)))

    def close(self):
        if self.ctx:
            lib().ea_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # inputs / outputs
    def set_temperatures(self, betas, cum):
        b = np.ascontiguousarray(betas, np.float64)
        c = np.ascontiguousarray(cum, np.uint64)
        _ck(lib().ea_set_temperatures(self.ctx, P(b), P(c)))

    def set_spins(self, s, even, odd):
        _ck(lib().ea_set_spins(self.ctx, s, P(np.ascontiguousarray(even, np.uint64)),
                               P(np.ascontiguousarray(odd, np.uint64))))

    def get_spins(self, s):
        n = self.g.nbetas * self.half * self.g.nrep
        ev = np.zeros(n, np.uint64)
        od = np.zeros(n, np.uint64)
        _ck(lib().ea_get_spins(self.ctx, s, P(ev), P(od)))
        return ev, od

    def set_couplings(self, s, Jw):
        _ck(lib().ea_set_couplings(self.ctx, s, P(np.ascontiguousarray(Jw, np.uint64))))

    def set_generators(self, gen, pt):
        _ck(lib().ea_set_generators(self.ctx, C.byref(gen), pt))

    def get_generators(self):
        gen = Generators()
        pt = (HQ * (self.g.nsamples * self.g.nrep))()
        _ck(lib().ea_get_generators(self.ctx, C.byref(gen), pt))
        return gen, pt

    def set_permutations(self, wctb=None):
        if wctb is None:
            _ck(lib().ea_set_permutations(self.ctx, None))
        else:
            _ck(lib().ea_set_permutations(self.ctx, P(np.ascontiguousarray(wctb, np.uint8))))

    def get_permutations(self):
        shape = (self.g.nsamples, self.g.nrep, self.g.nbetas)
        a = np.zeros(shape, np.uint8)
        b = np.zeros(shape, np.uint8)
        _ck(lib().ea_get_permutations(self.ctx, P(a), P(b)))
        return a, b

    def get_pt_stats(self):
        shape = (self.g.nsamples, self.g.nrep, self.g.nbetas - 1)
        acc, att, raw = (np.zeros(shape) for _ in range(3))
        _ck(lib().ea_get_pt_stats(self.ctx, P(acc), P(att), P(raw)))
        return acc, att, raw

    def set_counter(self, it, jobid=0):
        _ck(lib().ea_set_counter(self.ctx, C.c_int64(it), C.c_uint32(jobid)))

    def get_counter(self):
        v = C.c_int64(0)
        _ck(lib().ea_get_counter(self.ctx, C.byref(v)))
        return v.value

    # hot path
    def monte_carlo(self, n):
        _ck(lib().ea_monte_carlo(self.ctx, n))

    def measure_energy(self):
        E = np.zeros((self.g.nsamples, self.g.nrep, self.g.nbetas), np.int32)
        _ck(lib().ea_measure_energy(self.ctx, P(E)))
        return E

    def parallel_tempering(self):
        _ck(lib().ea_parallel_tempering(self.ctx))

    def houdayer(self, nclust=0):
        _ck(lib().ea_houdayer(self.ctx, nclust))

    def run_bin(self, itmax, houfr, mesfr, ptfr, cluster=True, nclust=0):
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        avg = np.zeros((self.g.nsamples, self.g.nrep, self.g.nbetas))
        hist = np.zeros(self.g.nsamples * self.g.nrep * 512 * self.g.nbetas, np.uint8)
        mx = C.c_int32(0)
        _ck(lib().ea_run_bin(self.ctx, C.byref(cad), P(avg), P(hist), C.byref(mx)))
        m = mx.value
        return avg, hist[:self.g.nsamples * self.g.nrep * m * self.g.nbetas].reshape(
            self.g.nsamples, self.g.nrep, m, self.g.nbetas)

    def run_cycles(self, itmax, houfr, mesfr, ptfr, cluster=True, nclust=0):
        """Enqueue one bin without copying anything back (asynchronous)."""
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_run_bin(self.ctx, C.byref(cad), None, None, None))

    def bin_results(self):
        """Energy averages and temperature history of the last bin (plain or batched)."""
        avg = np.zeros((self.g.nsamples, self.g.nrep, self.g.nbetas))
        hist = np.zeros(self.g.nsamples * self.g.nrep * 512 * self.g.nbetas, np.uint8)
        mx = C.c_int32(0)
        _ck(lib().ea_bin_results(self.ctx, P(avg), P(hist), C.byref(mx)))
        m = mx.value
        return avg, hist[:self.g.nsamples * self.g.nrep * m * self.g.nbetas].reshape(
            self.g.nsamples, self.g.nrep, m, self.g.nbetas)

    def check_exact(self):
        _ck(lib().ea_check_exact(self.ctx))

    def sync(self):
        _ck(lib().ea_sync(self.ctx))

    def join(self):
        _ck(lib().ea_join(self.ctx))

    def set_rng_sms(self, nsm):
        """SM split between the cluster-uniform generator and the job (0: none,
        negative: automatic); before the first cluster move only."""
        _ck(lib().ea_set_rng_sms(self.ctx, int(nsm)))

    def rng_sms(self):
        v = C.c_int32()
        _ck(lib().ea_get_rng_sms(self.ctx, C.byref(v)))
        return v.value

    def stream(self):
        v = C.c_void_p()
        _ck(lib().ea_get_stream(self.ctx, C.byref(v)))
        return v.value


def curand_uniforms(seed, offset, n, device=0):
    out = np.zeros(n, np.float64)
    _ck(lib().ea_curand_uniforms(device, C.c_uint64(seed), C.c_uint64(offset), C.c_uint64(n), P(out)))
    return out


class Batch:
    """Many jobs advanced together by the persistent batched kernels."""

    def __init__(self, jobs, tile=0):
        self.jobs = list(jobs)
        arr = (C.c_void_p * len(self.jobs))(*[j.ctx.value if isinstance(j.ctx, C.c_void_p) else j.ctx
                                              for j in self.jobs])
        self.b = C.c_void_p()
        _ck(lib().ea_batch_create(arr, len(self.jobs), int(tile), C.byref(self.b)))

    def tile(self):
        v = C.c_int32()
        _ck(lib().ea_batch_tile(self.b, C.byref(v)))
        return v.value

    def run_bin(self, itmax, houfr, mesfr, ptfr, cluster=True, nclust=0):
        """Enqueue one bin for every job (asynchronous)."""
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_batch_run_bin(self.b, C.byref(cad)))

    def sync(self):
        _ck(lib().ea_batch_sync(self.b))

    def stream(self):
        v = C.c_void_p()
        _ck(lib().ea_batch_stream(self.b, C.byref(v)))
        return v.value

    def close(self):
        if self.b:
            _ck(lib().ea_batch_destroy(self.b))
            self.b = None


def new_job(L, Lz, betas, cum, nsamples=1, NR=8, bc=EA_OBC, masters=(1, 2, 3, 4), list_samples=None,
            device=0, iter0=0, jobid=0):
    """A job initialised exactly as the reference initialises a new run (flag 1)."""
    g = geom(L, Lz, len(betas), NR, nsamples, bc)
    job = Job(g, device)
    job.set_temperatures(betas, cum)
    sJ, su, sMC = host_seeds(masters, nsamples, NR, list_samples)
    gen, pt = host_generators(sMC, nsamples, masters[3], list_samples)
    job.set_generators(gen, pt)
    for s in range(nsamples):
        ev, od = host_init_spins(g, int(su[s]))
        job.set_spins(s, ev, od)
        J6, Jw, _ = host_init_couplings(g, int(sJ[s]))
        job.set_couplings(s, Jw)
    job.set_permutations(None)
    job.set_counter(iter0, jobid)
    return job


def job_bytes(g, cad=None, betas=None):
    """Device bytes a job holds (ea_job_bytes): what admission charges."""
    out = C.c_uint64()
    b = None if betas is None else np.ascontiguousarray(betas, np.float64)
    _ck(lib().ea_job_bytes(C.byref(g), None if cad is None else C.byref(cad), None if b is None else P(b),
                           C.byref(out)))
    return out.value


def init_run(job, masters, iter0=0, jobid=0, list_samples=None):
    """ea_init_run: a new run on an existing job, set up in the library."""
    m = (C.c_uint64 * 4)(*[int(x) for x in masters])
    ls = None if list_samples is None else np.ascontiguousarray(list_samples, np.int32)
    _ck(lib().ea_init_run(job.ctx, m, None if ls is None else P(ls), C.c_int64(iter0), C.c_uint32(jobid)))


class ServedJob(Job):
    """View of a finished server job (the context stays owned by the server)."""

    def __init__(self, g, ctx):
        self.g = g
        self.half, self.V = sizes(g)
        self.ctx = ctx

    def close(self):
        self.ctx = None

    def __del__(self):
        pass


class Server:
    """Continuous batching server (ea_server_*): submit jobs at any time, wait
    for each, read its results, release it."""

    def __init__(self, device=0, max_jobs=0, depth=0, tile=0, nb_max=0, hbm_budget=0):
        cfg = ServerConfig(device, max_jobs, depth, tile, nb_max, 0, hbm_budget)
        self.s = C.c_void_p()
        _ck(lib().ea_server_create(C.byref(cfg), C.byref(self.s)))
        self._geoms = {}
        self._sp_geom = {}

    def submit(self, L, Lz, betas, cum, nsamples, NR, bc, masters, nbins, itmax, houfr, mesfr, ptfr,
               cluster=True, nclust=0, jobid=0, iter0=0, layout=EA_LAYOUT_MULTISPIN, nwords=1):
        betas = np.ascontiguousarray(betas, np.float64)
        cum = np.ascontiguousarray(cum, np.uint64)
        g = geom(L, Lz, len(betas), NR, nsamples, bc)
        r = Request(g, betas.ctypes.data, cum.ctypes.data, (C.c_uint64 * 4)(*[int(x) for x in masters]),
                    Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust), nbins, jobid, iter0, layout, nwords)
        t = C.c_int64()
        _ck(lib().ea_server_submit(self.s, C.byref(r), C.byref(t)))
        self._geoms[t.value] = g
        if layout == EA_LAYOUT_SAMPLE_PACKED:
            self._sp_geom[t.value] = (SpGeom(L, Lz, len(betas), NR, nwords, bc), betas)
        return t.value

    def sp_job(self, ticket):
        """View of a finished sample-packed job (owned by the server)."""
        h = C.c_void_p()
        _ck(lib().ea_server_sp_job(self.s, C.c_int64(ticket), C.byref(h)))
        g, betas = self._sp_geom[ticket]
        return SpView(g, betas, h)

    def wait(self, ticket, timeout=-1.0):
        ctx = C.c_void_p()
        _ck(lib().ea_server_wait(self.s, C.c_int64(ticket), C.c_double(timeout), C.byref(ctx)))
        return ServedJob(self._geoms[ticket], ctx)

    def info(self, ticket):
        i = JobInfo()
        _ck(lib().ea_server_info(self.s, C.c_int64(ticket), C.byref(i)))
        return {f: getattr(i, f) for f, _ in JobInfo._fields_}

    def release(self, ticket):
        _ck(lib().ea_server_release(self.s, C.c_int64(ticket)))

    def stats(self):
        st = ServeStats()
        _ck(lib().ea_server_stats(self.s, C.byref(st)))
        return {f: getattr(st, f) for f, _ in ServeStats._fields_}

    def drain(self):
        _ck(lib().ea_server_drain(self.s))

    def close(self):
        if self.s:
            _ck(lib().ea_server_destroy(self.s))
            self.s = None


# ---------------------------------------------------------------------------
# Sample-packed layout (ea_sp_*): 64 samples per word, any L >= 2, Lz >= 2
# ---------------------------------------------------------------------------
class SpGeom(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("L", "Lz", "nbetas", "nrep", "nwords", "bc")]


def sp_graph(L, Lz, bc):
    """Bond graph: nb [V,6], mate [V,6], colour [V], ncol."""
    V = L * L * Lz
    nb = np.zeros((V, 6), np.int32)
    mate = np.zeros((V, 6), np.int32)
    col = np.zeros(V, np.uint8)
    n = C.c_int32()
    _ck(lib().ea_sp_graph(L, Lz, bc, P(nb), P(mate), P(col), C.byref(n)))
    return nb, mate, col, n.value


def sp_job_bytes(g, cad=None, betas=None):
    """Device bytes of a sample-packed job (ea_sp_job_bytes)."""
    out = C.c_uint64()
    b = None if betas is None else np.ascontiguousarray(betas, np.float64)
    _ck(lib().ea_sp_job_bytes(C.byref(g), None if cad is None else C.byref(cad), None if b is None else P(b),
                              C.byref(out)))
    return out.value


def sp_host_init(g, seed_J, seed_u):
    V = g.L * g.L * g.Lz
    J = np.zeros((g.nwords, V, 6), np.uint64)
    S = np.zeros((g.nwords, V, g.nrep, g.nbetas), np.uint64)
    _ck(lib().ea_sp_host_init(C.byref(g), C.c_uint64(seed_J), C.c_uint64(seed_u), P(J), P(S)))
    return J, S


def sp_presearch11(cum):
    """ea_sp_presearch11: the per-item pass's 11-bit pre-search of one
    temperature's thresholds (2064 bytes)."""
    c = np.ascontiguousarray(cum, np.uint64)
    pre = np.zeros(2064, np.uint8)
    _ck(lib().ea_sp_presearch11(P(c), P(pre)))
    return pre


class SpJob:
    """A sample-packed job (ea_sp): 64 * nwords samples of an L x L x Lz tube."""

    def __init__(self, L, Lz, betas, cum, nrep=2, nwords=1, bc=EA_PBC, seeds=(1, 2, 3, 4), jobid=0, device=0):
        betas = np.ascontiguousarray(betas, np.float64)
        self.g = SpGeom(L, Lz, len(betas), nrep, nwords, bc)
        self.V = L * L * Lz
        self.betas = betas
        self.h = C.c_void_p()
        _ck(lib().ea_sp_create(C.byref(self.g), device, C.byref(self.h)))
        _ck(lib().ea_sp_set_temperatures(self.h, P(betas), P(np.ascontiguousarray(cum, np.uint64))))
        sd = (C.c_uint64 * 4)(*[int(x) for x in seeds])
        _ck(lib().ea_sp_init(self.h, sd, C.c_uint32(jobid)))

    def close(self):
        if self.h:
            _ck(lib().ea_sp_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        nc, kt = C.c_int32(), C.c_int32()
        _ck(lib().ea_sp_info(self.h, C.byref(nc), C.byref(kt)))
        return nc.value, kt.value

    def stream(self):
        v = C.c_void_p()
        _ck(lib().ea_sp_stream(self.h, C.byref(v)))
        return v.value

    def sync(self):
        _ck(lib().ea_sp_sync(self.h))

    def set_bin_kernel(self, mode):
        """EA_BIN_AUTO, EA_BIN_GRAPH, EA_BIN_PERSISTENT or EA_BIN_RESIDENT (ea_sp_set_bin_kernel)."""
        _ck(lib().ea_sp_set_bin_kernel(self.h, int(mode)))

    def plane_overlaps(self, nrep):
        """ea_sp_plane_overlaps: differing spins per (word, sample, pair, slot, plane)."""
        g = self.g
        out = np.zeros((g.nwords, 64, nrep // 2, g.nbetas, g.Lz), np.int32)
        _ck(lib().ea_sp_plane_overlaps(self.h, int(nrep), P(out)))
        return out

    def plane_correlations(self, nrep, dmax):
        """ea_sp_plane_correlations: [samples][slot][d][3][3] correlation matrices."""
        g = self.g
        out = np.zeros((g.nwords * 64, g.nbetas, dmax + 1, 3, 3))
        _ck(lib().ea_sp_plane_correlations(self.h, int(nrep), int(dmax), P(out)))
        return out

    def set_tile(self, tile):
        """ea_sp_set_tile: colour passes in tiles of `tile` sites, or 0 for the per-item pass."""
        _ck(lib().ea_sp_set_tile(self.h, int(tile)))

    def autotune(self):
        """ea_sp_autotune: (tile width -- 0 for the per-item pass --, energy sites
        per thread, labelling block size) chosen."""
        kt, ec, ct = C.c_int32(), C.c_int32(), C.c_int32()
        _ck(lib().ea_sp_autotune(self.h, C.byref(kt), C.byref(ec), C.byref(ct)))
        return kt.value, ec.value, ct.value

    def bin_kernel_for(self, itmax, houfr=1, mesfr=1, ptfr=1, cluster=False, nclust=0):
        """The form ea_sp_run takes for such a bin (ea_sp_bin_kernel_for)."""
        m = C.c_int32()
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_sp_bin_kernel_for(self.h, C.byref(cad), C.byref(m)))
        return m.value

    def get_spins(self):
        S = np.zeros((self.g.nwords, self.V, self.g.nrep, self.g.nbetas), np.uint64)
        _ck(lib().ea_sp_get_spins(self.h, P(S)))
        return S

    def set_spins(self, S):
        _ck(lib().ea_sp_set_spins(self.h, P(np.ascontiguousarray(S, np.uint64))))

    def get_generators(self):
        gen = Generators()
        _ck(lib().ea_sp_get_generators(self.h, C.byref(gen)))
        return gen

    def counter(self):
        it, ps = C.c_int64(), C.c_uint64()
        _ck(lib().ea_sp_get_counter(self.h, C.byref(it), C.byref(ps)))
        return it.value, ps.value

    def sweeps(self, n):
        _ck(lib().ea_sp_sweeps(self.h, n))

    def energy(self):
        U2 = np.zeros((self.g.nwords, 64, self.g.nrep, self.g.nbetas), np.int32)
        _ck(lib().ea_sp_energy(self.h, P(U2)))
        return U2

    def parallel_tempering(self):
        _ck(lib().ea_sp_parallel_tempering(self.h))

    def tempering(self):
        nw, NR, NB = self.g.nwords, self.g.nrep, self.g.nbetas
        E = np.zeros((nw, 64, NR, NB), np.int32)
        perm = np.zeros((nw, 64, NR, NB), np.uint8)
        acc = np.zeros((nw, 64, NR, NB - 1), np.uint32)
        M = np.zeros((nw, NR, NB - 1), np.uint64)
        _ck(lib().ea_sp_get_tempering(self.h, P(E), P(perm), P(acc), P(M)))
        return E, perm, acc, M

    def houdayer(self, nclust=0):
        _ck(lib().ea_sp_houdayer(self.h, nclust))

    def run_bin(self, itmax, houfr=1, mesfr=1, ptfr=1, cluster=False, nclust=0):
        """One bin of the cadence; returns the bin's average energy of every
        (word, sample, replica, slot)."""
        avg = np.zeros((self.g.nwords, 64, self.g.nrep, self.g.nbetas))
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_sp_run(self.h, C.byref(cad), P(avg)))
        return avg

    def run_async(self, itmax, houfr=1, mesfr=1, ptfr=1, cluster=False, nclust=0):
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_sp_run(self.h, C.byref(cad), None))

    def bin_results(self):
        avg = np.zeros((self.g.nwords, 64, self.g.nrep, self.g.nbetas))
        _ck(lib().ea_sp_bin_results(self.h, P(avg)))
        return avg

    def exact(self, betas=None):
        """Density of states [nwords*64, 6V+1] and <E>(beta) [nwords*64, NB] (V <= 32)."""
        b = np.ascontiguousarray(self.betas if betas is None else betas, np.float64)
        ns = self.g.nwords * 64
        dos = np.zeros((ns, 6 * self.V + 1), np.uint64)
        mean = np.zeros((ns, len(b)))
        _ck(lib().ea_sp_exact(self.h, P(b), len(b), P(dos), P(mean)))
        return dos, mean


class SpView(SpJob):
    """A sample-packed job owned by someone else (a server): no create/destroy."""

    def __init__(self, g, betas, handle):
        self.g = g
        self.V = g.L * g.L * g.Lz
        self.betas = betas
        self.h = handle

    def close(self):
        self.h = None


class SpBatch:
    """Sample-packed jobs advanced together by the batched kernels (ea_sp_batch)."""

    def __init__(self, jobs):
        self.jobs = list(jobs)
        arr = (C.c_void_p * len(self.jobs))(*[j.h.value if isinstance(j.h, C.c_void_p) else j.h for j in self.jobs])
        self.b = C.c_void_p()
        _ck(lib().ea_sp_batch_create(arr, len(self.jobs), C.byref(self.b)))

    def run_bin(self, itmax, houfr=1, mesfr=1, ptfr=1, cluster=False, nclust=0):
        cad = Cadence(itmax, houfr, mesfr, ptfr, int(cluster), nclust)
        _ck(lib().ea_sp_batch_run(self.b, C.byref(cad)))

    def set_bin_kernel(self, mode):
        _ck(lib().ea_sp_batch_set_bin_kernel(self.b, int(mode)))

    def sync(self):
        _ck(lib().ea_sp_batch_sync(self.b))

    def stream(self):
        v = C.c_void_p()
        _ck(lib().ea_sp_batch_stream(self.b, C.byref(v)))
        return v.value

    def close(self):
        if self.b:
            _ck(lib().ea_sp_batch_destroy(self.b))
            self.b = None
