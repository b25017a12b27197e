"""Pin the CPU oracle against fixtures produced by the reference's own host code
(tests/golden/make_host_golden.py).  CPU only."""
import glob
import hashlib
import os

import numpy as np
import pytest

import oracle_py as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
HOST = sorted(glob.glob(os.path.join(GOLD, "host_*.npz")))
LUTS = sorted(glob.glob(os.path.join(GOLD, "lut_*.npz")))


def check(d, name, got):
    raw = np.ascontiguousarray(got).tobytes()
    if name in d:
        ref = d[name].tobytes()
        assert raw == ref, name
    else:
        assert hashlib.sha256(raw).digest() == d["sha256:" + name].tobytes(), name


@pytest.fixture(scope="module", params=HOST, ids=[os.path.basename(p)[5:-4] for p in HOST])
def fx(request):
    d = dict(np.load(request.param))
    L, Lz, NB, NR, nbits, bc = (int(x) for x in d["geom"])
    g = O.geom(L, Lz, NB, NR, nbits, bc)
    return d, g


def test_seeds_and_generators(fx):
    d, g = fx
    sd, prc, xo, keys, pt, rc = O.init_run(g, [int(x) for x in d["masters"]])
    assert list(sd.seeds_J[:g.nbits]) == list(d["seeds_J"])
    assert list(sd.seeds_u[:g.nbits]) == list(d["seeds_u"])
    assert list(sd.seeds_MC[:g.NR]) == list(d["seeds_MC"])
    assert np.array_equal(keys, d["keys"])
    check(d, "prc", np.frombuffer(O.as_bytes(prc), np.uint8))
    check(d, "xo", np.frombuffer(O.as_bytes(xo), np.uint8))
    check(d, "rc", np.frombuffer(O.as_bytes(rc), np.uint8))
    for s in range(g.nbits):
        check(d, "pt%d" % s, np.frombuffer(O.as_bytes(pt)[s * g.NR * 2080:(s + 1) * g.NR * 2080], np.uint8))


def test_tables(fx):
    d, g = fx
    neig, rot, bi, ne = O.tables(g)
    check(d, "neig", neig)
    check(d, "rot_even", rot[:g.half])
    check(d, "rot_odd", rot[g.half:])
    check(d, "bianchi", bi)
    check(d, "neri", ne)


def test_spins_couplings_energy(fx):
    d, g = fx
    sd, *_ = O.init_run(g, [int(x) for x in d["masters"]])
    for s in range(g.nbits):
        uu = O.init_spins(g, sd.seeds_u[s])
        ev, od = O.pack_spins(g, uu)
        check(d, "even%d" % s, ev)
        check(d, "odd%d" % s, od)
        assert np.array_equal(O.unpack_spins(g, ev, od), uu)
        J6, _ = O.init_couplings(g, sd.seeds_J[s])
        check(d, "J6_%d" % s, J6)
        Jw = O.pack_couplings(g, J6)
        check(d, "Jw%d" % s, Jw)
        # scalar energy (med.c) of every (replica, clone), and the multispin energy of d_computeEne
        es = np.array([O.lib().or_scalar_energy(O.C.byref(g), O.ptr(np.ascontiguousarray(uu[(r * g.NB + c) * g.V:(r * g.NB + c + 1) * g.V])), O.ptr(J6))
                       for r in range(g.NR) for c in range(g.NB)], np.int32)
        check(d, "escalar%d" % s, es)
        g1 = O.geom(g.L, g.Lz, g.NB, g.NR, 1, g.bc)
        E = np.zeros((1, g.NR, g.NB), np.int32)
        sp = np.stack([ev, od])[None]
        O.lib().or_energy(O.C.byref(g1), O.ptr(np.ascontiguousarray(sp)), O.ptr(Jw), O.ptr(E))
        assert np.array_equal(E.reshape(-1), es)


def test_fill_bits_counters(fx):
    d, g = fx
    sd, prc, xo, keys, pt, rc = O.init_run(g, [int(x) for x in d["masters"]])
    ctrs = []
    for h in range(6):
        ctrs.append(O.fill_bits(prc, xo, g.NR, 1000 + h, 37))
    check(d, "ctr_iter1000_job37", np.concatenate(ctrs))


def test_parallel_tempering(fx):
    d, g = fx
    sd, prc, xo, keys, pt, rc = O.init_run(g, [int(x) for x in d["masters"]])
    NB, NR = g.NB, g.NR
    en = d["pt_energies"].reshape(g.nbits, NR, 5, NB)
    perm = d["pt_perm"].reshape(g.nbits, NR, 5, NB)
    acc = np.zeros((g.nbits, NR, NB - 1))
    att = np.zeros_like(acc)
    accraw = np.zeros_like(acc)
    betas = np.ascontiguousarray(d["betas"], np.float64)
    for s in range(g.nbits):
        for r in range(NR):
            wctb = np.arange(NB, dtype=np.uint8)
            wbtc = wctb.copy()
            for k in range(5):
                E = np.ascontiguousarray(en[s, r, k])
                O.lib().or_parallel_tempering(O.C.byref(pt[s * NR + r]), O.ptr(wctb), O.ptr(wbtc), O.ptr(E),
                                             O.ptr(betas), NB, O.ptr(acc[s, r]), O.ptr(att[s, r]), O.ptr(accraw[s, r]))
                assert np.array_equal(wctb, perm[s, r, k])
                assert np.array_equal(np.argsort(wctb), wbtc)
    check(d, "pt_acc", acc)
    check(d, "pt_accraw", accraw)
    check(d, "pt_state_after", np.frombuffer(O.as_bytes(pt), np.uint8))


@pytest.mark.parametrize("path", LUTS, ids=[os.path.basename(p)[4:-4] for p in LUTS])
def test_lut_thresholds(path):
    d = np.load(path)
    if "matches_shipped_file" in d:
        assert int(d["matches_shipped_file"][0]) == 1
    for i, b in enumerate(d["betas"]):
        cum, umb, pre = O.lut_beta(float(b))
        assert np.array_equal(cum, d["cum"][i]), i
        if i == 0:
            assert np.array_equal(pre, d["prebusqueda0"])


def test_lut_search_is_first_threshold_above():
    d = np.load(os.path.join(GOLD, "lut_T06_16_N32.npz"))
    rng = np.random.default_rng(5)
    for i in (0, 15, 31):
        cum = np.ascontiguousarray(d["cum"][i])
        for R in list(rng.integers(0, 2**63, 200, dtype=np.uint64) * np.uint64(2)) + list(cum[:3]) + [cum[253], cum[254], np.uint64(2**64 - 1)]:
            n = O.lib().or_lut_search(O.C.c_uint64(int(R)), O.ptr(cum))
            want = int(np.searchsorted(cum, R, side="right"))
            assert n == min(want, 255)
