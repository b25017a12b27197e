"""CPU tests of libeagb.so's host-side entry points: the job set-up must match
the reference (fixtures of tests/golden/) and the oracle.  No GPU calls."""
import ctypes as C
import glob
import hashlib
import os
import re

import numpy as np
import pytest

import oracle_py as O
from conftest import ROOT

import importlib.util

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)

GOLD = os.path.join(ROOT, "tests", "golden")
HOST = sorted(glob.glob(os.path.join(GOLD, "host_*.npz")))


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def check(d, name, got):
    raw = np.ascontiguousarray(got).tobytes()
    if name in d:
        assert raw == d[name].tobytes(), name
    else:
        assert hashlib.sha256(raw).digest() == d["sha256:" + name].tobytes(), name


def test_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "eagb.h")).read()
    names = sorted(set(re.findall(r"\b(?:int|const char \*)\s*(ea_\w+)\s*\(", hdr)))
    assert len(names) >= 25
    lib = C.CDLL(eagb.LIB_PATH)
    for n in names:
        assert hasattr(lib, n), n
    assert lib.ea_version() == 100


@pytest.mark.parametrize("path", HOST, ids=[os.path.basename(p)[5:-4] for p in HOST])
def test_setup_matches_reference(path):
    d = dict(np.load(path))
    L, Lz, NB, NR, nbits, bc = (int(x) for x in d["geom"])
    m = [int(x) for x in d["masters"]]
    sJ, su, sMC = eagb.host_seeds(m, nbits, NR)
    assert list(sJ) == list(d["seeds_J"]) and list(su) == list(d["seeds_u"]) and list(sMC) == list(d["seeds_MC"])
    gen, pt = eagb.host_generators(sMC, nbits, m[3])
    prc = bytes(memoryview(gen.prc).cast("B"))[:NR * 2080]
    xo = bytes(memoryview(gen.xo).cast("B"))[:NR * 48]
    check(d, "prc", np.frombuffer(prc, np.uint8))
    check(d, "xo", np.frombuffer(xo, np.uint8))
    check(d, "rc", np.frombuffer(bytes(memoryview(gen.rc).cast("B")), np.uint8))
    assert list(gen.keys[:NR]) == list(d["keys"])
    ptb = bytes(memoryview(pt).cast("B"))
    g = eagb.geom(L, Lz, NB, NR, nbits, bc)
    for s in range(nbits):
        check(d, "pt%d" % s, np.frombuffer(ptb[s * NR * 2080:(s + 1) * NR * 2080], np.uint8))
        ev, od = eagb.host_init_spins(g, int(su[s]))
        check(d, "even%d" % s, ev)
        check(d, "odd%d" % s, od)
        J6, Jw, cnt = eagb.host_init_couplings(g, int(sJ[s]))
        check(d, "J6_%d" % s, J6)
        check(d, "Jw%d" % s, Jw)
        if "escalar%d" % s in d:
            half, V = eagb.sizes(g)
            u = np.zeros(NB * V, np.uint8)
            eagb._ck(eagb.lib().ea_host_unpack_replica(C.byref(g), eagb.P(ev), eagb.P(od), 0, eagb.P(u)))
            E = C.c_int32()
            eagb._ck(eagb.lib().ea_host_scalar_energy(C.byref(g), eagb.P(u[:V].copy()), eagb.P(J6), C.byref(E)))
            assert E.value == d["escalar%d" % s][0]
            ev2 = np.zeros_like(ev)
            od2 = np.zeros_like(od)
            for r in range(NR):
                eagb._ck(eagb.lib().ea_host_unpack_replica(C.byref(g), eagb.P(ev), eagb.P(od), r, eagb.P(u)))
                eagb._ck(eagb.lib().ea_host_pack_replica(C.byref(g), eagb.P(u), r, eagb.P(ev2), eagb.P(od2)))
            assert np.array_equal(ev, ev2) and np.array_equal(od, od2)


def test_rejects_bad_geometry():
    for L, Lz, NB in ((6, 24, 4), (8, 12, 4), (8, 8, 1)):
        g = eagb.geom(L, Lz, NB)
        ev = np.zeros(1 << 12, np.uint64)
        rc = eagb.lib().ea_host_init_spins(C.byref(g), C.c_uint64(1), eagb.P(ev), eagb.P(ev))
        assert rc == -1
        assert b"geometry" in eagb.lib().ea_last_error()


def test_sample_list_and_seed_errors():
    with pytest.raises(eagb.EAError):
        eagb.host_seeds((0, 1, 2, 3), 2)
    with pytest.raises(eagb.EAError):
        eagb.host_seeds((1, 1, 2, 3), 2, list_samples=[3, 3])
    sJ, su, _ = eagb.host_seeds((5, 6, 7, 8), 2, list_samples=[4, 9])
    sJ_all, su_all, _ = eagb.host_seeds((5, 6, 7, 8), 32)
    assert sJ[0] == sJ_all[4] and sJ[1] == sJ_all[9] and su[1] == su_all[9]
