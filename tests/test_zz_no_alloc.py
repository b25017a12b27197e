"""GPU test of ea_measure_energy_noalloc, the energy entry point that allocates
no device memory.  It serves callers that cannot call cudaMalloc: frameworks
that own every device byte through their own pool, and loops that cannot
take the synchronisation an allocation may imply.  Its energies must equal
those of ea_measure_energy -- integer sums, so the tolerance is zero -- on two
calls in a row, through the C ABI, for every replica count it takes (NR = 8,
4, 2: tile widths 4, 8, 16) and for a lattice at its half-site limit.  This
file is collected last on purpose: a run that stops at the first failure has
run every other test before it."""
import ctypes as C
import importlib.util
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)

MASTERS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)
EA_ERR_ARG = -1


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


@pytest.fixture
def noalloc():
    """The entry point with its argument types, and ea_last_error returning the
    message text (set before any call, so that a failure shows the message)."""
    lib = eagb.lib()
    lib.ea_last_error.restype = C.c_char_p
    fn = lib.ea_measure_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn, lib


def device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int64)).cuda()


# L, Lz, temperature set (first NB temperatures), boundary, samples, replicas
CASES = [(16, 24, "T07_16_N8", 8, eagb.EA_OBC_STRONG, 2, 8),
         (8, 8, "T08_16_N4", 4, eagb.EA_PBC, 3, 8),
         (8, 16, "T07_16_N6", 6, eagb.EA_OBC, 2, 4),
         (16, 8, "T08_16_N4", 4, eagb.EA_OBC_WEAK, 3, 2),
         (64, 256, "T08_16_N4", 2, eagb.EA_OBC, 1, 2)]   # (L/4)^2 (Lz/4) / 2 = 8192 half-sites: the limit


@pytest.mark.parametrize("L,Lz,lut,nb,bc,ns,NR", CASES)
def test_noalloc_energy_matches_allocating_path(noalloc, L, Lz, lut, nb, bc, ns, NR):
    torch = pytest.importorskip("torch")
    fn, lib = noalloc
    d = np.load(os.path.join(ROOT, "tests", "golden", "lut_%s.npz" % lut))
    betas, cum = d["betas"][:nb], d["cum"][:nb]
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, NR=NR, bc=bc, masters=MASTERS)
    g = job.g
    assert g.nrep == NR
    sJ, su, sMC = eagb.host_seeds(MASTERS, ns, NR)
    Jw = np.stack([eagb.host_init_couplings(g, int(sJ[s]))[1] for s in range(ns)])
    d_J = device_copy(torch, Jw)
    d_E = torch.zeros(ns * g.nrep * g.nbetas, dtype=torch.int32, device="cuda")
    for call in range(2):
        job.monte_carlo(1 + call)
        want = job.measure_energy()
        spins = np.stack([np.stack(job.get_spins(s)) for s in range(ns)])
        d_S = device_copy(torch, spins)
        d_E.fill_(-1)
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(C.byref(g), C.c_void_p(d_S.data_ptr()), C.c_void_p(d_J.data_ptr()), C.c_void_p(d_E.data_ptr()),
                C.c_void_p(stream))
        assert rc == 0, lib.ea_last_error()
        torch.cuda.synchronize()
        got = d_E.cpu().numpy().reshape(ns, g.nrep, g.nbetas)
        assert np.array_equal(got, want), "call %d" % call
    job.close()


@pytest.mark.parametrize("L,Lz,NB,NR,ns,what", [(64, 512, 40, 8, 32, "half-sites"),
                                                (64, 256, 32, 8, 3, "partial sums"),
                                                (8, 8, 4, 6, 1, "replicas")])
def test_noalloc_rejects_jobs_beyond_its_scratch(noalloc, L, Lz, NB, NR, ns, what):
    """16384 half-sites > 8192; 8192 half-sites with KT=4 and 3 x 32 x 8
    columns give 3 x 2^19 partial sums > 2^20; NR=6 has no tile width.  The
    call is refused before any launch, with EA_ERR_ARG and a message."""
    torch = pytest.importorskip("torch")
    fn, lib = noalloc
    g = eagb.geom(L, Lz, NB, NR, ns, eagb.EA_OBC)
    x = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = fn(C.byref(g), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), None)
    assert rc == EA_ERR_ARG, what
    msg = lib.ea_last_error()
    assert (b"NR must be" if what == "replicas" else b"scratch") in msg, msg
