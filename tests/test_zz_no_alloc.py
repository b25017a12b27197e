"""GPU test of ea_measure_energy_noalloc, the energy entry point that allocates
no device memory (for callers that cannot call cudaMalloc, e.g. while a CUDA
graph is being captured).  It must give exactly the energies of
ea_measure_energy -- integer sums, so the tolerance is zero -- on two calls in
a row, through the C ABI.  This file is collected last on purpose."""
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


@pytest.fixture(scope="module", autouse=True)
def built():
    import subprocess
    import sys
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def device_copy(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int64)).cuda()


@pytest.mark.parametrize("L,Lz,lut,bc,ns", [(16, 24, "T07_16_N8", eagb.EA_OBC_STRONG, 2),
                                            (8, 8, "T08_16_N4", eagb.EA_PBC, 3)])
def test_noalloc_energy_matches_allocating_path(L, Lz, lut, bc, ns):
    torch = pytest.importorskip("torch")
    d = np.load(os.path.join(ROOT, "tests", "golden", "lut_%s.npz" % lut))
    betas, cum = d["betas"], d["cum"]
    job = eagb.new_job(L, Lz, betas, cum, nsamples=ns, bc=bc, masters=MASTERS)
    lib = eagb.lib()
    fn = lib.ea_measure_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    g = job.g
    sJ, su, sMC = eagb.host_seeds(MASTERS, ns)
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


def test_noalloc_rejects_jobs_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = eagb.lib()
    fn = lib.ea_measure_energy_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.ea_last_error.restype = C.c_char_p
    g = eagb.geom(64, 512, 40, 8, 32, eagb.EA_OBC)   # 16384 half-sites > 8192
    x = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = fn(C.byref(g), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), None)
    assert rc == -1
    assert b"scratch" in lib.ea_last_error()
