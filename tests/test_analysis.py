"""Configuration analysis (plane-overlap correlation functions).

CPU: the observables of analysis.py -- sample means, normalised matrices,
determinants, 2 x 2 minors, jackknife errors -- against direct numpy, and the
seven-column file layout.  GPU: ea_sp_plane_overlaps against counts made
from the spin words, and ea_sp_plane_correlations against a restatement in
Python floats with the same order of operations (exact: tolerance 0)."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import ROOT

spec = importlib.util.spec_from_file_location("eagb", os.path.join(ROOT, "ea-lcd-mc_gb300", "eagb.py"))
eagb = importlib.util.module_from_spec(spec)
spec.loader.exec_module(eagb)
aspec = importlib.util.spec_from_file_location("analysis", os.path.join(ROOT, "ea-lcd-mc_gb300", "analysis.py"))
analysis = importlib.util.module_from_spec(aspec)
aspec.loader.exec_module(analysis)

SEEDS = (0x1234567890ABCDEF, 0x0FEDCBA987654321, 0x1111222233334444, 0x5555666677778888)


def test_observables_and_jackknife():
    rng = np.random.default_rng(3)
    ns, nb, nd = 40, 3, 4
    A = rng.normal(size=(ns, nb, nd, 3, 3))
    C = A @ np.swapaxes(A, -1, -2) + 3 * np.eye(3)   # symmetric positive matrices
    obs = analysis.correlation_observables(C, nblocks=8)
    M = C.mean(0)
    assert np.allclose(obs["C_Q_Q3"][0], M[..., 0, 1])
    assert np.allclose(obs["DET"][0], np.linalg.det(M))
    assert np.allclose(obs["MIN_Q_signQ"][0], M[..., 0, 0] * M[..., 2, 2] - M[..., 0, 2] * M[..., 2, 0])
    d0 = np.diagonal(M[:, 0], axis1=-2, axis2=-1)
    Mn = M / np.sqrt(d0[:, None, :, None] * d0[:, None, None, :])
    assert np.allclose(obs["C_Q3_Q3"][2][:, 0], 1.0)
    assert np.allclose(obs["DET"][2], np.linalg.det(Mn))
    # jackknife of the mean of one entry over 8 blocks of 5 samples
    x = C[:, 1, 2, 0, 1]
    blocks = x.reshape(8, 5).sum(1)
    jk = (blocks.sum() - blocks) / 35
    err = np.sqrt(7 / 8 * ((jk - jk.mean()) ** 2).sum())
    assert np.isclose(obs["C_Q_Q3"][1][1, 2], err)


def test_jackknife_block_edges():
    """Fewer samples than blocks: one sample a block (the plain jackknife);
    a single sample has no error estimate and is refused."""
    rng = np.random.default_rng(6)
    C = rng.normal(size=(3, 1, 2, 3, 3))
    obs = analysis.correlation_observables(C, nblocks=10)
    x = C[:, 0, 1, 0, 2]
    jk = (x.sum() - x) / 2
    assert np.isclose(obs["C_Q_signQ"][1][0, 1], np.sqrt(2 / 3 * ((jk - jk.mean()) ** 2).sum()))
    with pytest.raises(ValueError):
        analysis.correlation_observables(C[:1])


def test_data_file_layout(tmp_path):
    rng = np.random.default_rng(4)
    C = rng.normal(size=(16, 2, 3, 3, 3))
    C = C @ np.swapaxes(C, -1, -2)
    obs = analysis.correlation_observables(C, nblocks=4)
    paths = analysis.write_data_files(str(tmp_path), obs, [1.25, 1.1], nrep=4, nsamples=16)
    assert len(paths) == 9 + 1 + 3
    names = sorted(os.path.basename(p) for p in paths)
    assert "DET_n1_NS16.dat" in names and "C_Q_signQ_n1_NS16.dat" in names and "MIN_Q3_signQ_n1_NS16.dat" in names
    rows = [l.split() for l in open(os.path.join(str(tmp_path), "C_Q_Q_n1_NS16.dat"))]
    assert len(rows) == 2 * 3 and all(len(r) == 7 for r in rows)
    assert rows[4][0] == "1" and float(rows[4][1]) == 1.1 and rows[4][2] == "1"


def restated_correlations(diff, L2, Lz, pbc, dmax):
    """Python floats, the kernel's order: pairs, then planes."""
    nw, _, npairs, NB, _ = diff.shape
    out = np.zeros((nw * 64, NB, dmax + 1, 3, 3))
    inv = 1.0 / L2

    def basis(x):
        return (x, (x * x) * x, 1.0 if x > 0 else (-1.0 if x < 0 else 0.0))

    for w in range(nw):
        for lane in range(64):
            for b in range(NB):
                for dd in range(dmax + 1):
                    acc = [0.0] * 9
                    n = 0
                    for k in range(npairs):
                        row = diff[w, lane, k, b]
                        for z in range(Lz if pbc else Lz - dd):
                            z2 = (z + dd) % Lz if pbc else z + dd
                            f = basis(1.0 - (2.0 * inv) * float(row[z]))
                            g = basis(1.0 - (2.0 * inv) * float(row[z2]))
                            for p in range(3):
                                for q in range(3):
                                    acc[p * 3 + q] = acc[p * 3 + q] + f[p] * g[q]
                            n += 1
                    out[w * 64 + lane, b, dd] = np.array([a / n if n else 0.0 for a in acc]).reshape(3, 3)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("L,Lz,bc,NR,nrep", [(4, 6, eagb.EA_PBC, 4, 4), (3, 5, eagb.EA_OBC, 2, 2)])
def test_plane_overlaps_and_correlations(L, Lz, bc, NR, nrep):
    d = np.load(os.path.join(ROOT, "tests", "golden", "lut_T07_16_N6.npz"))
    betas, cum = d["betas"][:3], d["cum"][:3]
    job = eagb.SpJob(L, Lz, betas, cum, nrep=NR, nwords=1, bc=bc, seeds=SEEDS)
    job.run_bin(3, 1, 1, 1, cluster=False)
    S = job.get_spins()                      # [w][site][r][b]
    diff = job.plane_overlaps(nrep)
    L2 = L * L
    want = np.zeros_like(diff)
    for k in range(nrep // 2):
        x = S[:, :, 2 * k, :] ^ S[:, :, 2 * k + 1, :]          # [w][site][b]
        bits = (x[..., None] >> np.arange(64, dtype=np.uint64)) & np.uint64(1)   # [w][site][b][lane]
        per = bits.reshape(1, Lz, L2, len(betas), 64).sum(2)   # [w][z][b][lane]
        want[:, :, k] = np.transpose(per, (0, 3, 2, 1))
    assert np.array_equal(diff, want)
    dmax = Lz - 1
    C = job.plane_correlations(nrep, dmax)
    assert np.array_equal(C, restated_correlations(diff, L2, Lz, bc == eagb.EA_PBC, dmax))
    # sign(q)^2 at distance 0: the fraction of planes whose overlap is not zero
    nonzero = (2 * diff != L2).mean(axis=(2, 4)).reshape(64, len(betas))
    assert np.allclose(C[:, :, 0, 2, 2], nonzero)
    job.close()


def test_multispin_plane_diff_and_host_correlations():
    """Multispin configurations (the reference's layout): plane counts from
    the packed words equal counts from the bytes they were packed from, with
    each replica's clone at each beta; the host correlations equal the
    restatement within FP64 rounding (numpy sums in another order)."""
    L, Lz, NB, NR, ns = 8, 16, 3, 4, 2
    g = eagb.geom(L, Lz, NB, NR=NR, nsamples=ns, bc=eagb.EA_PBC)
    half, V = eagb.sizes(g)
    rng = np.random.default_rng(9)
    spins, bytes_ = [], []
    for s in range(ns):
        even = np.zeros(NB * half * NR, np.uint64)
        odd = np.zeros(NB * half * NR, np.uint64)
        u = rng.integers(0, 2, size=(NR, NB, V), dtype=np.uint8)
        for r in range(NR):
            eagb.host_pack_replica(g, u[r], r, even, odd)
        spins.append((even, odd))
        bytes_.append(u)
    wctb = np.array([[rng.permutation(NB) for _ in range(NR)] for _ in range(ns)])
    diff = analysis.multispin_plane_diff(eagb, g, spins, wctb, 4)
    for s in range(ns):
        for k in range(2):
            for b in range(NB):
                a = bytes_[s][2 * k][wctb[s][2 * k][b]]
                c = bytes_[s][2 * k + 1][wctb[s][2 * k + 1][b]]
                assert np.array_equal(diff[s, k, b], (a != c).reshape(Lz, L * L).sum(1))
    C = analysis.plane_correlations(diff, L * L, True, 5)
    # the restatement walks 64 lanes of one word: the samples, then zero padding
    padded = np.concatenate([diff[None], np.zeros((1, 64 - ns, 2, NB, Lz), np.int32)], 1)
    want = restated_correlations(padded, L * L, Lz, True, 5)[:ns]
    assert np.allclose(C, want, rtol=1e-12, atol=1e-14)
