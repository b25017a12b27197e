"""Configuration analysis: observables of the plane-overlap correlation
functions and the reference's data-file layout.

The per-sample correlation matrices come from ea_sp_plane_correlations
(`SpJob.plane_correlations(nrep, dmax)`, on the GPU) for sample-packed jobs,
or from `multispin_plane_diff` + `plane_correlations` (on the host) for
configurations in the reference's multispin layout: C[sample][slot][d][f][g],
f, g in (x, x^3, sign x) of the plane overlap q.  From them, per temperature
slot and distance d (the abscissa):

    C_fg(d)        the sample mean; normalised: C_fg(d) / sqrt(C_ff(0) C_gg(0))
    DET(d)         det of the 3 x 3 matrix C(d); normalised: det of the
                   normalised matrix
    MIN_fg(d)      det of the 2 x 2 matrix of (f, g); normalised likewise

with jackknife errors over `nblocks` consecutive blocks of samples.  Files
follow the column layout of the reference's data description
(DATA/README.md): temperature index, beta, abscissa, observable, error,
normalised observable, normalised error.  Names: `C_<f>_<g>`, `DET`,
`MIN_<f>_<g>`, then `_n<n>_NS<samples>.dat`, n = r/2 - 1 for r replicas and
f, g written Q, Q3, signQ as the reference's file names write them.
"""
import itertools
import os

import numpy as np

NAMES = ("Q", "Q3", "signQ")


def multispin_plane_diff(eagb, g, spins, wctb, nrep):
    """Differing spins per (sample, pair, beta, plane) of multispin
    configurations (the reference's layout): spins[s] = (even, odd) words of
    sample s, wctb[s][r][b] the clone of replica r at beta b.  The words are
    unpacked on the host (ea_host_unpack_replica); pairs (0,1), (2,3), ...
    Returns diff [nsamples][nrep/2][NB][Lz]."""
    L, Lz, NB = g.L, g.Lz, g.nbetas
    ns = len(spins)
    out = np.zeros((ns, nrep // 2, NB, Lz), np.int32)
    for s, (even, odd) in enumerate(spins):
        u = [eagb.host_unpack_replica(g, even, odd, r) for r in range(nrep)]
        for k in range(nrep // 2):
            for b in range(NB):
                a = u[2 * k][wctb[s][2 * k][b]]
                c = u[2 * k + 1][wctb[s][2 * k + 1][b]]
                out[s, k, b] = (a != c).reshape(Lz, L * L).sum(1)
    return out


def plane_correlations(diff, L2, pbc, dmax):
    """The correlation matrices of ea_sp_plane_correlations computed on the
    host from plane counts diff[sample][pair][beta][z] (numpy summation
    order): C[sample][beta][d][3][3]."""
    q = 1.0 - (2.0 / L2) * diff.astype(np.float64)
    F = np.stack([q, q * q * q, np.sign(q)], -1)            # [s][pair][b][z][3]
    Lz = diff.shape[-1]
    ns, _, NB, _ = diff.shape
    out = np.zeros((ns, NB, dmax + 1, 3, 3))
    for d in range(dmax + 1):
        if pbc:
            A, B = F, np.roll(F, -d, axis=3)
        else:
            A, B = F[:, :, :, :Lz - d], F[:, :, :, d:]
        if A.shape[3] == 0:
            continue
        out[:, :, d] = np.einsum("skbzf,skbzg->sbfg", A, B) / (A.shape[1] * A.shape[3])
    return out


def _normalised(M):
    """M[..., d, 3, 3] -> M / sqrt(diag(M(d=0)) outer diag(M(d=0)))."""
    diag = np.diagonal(M[..., 0, :, :], axis1=-2, axis2=-1)  # [..., 3]
    scale = np.sqrt(np.abs(diag[..., :, None] * diag[..., None, :]))
    with np.errstate(divide="ignore", invalid="ignore"):
        return M / scale[..., None, :, :]


def _observables(M):
    """Every observable of a mean matrix set M[slot][d][3][3]: a dict of
    name -> (plain [slot][d], normalised [slot][d])."""
    Mn = _normalised(M)
    out = {}
    for f, g in itertools.product(range(3), range(3)):
        out["C_%s_%s" % (NAMES[f], NAMES[g])] = (M[..., f, g], Mn[..., f, g])
    out["DET"] = (np.linalg.det(M), np.linalg.det(Mn))
    for f, g in itertools.combinations(range(3), 2):
        sub = np.ix_([f, g], [f, g])
        out["MIN_%s_%s" % (NAMES[f], NAMES[g])] = (np.linalg.det(M[..., sub[0], sub[1]]),
                                                   np.linalg.det(Mn[..., sub[0], sub[1]]))
    return out


def correlation_observables(C, nblocks=10):
    """C: [samples][slot][d][3][3] per-sample matrices.  Returns name ->
    (value, error, normalised, normalised error), each [slot][d]; errors by
    the jackknife over `nblocks` consecutive blocks of samples."""
    C = np.asarray(C, np.float64)
    ns = C.shape[0]
    if ns < 2:
        raise ValueError("the jackknife needs at least 2 samples, got %d" % ns)
    nb = max(2, min(nblocks, ns))
    edges = np.linspace(0, ns, nb + 1).astype(int)
    sums = np.stack([C[edges[i]:edges[i + 1]].sum(0) for i in range(nb)])
    counts = np.diff(edges).astype(np.float64)
    full = _observables(sums.sum(0) / ns)
    jk = [_observables((sums.sum(0) - sums[i]) / (ns - counts[i])) for i in range(nb)]
    res = {}
    for name, (v, vn) in full.items():
        a = np.stack([j[name][0] for j in jk])
        an = np.stack([j[name][1] for j in jk])
        err = np.sqrt((nb - 1) / nb * ((a - a.mean(0)) ** 2).sum(0))
        errn = np.sqrt((nb - 1) / nb * ((an - an.mean(0)) ** 2).sum(0))
        res[name] = (v, err, vn, errn)
    return res


def write_data_files(outdir, obs, betas, nrep, nsamples):
    """One file per observable, the reference's seven columns."""
    os.makedirs(outdir, exist_ok=True)
    n = nrep // 2 - 1
    paths = []
    for name, (v, e, vn, en) in obs.items():
        path = os.path.join(outdir, "%s_n%d_NS%d.dat" % (name, n, nsamples))
        with open(path, "w") as f:
            for b in range(v.shape[0]):
                for d in range(v.shape[1]):
                    f.write("%d %.10g %d %.10g %.10g %.10g %.10g\n" % (b, betas[b], d, v[b, d], e[b, d], vn[b, d], en[b, d]))
        paths.append(path)
    return paths
