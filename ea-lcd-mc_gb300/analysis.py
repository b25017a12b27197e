"""Configuration analysis: observables of the plane-overlap correlation
functions and the reference's data-file layout.

The per-sample correlation matrices come from ea_sp_plane_correlations
(`SpJob.plane_correlations(nrep, dmax)`): C[sample][slot][d][f][g], f, g in
(x, x^3, sign x) of the plane overlap q.  From them, per temperature slot and
distance d (the abscissa):

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
