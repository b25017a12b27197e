"""Pin the oracle against the reference CUDA binary: the reference's flow driven
by the oracle (tests/refflow.py) must write, byte for byte, the output files
the reference binary wrote on a GB300 (tests/golden/ref_*.npz, produced by
tests/golden/make_ref_golden.py): checkpoints with spins, energies, PT
permutations and every generator state, energy averages, PT acceptances,
temperature histories, couplings and seed files -- for new runs and restarts."""
import hashlib
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_ref_golden as MRG  # noqa: E402
import refflow  # noqa: E402

BC = {"PBC": 0, "OBC": 1, "WEAK": 2, "STRONG": 3}
GOLD = os.path.join(ROOT, "tests", "golden")


def compare_tree(fixture, outdir):
    d = np.load(fixture)
    checked = 0
    for key in d.files:
        kind, rel = key.split(":", 1)
        rel = rel.replace("|", "/")
        if not rel.startswith("I") or rel.endswith("run.log"):
            continue
        path = os.path.join(outdir, rel)
        assert os.path.exists(path), rel
        raw = open(path, "rb").read()
        if kind == "file":
            assert raw == d[key].tobytes(), rel
        else:
            assert hashlib.sha256(raw).digest() == d[key].tobytes(), rel
        checked += 1
    return checked


@pytest.mark.parametrize("tag", list(MRG.CASES))
def test_oracle_writes_the_reference_files(tag, tmp_path):
    fx = os.path.join(GOLD, "ref_%s.npz" % tag)
    if not os.path.exists(fx):
        pytest.skip("no fixture")
    L, Lz, bc, cl, lutname, isample, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, resume = MRG.CASES[tag]
    MRG.case_inputs(tag, str(tmp_path))
    args = (str(tmp_path), isample, nbits, str(tmp_path / "betas"), str(tmp_path / "input.in"), str(tmp_path / "LUT"),
            str(tmp_path / "list") if lst else None)
    refflow.run(*args, bc=BC[bc], cluster=bool(cl))
    if resume:
        refflow.set_resume(str(tmp_path), resume)
        refflow.run(*args, bc=BC[bc], cluster=bool(cl))
    n = compare_tree(fx, str(tmp_path))
    assert n > 10
