"""The ea_gb command-line driver: the reference's command line, input files and
output tree.  CPU tests cover argument handling (no device needed); the GPU
test runs the driver on every golden case of the reference binary (with the
same restarts) and compares each output file byte for byte."""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_ref_golden as MRG  # noqa: E402

EXE = os.path.join(ROOT, "ea-lcd-mc_gb300", "ea_gb")
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    subprocess.run([sys.executable, os.path.join(ROOT, "ea-lcd-mc_gb300", "build.py")], check=True,
                   stdout=subprocess.DEVNULL)


def run(args, cwd=None, exe=EXE):
    return subprocess.run([exe] + [str(a) for a in args], cwd=cwd, capture_output=True, text=True, timeout=600)


def test_help_and_usage():
    r = run(["-h"])
    assert r.returncode == 0
    assert "isample ibit beta.dat input.in LUT device [max_time [list_samples]]" in r.stdout
    assert "max_time (opt.)" in r.stdout
    r = run([1, 2, 3])
    assert r.returncode == 1 and "Usage:" in r.stderr


def test_argument_ranges():
    r = run([0, 32, "b", "i", "l", 0])
    assert r.returncode == 1 and "nbits out of range, 0 <= bit < 32" in r.stderr
    r = run([-1, 2, "b", "i", "l", 0])
    assert r.returncode == 1 and "sample out of range" in r.stderr
    r = run([16384, 2, "b", "i", "l", 0])
    assert r.returncode == 1 and "cannot accomodate more than 16384 samples" in r.stderr


def exe_name(L, Lz, NB, bc, cluster):
    suffix = {"PBC": "_PBC", "OBC": "_OBC", "WEAK": "_OBC_WEAK", "STRONG": "_OBC_STRONG"}[bc]
    return "EA_CUBE_L%d_Lz%d_NB%d_NBPRE12%s%s" % (L, Lz, NB, suffix, "" if cluster else "_NO_CLUSTER")


def compare_tree(fixture, outdir):
    d = np.load(fixture)
    n = 0
    for key in d.files:
        kind, rel = key.split(":", 1)
        rel = rel.replace("|", "/")
        if not rel.startswith("I") or rel.endswith("run.log"):
            continue
        raw = open(os.path.join(outdir, rel), "rb").read()
        if kind == "file":
            assert raw == d[key].tobytes(), rel
        else:
            assert hashlib.sha256(raw).digest() == d[key].tobytes(), rel
        n += 1
    return n


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(MRG.CASES))
def test_driver_writes_the_reference_files(tag, tmp_path):
    L, Lz, bc, cl, lutname, isample, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, resume = MRG.CASES[tag]
    nb = MRG.case_inputs(tag, str(tmp_path))
    link = tmp_path / exe_name(L, Lz, nb, bc, cl)
    os.symlink(EXE, link)
    args = [isample, nbits, "betas", "input.in", "LUT", 0, 0] + (["list"] if lst else [])
    r = run(args, cwd=str(tmp_path), exe=str(link))
    assert r.returncode == 0, r.stderr + r.stdout[-2000:]
    assert "finished at iteration %d" % nbin in r.stdout
    if resume:
        import refflow
        refflow.set_resume(str(tmp_path), resume)
        r = run(args, cwd=str(tmp_path), exe=str(link))
        assert r.returncode == 0, r.stderr
        assert "finished at iteration %d" % resume in r.stdout
    assert compare_tree(os.path.join(GOLD, "ref_%s.npz" % tag), str(tmp_path)) > 10
    assert not os.path.exists(tmp_path / ("I%03d" % isample) / "running")


@pytest.mark.gpu
def test_driver_refuses_second_instance_and_bad_restart(tmp_path):
    tag = "r3_L8_Lz16_WEAK"
    L, Lz, bc, cl, lutname, isample, nbits, lst, nbin, itmax, houfr, mesfr, ptfr, resume = MRG.CASES[tag]
    nb = MRG.case_inputs(tag, str(tmp_path))
    link = tmp_path / exe_name(L, Lz, nb, bc, cl)
    os.symlink(EXE, link)
    base = tmp_path / ("I%03d" % isample)
    base.mkdir()
    (base / "running").write_text("otherhost 1 0 x\n")
    args = [isample, nbits, "betas", "input.in", "LUT", 0, 0]
    r = run(args, cwd=str(tmp_path), exe=str(link))
    assert r.returncode == 1 and "running exists" in r.stderr
    (base / "running").unlink()
    r = run(args, cwd=str(tmp_path), exe=str(link))
    assert r.returncode == 0
    # a new run (flag 1) over existing configurations is refused
    r = run(args, cwd=str(tmp_path), exe=str(link))
    assert r.returncode == 1 and "There are confs" in r.stderr
    # a truncated checkpoint is detected on restart
    import refflow
    refflow.set_resume(str(tmp_path), nbin + 1)
    conf = base / "BIT000" / "R03" / "conf"
    data = conf.read_bytes()
    os.unlink(conf)
    conf.write_bytes(data[:-7])
    r = run(args, cwd=str(tmp_path), exe=str(link))
    assert r.returncode == 1 and "Problems reading confs" in r.stderr
    assert "There are only" in (base / "error").read_text()
