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


# ---------------------------------------------------------------------------
# Run management (io.c:870-938, timing.c:43-74): signals, changenbin.in and
# the wall-time budget.  Every failure here is made on the host (a signal to
# the driver process, a file dropped in its directory); nothing faults a GPU.
# The geometry is golden case r1 (PBC, no cluster moves, houfr = 1): with
# houfr = 1 the restart counter equals the continuous one and no cluster
# uniforms are drawn, so a restarted run must end byte-identical to a
# continuous one.
# ---------------------------------------------------------------------------
def _r1_inputs(path, nbin):
    import refflow
    L, Lz, bc, cl, lutname, isample, nbits, lst, _, itmax, houfr, mesfr, ptfr, _ = MRG.CASES["r1_L8_Lz8_PBC_nocl"]
    d = np.load(os.path.join(GOLD, "lut_%s.npz" % lutname))
    refflow.write_case_inputs(str(path), L, Lz, d["betas"], d["cum"], nbits, None, nbin, itmax, houfr, mesfr, ptfr,
                              MRG.MASTERS)
    link = path / exe_name(L, Lz, len(d["betas"]), bc, cl)
    os.symlink(EXE, link)
    return str(link), [isample, nbits, "betas", "input.in", "LUT", 0], path / ("I%03d" % isample), nbits


def _confs(base):
    p = base / "BIT000" / "R00"
    return sorted(f for f in os.listdir(p) if f.startswith("conf.")) if p.is_dir() else []


def _wait(pred, timeout, proc=None):
    import time
    t_end = time.time() + timeout
    while time.time() < t_end:
        if pred():
            return True
        if proc is not None and proc.poll() is not None:
            return pred()
        time.sleep(0.002)
    return False


def _same_outputs(a, b, nbits, names=("evol.txt", "history_b.dat")):
    """Restarted tree a against continuous tree b: the files byte for byte;
    the checkpoints too, except the run-data header's restart flag (bytes
    28..31, the input file's flag: 0 for the restart, 1 for the new run)."""
    n = 0
    for i in range(nbits):
        for r in range(8):
            ra, rb = a / ("BIT%03d" % i) / ("R%02d" % r), b / ("BIT%03d" % i) / ("R%02d" % r)
            for f in names:
                assert (ra / f).read_bytes() == (rb / f).read_bytes(), (i, r, f)
                n += 1
            ca, cb = (ra / "conf").read_bytes(), (rb / "conf").read_bytes()
            assert len(ca) == len(cb)
            assert ca[28:32] == (0).to_bytes(4, "little") and cb[28:32] == (1).to_bytes(4, "little")
            assert ca[:28] == cb[:28] and ca[32:] == cb[32:], (i, r, "conf")
            n += 1
    return n


@pytest.mark.gpu
def test_sigterm_between_bins_then_restart_is_byte_identical(tmp_path):
    """SIGTERM while bins run: the driver writes <dir>/error ('Received
    SIGTERM'), removes the lock file and exits 1.  Signals are ignored while
    it writes its files (main.cu:235,262), so the test repeats the signal
    until the process is gone.  A restart (flag 0) from the last checkpoint
    then ends byte-identical -- checkpoints, evol.txt, history_b.dat -- to a
    run that was never interrupted."""
    import signal
    import time
    import refflow
    run_dir, cont_dir = tmp_path / "run", tmp_path / "cont"
    run_dir.mkdir()
    cont_dir.mkdir()
    exe, args, base, nbits = _r1_inputs(run_dir, 1000000)
    p = subprocess.Popen([exe] + [str(a) for a in args], cwd=str(run_dir), stdout=subprocess.PIPE,
                         stderr=subprocess.PIPE, text=True)
    try:
        assert _wait(lambda: len(_confs(base)) >= 3, 300, p), "no bins were written"
        t_end = time.time() + 60
        while p.poll() is None and time.time() < t_end:
            p.send_signal(signal.SIGTERM)
            time.sleep(0.01)
        out, err = p.communicate(timeout=60)
    finally:
        if p.poll() is None:
            p.kill()
            p.wait()
    assert p.returncode == 1, (p.returncode, err[-2000:])
    assert "Aborting programma (SIGNAL=%d)" % signal.SIGTERM in out + err
    assert (base / "error").read_text().startswith("Received SIGTERM")
    assert not (base / "running").exists()
    done = len(_confs(base))
    assert done >= 3
    # restart from the last checkpoint up to done + 2 bins
    refflow.set_resume(str(run_dir), done + 2)
    r = run(args, cwd=str(run_dir), exe=exe)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "finished at iteration %d" % (done + 2) in r.stdout
    # the same run without interruption
    exe2, args2, base2, _ = _r1_inputs(cont_dir, done + 2)
    r = run(args2, cwd=str(cont_dir), exe=exe2)
    assert r.returncode == 0, r.stderr[-2000:]
    assert _same_outputs(base, base2, nbits) == nbits * 8 * 3


@pytest.mark.gpu
def test_changenbin_file_is_honoured(tmp_path):
    """<dir>changenbin.in overrides nbin (io.c:870-891): read at start-up and
    after every bin, then removed.  Dropped before the run it cuts 50 bins to
    3; dropped while a practically endless run is going, the run ends at the
    bin it names."""
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    exe, args, base, nbits = _r1_inputs(a, 50)
    base.mkdir()
    (base / "changenbin.in").write_text("3\n")
    r = run(args, cwd=str(a), exe=exe)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "nbin changed to 3" in r.stdout and "finished at iteration 3" in r.stdout
    assert not (base / "changenbin.in").exists()
    assert len(_confs(base)) == 3
    exe, args, base, nbits = _r1_inputs(b, 1000000)
    p = subprocess.Popen([exe] + [str(x) for x in args], cwd=str(b), stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                         text=True)
    try:
        assert _wait(lambda: len(_confs(base)) >= 2, 300, p), "no bins were written"
        target = len(_confs(base)) + 200
        (base / "changenbin.in.tmp").write_text("%d\n" % target)
        os.rename(base / "changenbin.in.tmp", base / "changenbin.in")   # appears whole
        out, err = p.communicate(timeout=600)
    finally:
        if p.poll() is None:
            p.kill()
            p.wait()
    assert p.returncode == 0, err[-2000:]
    assert "nbin changed to %d" % target in out and "finished at iteration %d" % target in out
    assert len(_confs(base)) == target
    assert not (base / "changenbin.in").exists()


@pytest.mark.gpu
def test_time_budget_stops_cleanly(tmp_path):
    """max_time (timing.c:43-74): the run stops once mean + 3 sigma of a bin
    (whole seconds, plus one) no longer fits in the budget.  With a budget of
    1 s the first check already finds no room: one bin is written, the lock
    is removed, no error file, exit 0.  A large budget lets every bin run."""
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    exe, args, base, nbits = _r1_inputs(a, 1000)
    r = run(args + [1], cwd=str(a), exe=exe)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "finished at iteration" in r.stdout
    assert len(_confs(base)) == 1
    assert not (base / "running").exists() and not (base / "error").exists()
    exe, args, base, nbits = _r1_inputs(b, 4)
    r = run(args + [10 ** 9], cwd=str(b), exe=exe)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "finished at iteration 4" in r.stdout and len(_confs(base)) == 4
