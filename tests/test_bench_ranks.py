"""bench.py's multi-rank host logic on CPU: two gloo ranks (one replica
each, no collective on the data path).  The timings are reduced to the
slowest rank's on every rank, and the reference arm prints one JSON line
from rank 0 while the other rank exits without work."""
import contextlib
import importlib.util
import io
import json
import os
import socket

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
        bench = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(bench)
        got = bench.max_over_ranks(torch, [1.0 + rank, 10.0 - rank, 5.0], "cpu", world)
        # the reference arm with a stand-in for the host cycle (the oracle's
        # timing is not what this checks)
        bench.cpu_cycle = lambda steps, warmup: (4.0e12 * steps, 2.0 * steps)
        args = type("A", (), {"steps": 3, "warmup": 1})()
        out = io.StringIO()
        with contextlib.redirect_stdout(out):
            bench.run_reference(args, rank, world)
        torch.distributed.barrier()
        q.put((rank, got, out.getvalue()))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        rank, got, out = q.get(timeout=120)
        res[rank] = (got, out)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        assert res[rank][0] == [2.0, 10.0, 5.0]
    assert res[1][1] == ""
    lines = [l for l in res[0][1].splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] == pytest.approx(2.0) and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["value"] == line["value"]
