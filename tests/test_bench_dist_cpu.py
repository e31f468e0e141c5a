"""The benchmark's multi-rank path on CPU (gloo, world size 2): every rank sees the slowest rank's
time, the whole-job rate counts all ranks' units over it, and the reference arm runs on rank 0
only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
    m = bench.max_over_ranks(local_ms, world)
    q.put((rank, m, bench.whole_job_rate(1000, world, m)))
    dist.destroy_process_group()


def test_max_over_ranks_and_rate_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [150.0, 150.0]
    assert all(abs(g[2] - 2 * 1000 / 0.150) < 1e-6 for g in got)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_rate(65536, 1, 4.0) == 65536 / 0.004


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    out = io.StringIO()
    with redirect_stdout(out):
        monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "3",
                                          "--warmup", "3"])
        assert bench.run_reference(bench.parse()) is None
    assert out.getvalue() == ""
