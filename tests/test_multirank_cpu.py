"""The multi-rank bench logic on CPU ranks (gloo, world size 2): the slowest
rank's time wins, the whole-job rate counts every replica, ranks read their
identity from the launcher's environment, and only rank 0 runs the
reference arm."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        ms = 10.0 + 5.0 * rank            # rank 1 is the slow one
        slowest = bench.max_over_ranks(ms, torch.device("cpu"))
        dist.barrier()
        out.put((r, w, local, slowest, bench.whole_job_mvis(w, 1_000_000, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for r, w, local, slowest, rate in res:
        assert w == 2 and local == r
        assert slowest == 15.0
        assert rate == pytest.approx(2 * 1e6 / 15e-3 / 1e6)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(3.5, torch.device("cpu")) == 3.5
    assert bench.whole_job_mvis(1, 2_000_000, 10.0) == pytest.approx(200.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1"])
    bench.run_reference(bench.parse())
    assert capsys.readouterr().out == ""


def test_reference_arm_line(monkeypatch, capsys):
    """The reference arm on rank 0: one JSON line with the contract's keys,
    timed on the host (the oracle's Complex32 restatement of the path)."""
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1",
                                      "--warmup", "0"])
    bench.run_reference(bench.parse())
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "Mvis/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    assert d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
