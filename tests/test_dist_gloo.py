"""bench.py's multi-rank plumbing on CPU: two gloo ranks, barrier and max/sum over ranks.

The path does not shard across GPUs (replicas only): each rank solves its own instance and the
reported time is the maximum over ranks; this checks that reduction without a GPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist("gloo")
    d.barrier()
    q.put((rank, d.max(1.0 + rank), d.sum(1.0), d.world))
    d.close()


def test_two_rank_max_and_sum():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=5) for _ in range(2))
    assert out == [(0, 2.0, 2.0, 2), (1, 2.0, 2.0, 2)]


def test_reference_arm_other_ranks_do_nothing(capsys, monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    assert bench.main(["--impl", "reference", "--steps", "1", "--warmup", "0"]) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_prints_line(capsys, monkeypatch):
    """The reference arm solves the configured grid itself (no scaled sample): here 31^3, one timed
    solve and the single-thread one; the reference's own build where it was compiled, else the port."""
    import json
    import bench
    monkeypatch.delenv("RANK", raising=False)
    assert bench.main(["--impl", "reference", "--steps", "1", "--warmup", "0", "--n", "31"]) == 0
    line = json.loads(capsys.readouterr().out.strip())
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["steps"] == 1 and line["warmup"] == 0 and "steps_requested" not in line
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["config"]["n"] == 31 and "31^3 itself" in line["cpu_baseline"]["sample"]
    assert line["cpu_baseline"]["single_thread"]["counts"] == [5, 12, 17]
