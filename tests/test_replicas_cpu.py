"""The N > 1 host path of bench.py on CPU: two gloo ranks.

The hot path does not shard (one GPU, replicas only), so N > 1 runs
independent replicas: a barrier around the timed region, the maximum of the
ranks' times, the units of all ranks over it, one line from rank 0, and a
reference arm that only rank 0 runs.
"""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                      RANK=str(rank), LOCAL_RANK=str(rank), AMPS_DIST_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench
    ws, r, local = bench.dist_env()
    dist = bench.init_dist(ws)
    try:
        bench.barrier(dist)
        # rank r processed (r + 1) * 1000 units in 10 + 5 r ms
        value, ms_max = bench.replica_throughput(dist, (r + 1) * 1000.0, 10.0 + 5.0 * r)
        top = bench.max_over_ranks(dist, float(r))
        total = bench.sum_over_ranks(dist, 1.0)
        bench.barrier(dist)
        q.put((r, ws, local, value, ms_max, top, total))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_aggregate():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for r, ws, local, value, ms_max, top, total in res:
        assert ws == 2 and local == r
        assert ms_max == 15.0                      # the slowest rank's time
        assert value == pytest.approx(3000.0 / 0.015)  # all units over it
        assert top == 1.0 and total == 2.0


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.init_dist(1) is None
    value, ms_max = bench.replica_throughput(None, 500.0, 2.0)
    assert ms_max == 2.0 and value == pytest.approx(250000.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """ranks other than 0 exit without work or output"""
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        workload = "amr_64c_128ppc"
        steps = 1
        warmup = 0
        ref_budget = 1.0
        ref_seconds = 1.0
    assert bench.run_reference(Args()) is None
    assert capsys.readouterr().out == ""
