"""Multi-process aggregation of bench.py on CPU: world-size-2 gloo group.

The fluid step runs as independent replicas (one scene per GPU, no data-path
collective); the only cross-rank operation is the max over ranks of the timed
region.  These tests run that aggregation with real gloo ranks on 127.0.0.1.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, secs_of_rank, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        value, secs = bench.replica_rate(1000, 5, secs_of_rank[rank], dist)
        out.put((rank, value, secs))
    finally:
        dist.destroy_process_group()


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    value, secs = bench.replica_rate(1000, 5, 2.0)
    assert secs == 2.0
    assert value == pytest.approx(2500.0)


def test_replica_rate_two_gloo_ranks_takes_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    secs_of_rank = [1.0, 4.0]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, secs_of_rank, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, secs in got:
        # both ranks see the slowest rank's time; 2 ranks x 1000 units x 5 steps in 4 s
        assert secs == 4.0
        assert value == pytest.approx(2 * 1000 * 5 / 4.0)


def test_reference_arm_non_zero_rank_exits_without_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(steps=1, warmup=0)
    assert bench.reference_arm(args) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_prints_the_contract_line(monkeypatch, capsys):
    """Rank 0 of the reference arm: the reference's CPU step on the sample
    scene (shortened here: a 2-step pre-roll, one process, 2 iterations) and
    one JSON line with the GPU arm's metric, unit and direction."""
    sys.path.insert(0, ROOT)
    import argparse
    import json
    import bench
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setattr(bench, "host_cores", lambda: 1)
    monkeypatch.setattr(bench, "REF_ITERS", 2)
    args = argparse.Namespace(steps=1, warmup=0, preroll=2)
    assert bench.reference_arm(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["iterations"] == 2 and line["config"]["processes"] == 1
    assert line["cpu_baseline"]["cores"] == 1 and line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
