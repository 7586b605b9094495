"""Replicas across ranks (bench.py, N > 1): every rank renders the same per-GPU work, the
step time is the slowest rank's, and the whole-job rate counts every rank's rays. Checked
with two gloo ranks on the CPU; the reference arm runs on rank 0 only."""
import os
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")  # rank 1 is the slow one
        out[rank] = (ms, bench.replica_throughput(2_073_600 * 16, world, ms))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = 29500 + os.getpid() % 2000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    ms, rate = out[0]
    assert ms == 15.0
    assert rate == pytest.approx(2 * 2_073_600 * 16 / 0.015 / 1e9)


def test_single_process_is_its_own_maximum():
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.replica_throughput(1_000_000, 1, 1.0) == pytest.approx(1.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    args = bench.argparse.Namespace(cpu_fraction=0.01, warmup=0, steps=1)
    assert bench.run_reference(args, "sphere") is None
    assert capsys.readouterr().out == ""
