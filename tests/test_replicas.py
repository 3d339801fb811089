"""Multi-GPU runs are replicas (the path needs no exchange at one GPU per
state): each rank runs the whole workload, and the only collective is the
max over ranks of the step time.  Covered here with 2 gloo ranks on CPU."""
import os
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = 100.0 + 50.0 * rank          # rank 1 is the slower replica
        ms, value = bench.replica_throughput(ms_local, 2.0, 3, dist, "cpu")
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_max_time_and_sum_the_work():
    port = 29500 + (os.getpid() % 1000)
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 150.0
    assert value == pytest.approx(2.0 * 2 * 3 / 0.150)


def test_single_replica_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench

    ms, value = bench.replica_throughput(200.0, 5.0, 4)
    assert ms == 200.0 and value == pytest.approx(5.0 * 4 / 0.2)
    _ = torch


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    import argparse

    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    args = argparse.Namespace(qubits=12, layers=1, steps=1, warmup=0, gpus=2)
    assert bench.reference_arm(args) is None
    assert capsys.readouterr().out == ""
