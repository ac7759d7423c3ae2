"""Replica aggregation of bench.py on two gloo ranks (CPU): the job's time is the slowest
rank's and the rate counts every rank's solves; the reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = [300.0, 500.0][rank]           # rank 1 is the slow one
    ms_step, rate = bench.replica_rate(ms_local, 5, world, dist, "cpu")
    out[rank] = (ms_step, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_is_max_over_ranks():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms_step, rate = res[rank]
        assert ms_step == pytest.approx(100.0)          # 500 ms / 5 steps, the slow rank
        assert rate == pytest.approx(world * 1e3 / 100.0)


def test_replica_rate_single_process():
    import bench
    assert bench.replica_rate(200.0, 4, 1) == (50.0, 20.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm prints from rank 0 only; other ranks exit 0 at
    once without work."""
    import argparse

    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(cpu_iters=1, assume_iters=10, warmup=0, steps=1, workload="sc4_w8")
    assert bench.run_reference_arm(args, bench.WORKLOADS["sc4_w8"]) == 0
    assert capsys.readouterr().out == ""
