"""The multi-GPU path is replicas only (rays are independent): each rank
builds and traces its own workload and the only collective is the timing
reduction.  Checked here with world_size-2 gloo process groups on the CPU."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, times, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_env() == (ws, rank, rank)
        ms = bench.replica_step_ms(times[rank], ws, "cpu")
        out[rank] = ms
    finally:
        dist.destroy_process_group()


def test_replica_step_time_is_the_max_over_ranks():
    ws, port = 2, _free_port()
    times = [7.5, 9.25]
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank_main, args=(ws, port, times, out), nprocs=ws, join=True)
    assert out[0] == out[1] == 9.25
    sys.path.insert(0, ROOT)
    import bench
    # weak scaling: every rank traces its own full workload
    assert bench.weak_value(2, 24_862_464, 9.25) == pytest.approx(2 * 24_862_464 / 9.25e-3 / 1e9)
    assert bench.replica_step_ms(7.5, 1, "cpu") == 7.5


def test_reference_arm_runs_on_rank_0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup, cpu_budget = 1, 3, 1.0
    # rank 1 returns at once without building anything
    assert bench.run_reference(Args()) is None
