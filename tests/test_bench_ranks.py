"""bench.py's N-rank arithmetic on the CPU: two gloo ranks, each timing its own
replica; the job's time is the slowest rank's (max over ranks), and alone (no
process group) a rank's own time is used."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        t = 1.5 + rank  # rank 1 is the slow one
        out[rank] = bench.max_over_ranks(t, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ws, port = 2, _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank, args=(ws, port, out), nprocs=ws, join=True, start_method="spawn")
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_without_process_group_is_identity():
    assert bench.max_over_ranks(3.25, "cpu") == 3.25


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the reference arm's other ranks exit without work."""
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(None) is None
