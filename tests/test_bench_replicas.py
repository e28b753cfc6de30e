"""Multi-GPU runs of this path are replicas only (one independent H.v per rank, no exchange): the
bench's per-rank time is the max over ranks and the job's throughput the sum of the replicas'.
Checked here on CPU with two gloo ranks (no GPU involved)."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = [10.0, 25.0][rank]
    out[rank] = bench.reduce_max(ms, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_time_is_max_over_ranks_and_value_sums():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0] == out[1] == 25.0
    per = 2 ** 32 * 16
    assert bench.replicas_gbs(per, world, 25.0) == pytest.approx(2 * per / 25e-3 / 1e9)
