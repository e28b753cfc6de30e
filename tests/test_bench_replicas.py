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


def test_reference_arm_json_line():
    """`bench.py --impl reference` prints one JSON line with the keys of the bench contract: the
    reference's CPU path (the oracle port) timed on a bounded sample of the same workload, its
    config identical to the GPU arm's, and an e2e entry without host/device copies."""
    import json
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--sites", "20",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "GB/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"] == bench.workload_config(20, 1)
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
