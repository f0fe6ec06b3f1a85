"""Multi-rank logic of bench.py on CPU: two gloo ranks stand in for two GPUs.

Rays shard with no exchange, so `bench.py --gpus N` runs N replicas; the only
cross-rank step is the max over ranks of the timed region.  These tests check
that step and the whole-job value with world size 2, and that the reference
arm prints from rank 0 only.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
        total = bench.reduce_max(local_ms, dist, "cpu")
        ms_step, per_s = bench.whole_job(total, 10, 1_000_000, world)
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"total": total, "ms_step": ms_step, "per_s": per_s}, f)


def test_max_over_ranks_gloo(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    for r in res:
        assert r["total"] == 150.0  # every rank sees the slowest rank's time
        assert r["ms_step"] == 15.0
        assert r["per_s"] == pytest.approx(1_000_000 * world / 0.015)


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(3.5) == 3.5
    ms, per_s = bench.whole_job(80.0, 4, 2_000, 1)
    assert ms == 20.0 and per_s == pytest.approx(100_000.0)


def test_reference_arm_prints_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
