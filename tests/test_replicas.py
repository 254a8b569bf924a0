"""Multi-GPU path of bench.py (replicas: one process per GPU, each on its own shard of
instances, gloo only for the barrier and the max-over-ranks time), exercised with
world_size 2 on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    local_seconds = 1.0 + rank          # rank 1 is the slow one
    job_seconds = bench.max_over_ranks(local_seconds, world)
    rate = bench.job_rate(100, 5, world, job_seconds)
    _, _, vals = bench.workload(rank)
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.txt").write_text(f"{job_seconds} {rate} {float(vals[0].sum())!r}")


def test_replica_timing_and_shards_with_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [Path(tmp_path, f"rank{r}.txt").read_text().split() for r in range(world)]
    for job_seconds, rate, _ in res:
        assert float(job_seconds) == 2.0                    # max over ranks
        assert float(rate) == pytest.approx(100 * 5 * 2 / 2.0)
    assert res[0][2] != res[1][2]                           # distinct instance shards


def test_select_device_picks_the_local_rank_gpu(monkeypatch):
    import bench
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    assert bench.select_device(3) == "3"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    assert bench.select_device(1) == "5"
