"""The N>1 path of bench.py on CPU: world_size-2 `gloo` ranks. The bake does not shard (each GPU
bakes its own replica of the workload), so the only cross-rank steps are the barrier and the
reduction of the timing: whole-job voxels/s = the sum of every rank's voxels over the slowest rank's
seconds. The reference arm runs on rank 0 alone; other ranks exit without work."""
from __future__ import annotations

import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        red_max, red_sum = bench.reducers(dist, "cpu")
        dist.barrier()
        # rank r bakes (r + 1) * 1000 voxels in (1 + r) seconds
        value, secs = bench.aggregate(1000.0 * (rank + 1), 1.0 + rank, red_max, red_sum)
        dist.barrier()
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"value": value, "secs": secs}, f)
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregate_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        got = json.load(open(tmp_path / f"rank{r}.json"))
        assert got["secs"] == pytest.approx(2.0)             # slowest rank
        assert got["value"] == pytest.approx(3000.0 / 2.0)   # all ranks' voxels / slowest time


def test_single_rank_aggregate_is_local():
    sys.path.insert(0, ROOT)
    import bench
    red_max, red_sum = bench.reducers(None, "cpu")
    assert bench.aggregate(500.0, 2.0, red_max, red_sum) == (250.0, 2.0)


def test_reference_arm_runs_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    args = bench.parse(["--impl", "reference", "--steps", "1", "--warmup", "0"])
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
