"""bench.py's host-side pieces that need no GPU: the argument contract, the committed DRAM-traffic
record the roofline reads, and the whole-job aggregation."""
from __future__ import annotations

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_defaults_and_workloads():
    a = bench.parse([])
    assert (a.gpus, a.workload, a.impl) == (1, "batch64", "ours")
    assert a.warmup >= 3 and a.steps >= 1
    assert bench.parse(["--workload", "displaced-sphere-256"]).workload == "c2"
    for w in ("c1", "c2", "c3", "sparse"):
        assert bench.parse(["--workload", w]).workload == w


def test_traffic_records_are_complete():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    with open(path) as f:
        recs = json.load(f)
    for name in ("batch64", "c2"):
        r = bench.traffic_record(name)
        assert r is not None, name
        assert r["bytes"] == recs[name]["dram_read_bytes"] + recs[name]["dram_write_bytes"] > 0
        # the record names the kernel and the ncu command that produced it
        assert "k_distance" in r["kernel"] and "--clock-control none" in r["command"]
    assert bench.traffic_record("no-such-workload") is None


def test_aggregate_is_sum_over_slowest():
    v, secs = bench.aggregate(100.0, 2.0, lambda x: max(x, 4.0), lambda x: x * 2)
    assert secs == 4.0 and v == 50.0
