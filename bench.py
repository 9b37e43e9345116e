#!/usr/bin/env python
"""Benchmark of the GB300 mesh -> SDF bake.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batch64|c1|c2|c3|sparse] [--serve-seconds S] [--no-serve] [--no-configs]

Workloads (seeded synthetic meshes generated in-process; no dataset is involved):

* ``batch64`` (default): 64 meshes, triangle counts log-uniform in [1e3, 1e6] (displaced icospheres
  and tori), grids drawn uniformly from {32, 64, 128, 256}^3 over [-0.5, 0.5]^3, exact parity sign,
  occupancy on. One step = the whole batch baked by one call (sdfb_bake_batch_device: one BVH
  build, one persistent distance launch over every mesh's tiles, replayed from a CUDA graph).
  ``value`` is voxels/s of that step with meshes and outputs in HBM; ``plain`` times the same 64
  meshes through 64 single-mesh calls (sdfb_bake_device) in the same run.
* ``c1``: the plain-bake UV sphere (r 0.4, 64 x 32 segments, 4,096 triangles, 128 of them degenerate
  at the poles) on a 64^3 grid, parity sign.
* ``c2`` (alias ``displaced-sphere-256``): the level-6 displaced icosphere (81,920 triangles) on a
  256^3 grid, parity sign.
* ``c3``: the 500k-triangle soup (displaced spheres and tori, 2% of faces deleted) on a 512^3 grid,
  FP32 distance, winding-number sign with FP64 inside the one-voxel band.
  For c1-c3 a step is one single-mesh bake (through the batch entry point, a batch of one).
* ``sparse``: a side workload for the sparse voxelizer (voxelizeMesh's cell list): the 1M-triangle
  displaced torus at resolution 512 through sdfb_voxelize_sparse, grid cells/s (a short line of
  its own, without the headline's keys).

The default line also carries ``configs``: for c1, c2 and c3 the single-mesh GPU bake time and
voxels/s (device buffers, and end to end from host buffers), max and RMS distance error over the
grid diagonal against the FP64 oracle (every cell for c1 and c2; for c3 the cells within 1.5 voxels
of the surface plus a seeded uniform sample of 10^6 cells), out-of-band sign mismatches (exact
parity on every cell; for c3 the FP64 winding number summed directly over every triangle on 4,096
uniform cells), occupancy mismatches on every cell, and the CPU bake of the same mesh timed in the
same run. ``batch_classes`` times the batch's meshes grouped by grid size, plain against batched.

Also reported: ``served`` -- a Poisson stream (200 requests/s for --serve-seconds, default 60) of
meshes drawn as in batch64 (30% of requests repeat an earlier mesh, the rest bring a new one) fed
to the serving loop under a 150 GB budget, with voxels/s and p50/p99 latency (arrival to
completion), beside the same stream's first seconds served by plain per-request bakes, and
(``served.light``) a 60 requests/s stream for up to 30 s, a load one GPU keeps up with;
``single_mesh`` -- the 256^3 displaced-sphere bake; ``roofline`` of the distance kernel (FP32
CUDA-core work: algorithmic flops per launch from the counting build of the same kernel over the
kernel's CUDA-event time, against a cuBLAS SGEMM measured in this run); ``cpu_baseline`` -- the
CPU bake (the reference's own SAT occupancy where it was compiled, else the oracle's restatement;
FP64 distance and exact parity from the oracle on all host threads) on a bounded sample.

Timing: W >= 3 untimed warm-up steps; CUDA events on the bake's stream; a 512 MB L2 flush
before every timed step; nvidia-smi clocks sampled during the timed region. Multi-GPU
(torchrun): every rank bakes its own replica (the bake has no exchange step); ``value`` sums all
ranks' voxels over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import queue
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "italy-rs_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SDF bake voxels/s & p99 latency, served vs plain, 1 GB300, err<=1e-5*diag"
L2_FLUSH_BYTES = 512 << 20


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="batch64", choices=["batch64", "c1", "c2", "c3", "displaced-sphere-256", "sparse"])
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    a = ap.parse_args(argv)
    if a.workload == "displaced-sphere-256":
        a.workload = "c2"
    return a


_T0 = time.monotonic()


def stage(name: str):
    """Progress on stderr (stdout carries only the result line)."""
    print(f"[bench {time.monotonic() - _T0:8.1f} s] {name}", file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def reducers(pg, device):
    """(max, sum) over ranks of one host float, through process group module `pg` (None: one rank)."""
    import torch

    def red(x, op):
        if not pg:
            return x
        t = torch.tensor([x], device=device, dtype=torch.float64)
        pg.all_reduce(t, op=op)
        return float(t.item())

    return (lambda x: red(x, pg.ReduceOp.MAX if pg else None)), (lambda x: red(x, pg.ReduceOp.SUM if pg else None))


def aggregate(voxels_per_rank: float, seconds_per_rank: float, all_reduce_max=None, all_reduce_sum=None):
    """Whole-job throughput: the sum of every rank's voxels over the slowest rank's time."""
    secs = all_reduce_max(seconds_per_rank) if all_reduce_max else seconds_per_rank
    vox = all_reduce_sum(voxels_per_rank) if all_reduce_sum else voxels_per_rank
    return vox / secs, secs


# ---------------------------------------------------------------------------------------------
# Workloads


def batch64_meshes():
    from sdfb import meshgen as mg
    return mg.batch_meshes(64, seed=2024)


def sphere256():
    from sdfb import meshgen as mg
    v, i = mg.displaced_sphere_mesh(seed=1234)
    return v, i, 256


CONFIG_NAMES = {
    "c1": "plain-bake UV sphere (4,096 triangles, 128 degenerate), 64^3, parity",
    "c2": "displaced icosphere level 6 (81,920 triangles), 256^3, parity",
    "c3": "500k-triangle soup (2% of faces deleted), 512^3, FP32 distance + winding number (FP64 band)",
}


def config_mesh(name):
    """(verts, idx, n, sign) of a single-mesh config."""
    from sdfb import meshgen as mg
    if name == "c1":
        v, i = mg.uv_sphere_mesh(0.4, 64, 32)
        return v, i, 64, "parity"
    if name == "c2":
        v, i, n = sphere256()
        return v, i, n, "parity"
    v, i = mg.soup_with_holes()
    return v, i, 512, "gwn"


def workload_meshes(name):
    if name == "batch64":
        return batch64_meshes(), "parity"
    v, i, n, sign = config_mesh(name)
    return [(v, i, n)], sign


def unit_grid(sdfb, n):
    return sdfb.make_grid((-0.5, -0.5, -0.5), 1.0 / n, (n, n, n))


# ---------------------------------------------------------------------------------------------
# Clocks


class ClockSampler:
    """nvidia-smi samples every 200 ms while a timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(pw) if pw else None}


# ---------------------------------------------------------------------------------------------
# CPU baseline (the reference's CPU occupancy code + the FP64 oracle)


def cpu_bake(orc, ref, v, i, n):
    """One CPU bake of mesh (v, i) on the n^3 unit grid; returns (seconds, FP64 unsigned distance,
    exact parity sign)."""
    from oracle.oracle import soup_of
    origin, voxel, dims = (-0.5, -0.5, -0.5), 1.0 / n, (n, n, n)
    soup = soup_of(v, i) if ref is not None else None
    t0 = time.perf_counter()
    if ref is not None:
        ref.occupancy(soup, origin, voxel, dims)
    else:
        orc.occupancy(v, i, origin, voxel, dims)
    d = orc.distance(v, i, origin, voxel, dims)
    s = orc.sign_parity(v, i, origin, voxel, dims, axis=2)
    (d * s).astype("float32")
    return time.perf_counter() - t0, d, s


def cpu_tools():
    from oracle.oracle import Oracle
    orc = Oracle()
    ref, kind = None, "port"
    try:
        from oracle import build_oracle
        if os.path.exists(build_oracle.REF_SO):
            from oracle.oracle import Reference
            ref = Reference(build_oracle.REF_SO)
            kind = "reference"
    except Exception:
        ref = None
    return orc, ref, kind


def cpu_sample(meshes, budget_s, seed, orc, ref, check=None):
    """CPU bakes of the workload's meshes in a seeded order until about budget_s seconds; check(k,
    d, s), when given, sees each baked mesh's result (outside the timing). Returns (voxels,
    seconds, meshes used)."""
    import numpy as np
    order = np.random.default_rng(seed).permutation(len(meshes))
    vox, secs, used = 0, 0.0, 0
    for k in order:
        v, i, n = meshes[k]
        est = n ** 3 * 1.5e-6 * max(1.0, math.log2(max(len(i), 2)) / 17)  # skip bakes far over budget
        if used and secs + est > budget_s * 1.5:
            continue
        dt, d, sg = cpu_bake(orc, ref, v, i, n)
        secs += dt
        vox += n ** 3
        used += 1
        if check is not None:
            check(k, d, sg)
        if secs >= budget_s:
            break
    return vox, secs, used


def cpu_baseline(meshes, budget_s=20.0, seed=0, gpu_grids=None):
    """The CPU baseline; given the GPU's signed grids of the same meshes (gpu_grids[k]) it also
    reports their error against the CPU bake of every sampled mesh, on every cell."""
    import numpy as np
    orc, ref, kind = cpu_tools()
    stats = {"max": 0.0, "sq": 0.0, "cells": 0, "sign_far_mismatch": 0, "meshes": 0}

    def check(k, d, sg):
        n = meshes[k][2]
        got = np.asarray(gpu_grids[k], np.float32).reshape(-1)
        err = np.abs(np.abs(got.astype(np.float64)) - d) / np.sqrt(3.0)
        stats["max"] = max(stats["max"], float(err.max()))
        stats["sq"] += float((err ** 2).sum())
        stats["cells"] += err.size
        far = d > 1.0 / n
        stats["sign_far_mismatch"] += int(np.count_nonzero((got[far] < 0) != (sg[far] < 0)))
        stats["meshes"] += 1

    vox, secs, used = cpu_sample(meshes, budget_s, seed, orc, ref, check if gpu_grids is not None else None)
    precision = None
    if gpu_grids is not None and stats["cells"]:
        precision = {"max_err_over_diag": stats["max"], "rms_err_over_diag": math.sqrt(stats["sq"] / stats["cells"]),
                     "cells": stats["cells"], "meshes": stats["meshes"],
                     "sign_mismatches_outside_1_voxel": stats["sign_far_mismatch"],
                     "reference": "FP64 oracle distance and exact parity on every cell of the sampled meshes"}
    return {"value": vox / secs, "unit": "voxels/s", "cores": orc.threads(), "kind": kind, "precision": precision,
            "sample": f"{used} of the workload's meshes in seeded order, {vox} voxels, {secs:.1f} s "
                      f"(occupancy: {'the reference triBoxOverlap' if kind == 'reference' else 'oracle port'}, 1 thread;"
                      f" FP64 distance + exact parity: {orc.threads()} threads)"}


def cpu_gwn_step(orc, ref, v, i, n, seed, n_dist=100_000, n_gwn=256):
    """One reference-arm step on a winding-number config: (cells, estimated CPU seconds for every
    cell) from occupancy of every cell plus sampled FP64 distance and direct winding number."""
    import numpy as np
    from oracle.oracle import soup_of
    origin, voxel, dims = (-0.5, -0.5, -0.5), 1.0 / n, (n, n, n)
    cells = n ** 3
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    if ref is not None:
        ref.occupancy(soup_of(v, i), origin, voxel, dims)
    else:
        orc.occupancy(v, i, origin, voxel, dims)
    t_occ = time.perf_counter() - t0
    sd = np.sort(rng.choice(cells, n_dist, replace=False)).astype(np.int64)
    t0 = time.perf_counter()
    orc.distance(v, i, origin, voxel, dims, samples=sd)
    t_d = time.perf_counter() - t0
    sw = np.sort(rng.choice(cells, n_gwn, replace=False)).astype(np.int64)
    t0 = time.perf_counter()
    orc.gwn(v, i, origin, voxel, dims, samples=sw)
    t_w = time.perf_counter() - t0
    return cells, t_occ + (t_d / n_dist + t_w / n_gwn) * cells


def run_reference(args, rank, world):
    """The reference arm: the CPU bake of the workload (the reference's own bake of this path is an
    OptiX ray-cast estimate and the OptiX SDK is absent, so its CPU occupancy code and the FP64
    oracle stand in). Each step bakes meshes of the workload in a seeded order for a bounded time."""
    if rank != 0:
        return
    meshes, sign = workload_meshes(args.workload)
    orc, ref, kind = cpu_tools()
    budget = max(5.0, min(25.0, 150.0 / max(args.steps, 1)))
    vox, secs, used = 0, 0.0, 0
    if sign == "gwn":
        # the 512^3 soup: each step times occupancy on every cell and distance + direct winding
        # number on a seeded sample of cells, and counts the whole grid at that per-cell cost
        v, i, n = meshes[0]
        for step in range(args.steps):
            a, b = cpu_gwn_step(orc, ref, v, i, n, step)
            vox, secs, used = vox + a, secs + b, used + 1
        what = ("occupancy of every cell + FP64 distance on 10^5 and direct FP64 winding number on 256 sampled "
                "cells, each step's per-cell cost scaled to the whole grid")
    else:
        for w in range(min(args.warmup, 1)):
            cpu_sample(meshes, 1.0, 1000 + w, orc, ref)
        for step in range(args.steps):
            a, b, c = cpu_sample(meshes, budget, step, orc, ref)
            vox, secs, used = vox + a, secs + b, used + c
        what = f"{used} mesh bakes over {args.steps} steps of ~{budget:.0f} s, {vox} voxels"
    value = vox / secs if secs else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload},
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": orc.threads(), "kind": kind,
                             "sample": what},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU arm


def hbm_peak_gbs():
    """The measured copy bandwidth of this GPU model (MEASURED_PEAKS.json beside this file), else
    the fallback figure."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def traffic_record(workload: str):
    """DRAM bytes of one distance launch of this workload from the committed ncu capture
    (profiles/traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            rec = json.load(f).get(workload)
        return None if rec is None else {**rec, "bytes": rec["dram_read_bytes"] + rec["dram_write_bytes"]}
    except (OSError, ValueError, KeyError):
        return None


def sgemm_peak(torch) -> float:
    """FP32 CUDA-core peak measured as cuBLAS SGEMM (TF32 off), TFLOP/s, best of 5."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def new_stats(sdfb):
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    return st


def percentile(xs, p):
    if not xs:
        return None
    ys = sorted(xs)
    k = min(len(ys) - 1, max(0, int(math.ceil(p / 100.0 * len(ys))) - 1))
    return ys[k]


_SLOT_BUFS: list = []


def serve_stream(sdfb, ctx, torch, base_meshes, seconds, seed=77, rate=200.0, repeat=0.3, workers=128,
                 wave_log2=28, max_inflight=128, closed_loop=False):
    """The Poisson serving stream. Returns the served record and the request list (for plain).
    closed_loop: no arrival times -- each of the `workers` clients submits its next request as soon
    as its last one returns, for `seconds` (the server's capacity at that concurrency); latency is
    then measured from submission."""
    import numpy as np
    rng = np.random.default_rng(seed)
    reqs, t, news = [], 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        n = int(rng.choice([32, 64, 128, 256]))
        if news and rng.uniform() < repeat:
            key = news[int(rng.integers(len(news)))]
        else:
            key = (int(rng.integers(len(base_meshes))), tuple(rng.uniform(-0.03, 0.03, 3).astype(np.float32)))
            news.append(key)
        reqs.append((t, key, n))
    # pinned output slots, sized for the largest grid (allocated once, shared by the streams)
    max_cells = 256 ** 3
    slots = queue.Queue()
    while len(_SLOT_BUFS) < workers:
        _SLOT_BUFS.append((torch.empty(max_cells, dtype=torch.float32).pin_memory().numpy(),
                           torch.empty(max_cells, dtype=torch.uint8).pin_memory().numpy()))
    slot_bufs = _SLOT_BUFS[:workers]
    for k in range(workers):
        slots.put(k)
    results = [None] * len(reqs)
    srv = sdfb.Server(ctx, hbm_budget_bytes=150 << 30, max_inflight=max_inflight, wave_voxels_log2=wave_log2)
    mesh_cache = {}
    lock = threading.Lock()
    work = queue.Queue()

    def mesh_of(key):
        b, off = key
        v, f, _ = base_meshes[b]
        return (v + np.asarray(off, np.float32)).astype(np.float32), f

    failures = []
    dropped = []
    deadline = [float("inf")]  # requests not started by then are dropped (reported, never timed)

    def worker():
        while True:
            item = work.get()
            if item is None:
                return
            k, arrival = item
            if closed_loop:
                arrival = time.monotonic()
            if time.monotonic() > deadline[0]:
                with lock:
                    dropped.append(k)
                continue
            _, key, n = reqs[k]
            v, f = mesh_of(key)
            slot = slots.get()
            try:
                d, o = slot_bufs[slot]
                g = unit_grid(sdfb, n)
                cells = g.cells
                for attempt in range(3):  # a mesh evicted between register and submit is registered again
                    mid = srv.register(v, f)
                    try:
                        rid = srv.submit(mid, g, d[:cells], o[:cells])
                        break
                    except sdfb.SdfbError as e:
                        if e.status != sdfb.ERR_NOT_FOUND or attempt == 2:
                            raise
                done, info = srv.poll(rid, 120000)
                if not done:
                    raise RuntimeError(f"request {k} not done after 120 s")
                results[k] = (arrival, info["t_submit_ms"] / 1e3, info["t_done_ms"] / 1e3, cells, info["status"])
            except Exception as e:  # recorded and reported; the stream goes on
                with lock:
                    failures.append(f"{type(e).__name__}: {e}")
            finally:
                slots.put(slot)

    threads = [threading.Thread(target=worker, daemon=True) for _ in range(workers)]
    for th in threads:
        th.start()
    watching = [True]

    def watch():  # progress on stderr every 10 s
        while watching[0]:
            time.sleep(10.0)
            n_done = sum(1 for r in results if r)
            stage(f"  serving: {n_done} done, {len(failures)} failed, {len(dropped)} dropped, "
                  f"{work.qsize()} queued")

    threading.Thread(target=watch, daemon=True).start()
    # warm the server (first-wave allocations) with one small request outside the stream
    v0, f0, _ = base_meshes[0]
    g0 = unit_grid(sdfb, 32)
    d0, o0 = slot_bufs[0]
    srv.poll(srv.submit(srv.register(v0, f0), g0, d0[:g0.cells], o0[:g0.cells]), 120000)
    t0 = time.monotonic()
    deadline[0] = t0 + (seconds if closed_loop else seconds + max(60.0, seconds))
    for k, (arr, key, n) in enumerate(reqs):
        now = time.monotonic() - t0
        if arr > now and not closed_loop:
            time.sleep(arr - now)
        work.put((k, t0 + arr))
    for _ in threads:
        work.put(None)
    for th in threads:
        th.join()
    watching[0] = False
    srv.close()
    if failures:
        print(f"serve_stream: {len(failures)} requests failed, first: {failures[0]}", file=sys.stderr)
    if dropped:
        print(f"serve_stream: {len(dropped)} requests dropped at the drain deadline", file=sys.stderr)
    lat = [r[2] - r[0] for r in results if r]
    done = [r for r in results if r and r[4] == 0]
    if not done:
        raise RuntimeError(f"serve_stream: no request completed ({len(failures)} failed)")
    span = max(r[2] for r in done) - t0
    vox = sum(r[3] for r in done)
    return {"requests": len(reqs), "completed": len(done), "failed": len(failures), "dropped": len(dropped),
            "new_meshes": len(news),
            "voxels_per_s": vox / span, "p50_ms": 1e3 * percentile(lat, 50), "p99_ms": 1e3 * percentile(lat, 99),
            "mean_ms": 1e3 * statistics.mean(lat), "seconds": span, "rate_per_s": rate, "repeat_fraction": repeat,
            "hbm_budget_gb": 150}, reqs


def plain_stream(sdfb, ctx, base_meshes, reqs, seconds):
    """The same stream served by plain per-request bakes (one at a time, in arrival order) for the
    arrivals of the first `seconds`."""
    import numpy as np
    sub = [r for r in reqs if r[0] < seconds]
    lat, vox = [], 0
    t0 = time.monotonic()
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO)
    limit = max(60.0, 6 * seconds)  # wall-clock cap; requests not reached by then are not counted
    done = 0
    for arr, (b, off), n in sub:
        now = time.monotonic() - t0
        if now > limit:
            break
        if arr > now:
            time.sleep(arr - now)
        v, f, _ = base_meshes[b]
        v = (v + np.asarray(off, np.float32)).astype(np.float32)
        g = unit_grid(sdfb, n)
        ctx.bake(v, f, g, opts)
        lat.append(time.monotonic() - t0 - arr)
        vox += g.cells
        done += 1
    span = time.monotonic() - t0
    return {"requests": len(sub), "completed": done, "voxels_per_s": vox / span, "p50_ms": 1e3 * percentile(lat, 50),
            "p99_ms": 1e3 * percentile(lat, 99), "seconds": span,
            "note": f"arrivals of the first {seconds:.0f} s of the same stream, one sdfb_bake per request"}


# ---------------------------------------------------------------------------------------------
# Per-config records (c1-c3): GPU time, FP64 precision, mismatches, CPU bake of the same mesh


def gpu_single(sdfb, ctx, torch, stream, flush, v, i, n, sign, reps=5):
    """Single-mesh bake on device buffers (sdfb_bake_device), median of `reps` timed bakes after two
    warm-ups, plus the same bake end to end from host buffers (sdfb_bake, pinned outputs). Returns
    (record, signed distances, occupancy) as host arrays."""
    import numpy as np
    g = unit_grid(sdfb, n)
    mode = sdfb.SIGN_PARITY if sign == "parity" else sdfb.SIGN_GWN
    opts = sdfb.make_opts(sign_mode=mode)
    dv, di = torch.from_numpy(v).cuda(), torch.from_numpy(i.astype(np.int32)).cuda()
    dd = torch.empty(g.cells, dtype=torch.float32, device="cuda")
    do = torch.empty(g.cells, dtype=torch.uint8, device="cuda")

    def bake(st=None):
        ctx.bake_device(dv.data_ptr(), len(v), di.data_ptr(), len(i), g, opts, dd.data_ptr(), do.data_ptr(),
                        stream.cuda_stream, st)

    for _ in range(2):
        bake()
    ms, st = [], None
    for _ in range(reps):
        flush.fill_(1.0)
        st = new_stats(sdfb)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bake(st)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    hd = torch.empty(g.cells, dtype=torch.float32).pin_memory().numpy().reshape(g.shape)
    ho = torch.empty(g.cells, dtype=torch.uint8).pin_memory().numpy().reshape(g.shape)
    ctx.bake(v, i, g, opts, out=(hd, ho))
    e2e = []
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.bake(v, i, g, opts, out=(hd, ho))
        e2e.append(time.perf_counter() - t0)
    med = statistics.median(ms)
    rec = {"triangles": int(len(i)), "voxels": int(g.cells), "grid": n, "sign": sign, "gpu_ms": med,
           "voxels_per_s": g.cells / (med * 1e-3), "e2e_ms": 1e3 * statistics.median(e2e),
           "e2e_voxels_per_s": g.cells / statistics.median(e2e),
           "stages_ms": {"build": st.ms_build, "occupancy": st.ms_occupancy, "sign": st.ms_sign,
                         "distance": st.ms_distance},
           "gwn_fp64_cells": int(st.gwn_fp64_cells) if sign == "gwn" else None}
    gpu_d = dd.cpu().numpy().reshape(g.shape) if sign == "parity" else hd.copy()
    gpu_o = do.cpu().numpy().reshape(g.shape)
    if sign == "gwn":
        gpu_o = ho.copy()
    del dv, di, dd, do
    return rec, gpu_d, gpu_o


def cpu_check(name, v, i, n, sign, gpu_d, gpu_o, seed=5):
    """The CPU bake of a config's mesh, timed, and the GPU grid's error against it. c1 and c2 are
    baked on every cell (occupancy: the reference's own code where compiled, one thread; FP64
    distance and exact parity: the oracle on all host threads). c3 compares every cell's
    occupancy, FP64 distance on the cells within 1.5 voxels of the surface and on a uniform sample
    of 10^6 cells, and the FP64 winding number summed over every triangle on 4,096 uniform cells;
    its CPU rate is the occupancy of every cell plus distance and winding number per sampled cell,
    scaled to the whole grid."""
    import numpy as np
    from oracle.oracle import soup_of
    orc, ref, kind = cpu_tools()
    origin, voxel, dims = (-0.5, -0.5, -0.5), 1.0 / n, (n, n, n)
    cells = n ** 3
    diag = math.sqrt(3.0)
    t0 = time.perf_counter()
    occ = ref.occupancy(soup_of(v, i), origin, voxel, dims) if ref is not None else orc.occupancy(v, i, origin, voxel, dims)
    t_occ = time.perf_counter() - t0
    occ_bad = int(np.count_nonzero(np.asarray(occ).reshape(-1) != gpu_o.reshape(-1)))
    got = gpu_d.reshape(-1).astype(np.float64)
    out = {"occupancy_mismatches": occ_bad, "occupancy_cells_compared": cells}
    if sign == "parity":
        t0 = time.perf_counter()
        d64 = orc.distance(v, i, origin, voxel, dims)
        sg = orc.sign_parity(v, i, origin, voxel, dims, axis=2)
        t_ds = time.perf_counter() - t0
        err = np.abs(np.abs(got) - d64) / diag
        far = d64 > voxel
        out.update({"max_err_over_diag": float(err.max()), "rms_err_over_diag": float(np.sqrt(np.mean(err ** 2))),
                    "distance_cells_compared": cells, "compared": "every cell",
                    "sign_mismatches_outside_1_voxel": int(np.count_nonzero((got[far] < 0) != (sg[far] < 0))),
                    "sign_cells_compared": int(np.count_nonzero(far)),
                    "sign_reference": "exact +z parity (oracle)"})
        cpu_s = t_occ + t_ds
        what = "every cell"
    else:
        rng = np.random.default_rng(seed)
        band = np.flatnonzero(np.abs(got) <= 1.5 * voxel).astype(np.int64)
        uni = np.sort(rng.choice(cells, 1_000_000, replace=False)).astype(np.int64)
        t0 = time.perf_counter()
        d_uni = orc.distance(v, i, origin, voxel, dims, samples=uni)
        t_du = time.perf_counter() - t0
        d_band = orc.distance(v, i, origin, voxel, dims, samples=band)
        e_uni = np.abs(np.abs(got[uni]) - d_uni) / diag
        e_band = np.abs(np.abs(got[band]) - d_band) / diag
        err = np.concatenate([e_uni, e_band])
        ws = np.sort(rng.choice(uni, 4096, replace=False)).astype(np.int64)
        t0 = time.perf_counter()
        w = orc.gwn(v, i, origin, voxel, dims, samples=ws)
        t_w = time.perf_counter() - t0
        d_ws = orc.distance(v, i, origin, voxel, dims, samples=ws)
        far = (d_ws > voxel) & (np.abs(np.abs(w) - 0.5) > 1e-6)
        bad = int(np.count_nonzero((got[ws][far] < 0) != (np.abs(w[far]) > 0.5)))
        out.update({"max_err_over_diag": float(err.max()), "rms_err_over_diag": float(np.sqrt(np.mean(err ** 2))),
                    "distance_cells_compared": int(err.size),
                    "compared": f"{band.size} cells within 1.5 voxels of the surface + a seeded uniform sample "
                                f"of {uni.size} cells",
                    "sign_mismatches_outside_1_voxel": bad, "sign_cells_compared": int(np.count_nonzero(far)),
                    "sign_reference": "FP64 winding number summed over every triangle (oracle), 4,096 uniform cells"})
        cpu_s = t_occ + (t_du / uni.size + t_w / ws.size) * cells
        what = (f"occupancy of every cell ({t_occ:.1f} s) + FP64 distance ({1e6 * t_du / uni.size:.2f} us/cell on "
                f"{uni.size} cells) and direct FP64 winding number ({1e3 * t_w / ws.size:.2f} ms/cell on {ws.size} "
                f"cells), scaled to {cells} cells")
    out["cpu"] = {"seconds": cpu_s, "voxels_per_s": cells / cpu_s, "cores": orc.threads(), "kind": kind,
                  "what": what + (" (occupancy: the reference's triBoxOverlap, 1 thread)" if kind == "reference"
                                  else " (occupancy: oracle port, 1 thread)")}
    return out


def config_record(name, sdfb, ctx, torch, stream, flush, cpu=True):
    v, i, n, sign = config_mesh(name)
    rec, gd, go = gpu_single(sdfb, ctx, torch, stream, flush, v, i, n, sign)
    rec = {"workload": CONFIG_NAMES[name], **rec}
    if cpu:
        rec.update(cpu_check(name, v, i, n, sign, gd, go))
        rec["gpu_over_cpu"] = rec["voxels_per_s"] / rec["cpu"]["voxels_per_s"]
    return rec


def batch_classes(sdfb, ctx, torch, stream, flush, devm, grids, dptr, optr, opts, meshes, reps=3):
    """The batch's meshes grouped by grid size: per group the plain time (one sdfb_bake_device per
    mesh, summed) and the batched time (the group as one batch), in ms."""
    out = {}
    for n in sorted({m[2] for m in meshes}):
        ks = [k for k, m in enumerate(meshes) if m[2] == n]

        def plain():
            for k in ks:
                ctx.bake_device(devm[k][0], devm[k][1], devm[k][2], devm[k][3], grids[k], opts, dptr[k], optr[k],
                                stream.cuda_stream)

        def batched():
            ctx.bake_batch_device([devm[k] for k in ks], [grids[k] for k in ks], opts, [dptr[k] for k in ks],
                                  [optr[k] for k in ks], stream.cuda_stream)

        res = {}
        for label, fn in (("plain_ms", plain), ("batched_ms", batched)):
            fn()
            fn()
            t = []
            for _ in range(reps):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                e1.synchronize()
                t.append(e0.elapsed_time(e1))
            res[label] = statistics.median(t)
        vox = sum(grids[k].cells for k in ks)
        out[f"{n}^3"] = {"meshes": len(ks), "triangles": int(sum(len(meshes[k][1]) for k in ks)), "voxels": int(vox),
                         **res, "batched_over_plain": res["plain_ms"] / res["batched_ms"]}
    return out


def sparse_main(args):
    """voxelizeMesh's sparse cell list (sdfb_voxelize_sparse) of the 1M-triangle displaced torus at
    resolution 512 (134 M grid cells): occupancy, per-tile compaction and the insertion-order sort,
    timed end to end through the host entry point (soup up, cell list down), median of the steps.
    A side workload for the compaction kernels, not the headline line."""
    import numpy as np
    import torch

    import sdfb
    from sdfb import meshgen as mg

    ctx = sdfb.Context(0)
    v, f = mg.displaced_torus(1024, 512, 0.3, 0.1, 1114)
    soup = np.ascontiguousarray(np.asarray(v, np.float32)[np.asarray(f, np.int64)].reshape(-1, 3))
    bmin, bmax = soup.min(0), soup.max(0)
    res = 512
    stage(f"sparse: {len(f)} triangles, resolution {res}")
    for _ in range(max(args.warmup, 1)):
        cells, _, _ = ctx.voxelize_sparse(soup, bmin, bmax, res)
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cells, _, _ = ctx.voxelize_sparse(soup, bmin, bmax, res)
        times.append(time.perf_counter() - t0)
    times.sort()
    t = times[len(times) // 2]
    print(json.dumps({"metric": "sparse voxelize (voxelizeMesh cell list) grid cells/s", "value": res ** 3 / t,
                      "unit": "cells/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * t, "higher_is_better": True, "dtype": "u8",
                      "data": "synthetic (seeded mesh generated in-process)",
                      "config": {"workload": "sparse", "triangles": int(len(f)), "resolution": res,
                                 "cells_listed": int(len(cells)),
                                 "timing": "host wall clock around sdfb_voxelize_sparse (copies included)"}}),
          flush=True)
    ctx.close()


def main(argv=None):
    args = parse(argv)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "sparse":
        sparse_main(args)
        return
    import numpy as np
    import torch

    import sdfb

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    if not os.path.exists(sdfb.LIB_PATH):
        import build as pkg_build
        pkg_build.build()
    ctx = sdfb.Context(local)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    red_max, red_sum = reducers(pg, "cuda")

    stage("generating meshes")
    meshes, sign = workload_meshes(args.workload)
    stage(f"{len(meshes)} meshes, {sum(len(i) for _, i, _ in meshes)} triangles")
    grids = [unit_grid(sdfb, n) for _, _, n in meshes]
    cells = [g.cells for g in grids]
    total_cells = sum(cells)
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY if sign == "parity" else sdfb.SIGN_GWN)
    dev_v = [torch.from_numpy(v).cuda() for v, _, _ in meshes]
    dev_i = [torch.from_numpy(i.astype(np.int32)).cuda() for _, i, _ in meshes]
    dev_d = [torch.empty(c, dtype=torch.float32, device="cuda") for c in cells]
    dev_o = [torch.empty(c, dtype=torch.uint8, device="cuda") for c in cells]
    devm = [(a.data_ptr(), len(v), b.data_ptr(), len(i)) for a, b, (v, i, _) in zip(dev_v, dev_i, meshes)]
    dptr = [d.data_ptr() for d in dev_d]
    optr = [o.data_ptr() for o in dev_o]

    def step_batch(stats=None, o=opts):
        ctx.bake_batch_device(devm, grids, o, dptr, optr, stream.cuda_stream, stats)

    def step_plain(stats_list=None):
        for k in range(len(meshes)):
            ctx.bake_device(devm[k][0], devm[k][1], devm[k][2], devm[k][3], grids[k], opts, dptr[k], optr[k],
                            stream.cuda_stream, stats_list[k] if stats_list else None)

    stage("warm-up")
    for _ in range(max(args.warmup, 3)):
        step_batch()
    torch.cuda.synchronize()
    cst = new_stats(sdfb)
    stage("counting build")
    count_opts = sdfb.make_opts(sign_mode=opts.sign_mode, count_work=True)
    step_batch(cst, count_opts)  # counting build (untimed)
    stage("timed steps")

    # ---- timed region: the batched bake ----
    clocks = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    step_ms, dist_ms, launches, replayed = [], [], [], []
    for _ in range(args.steps):
        flush.fill_(1.0)
        st = new_stats(sdfb)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_batch(st)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        dist_ms.append(st.ms_distance)
        launches.append(st.kernel_launches)
        replayed.append(st.graph_replayed)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clk = clocks.stop()
    value, secs = aggregate(total_cells * args.steps, sum(step_ms) / 1e3, red_max, red_sum)

    stage(f"batched: {statistics.mean(step_ms):.1f} ms per step")
    # ---- the plain path on the same meshes (single-mesh calls) ----
    for _ in range(2):
        step_plain()
    plain_ms = []
    for _ in range(max(2, args.steps // 3)):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_plain()
        e1.record(stream)
        e1.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    plain_value, _ = aggregate(total_cells * len(plain_ms), sum(plain_ms) / 1e3, red_max, red_sum)

    stage(f"plain: {statistics.mean(plain_ms):.1f} ms per step")
    # ---- e2e: host buffers (pinned) through sdfb_bake_batch ----
    hmeshes = [(torch.from_numpy(v).pin_memory().numpy(),
                torch.from_numpy(i.astype(np.int32)).pin_memory().numpy().view(np.uint32)) for v, i, _ in meshes]
    hd = [torch.empty(c, dtype=torch.float32).pin_memory().numpy().reshape(g.shape) for c, g in zip(cells, grids)]
    ho = [torch.empty(c, dtype=torch.uint8).pin_memory().numpy().reshape(g.shape) for c, g in zip(cells, grids)]
    for _ in range(2):
        ctx.bake_batch(hmeshes, grids, opts, out=(hd, ho))
    e2e_s, e2e_dev_ms = [], []
    for _ in range(max(3, args.steps // 2)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        est = new_stats(sdfb)
        t0 = time.perf_counter()
        ctx.bake_batch(hmeshes, grids, opts, out=(hd, ho), stats=est)
        e2e_s.append(time.perf_counter() - t0)
        e2e_dev_ms.append(est.ms_total)
    e2e_value, _ = aggregate(total_cells * len(e2e_s), sum(e2e_s), red_max, red_sum)
    h2d = int(sum(v.nbytes + i.nbytes for v, i in hmeshes))
    stage(f"e2e: {1e3 * statistics.mean(e2e_s):.1f} ms per step")

    if rank != 0:
        if pg:
            pg.barrier()
            pg.destroy_process_group()
        return

    classes = None
    if args.workload == "batch64":
        classes = batch_classes(sdfb, ctx, torch, stream, flush, devm, grids, dptr, optr, opts, meshes)
        stage("grid-size classes: " + ", ".join(f"{k} {v['batched_over_plain']:.2f}x" for k, v in classes.items()))

    # ---- roofline of the distance kernel ----
    peak = sgemm_peak(torch)
    stage(f"SGEMM peak {peak:.1f} TFLOP/s")
    # as executed (terms a lane shares between its cells counted once), and the previous counting
    # that charges every cell for them (box 11, plane 9, rectangle 16, full test 31 flops)
    flops = float(cst.flops_distance)
    flops_count = (cst.box_tests * 11.0 + cst.plane_tests * 9.0 + cst.rect_tests * 16.0 + cst.tri_tests * 31.0)
    mean_dist_ms = statistics.mean(dist_ms)
    achieved = flops / (mean_dist_ms * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": "k_distance (+ k_distance_deferred)", "flops_per_launch": flops,
                "flops_per_launch_per_cell_count": flops_count,
                "frac_per_cell_count": flops_count / (mean_dist_ms * 1e-3) / 1e12 / peak,
                "box_tests": int(cst.box_tests), "tri_tests": int(cst.tri_tests),
                "plane_tests": int(cst.plane_tests), "rect_tests": int(cst.rect_tests),
                "tiles_deferred": int(cst.tiles_deferred), "tile_used": int(cst.tile_used),
                "kernel_ms": mean_dist_ms,
                "peak_source": "cuBLAS SGEMM 8192^3 FP32 (TF32 off), best of 5, measured in this run",
                "algorithmic_bytes_per_launch": total_cells * 4}
    # the memory side beside it: distance writes plus one read of every mesh's hierarchy
    hbm_peak, hbm_src = hbm_peak_gbs()
    bvh_bytes = sum(len(i) * (80 + 64) for _, i, _ in meshes)  # 80-byte triangle records + 64-byte nodes
    moved = total_cells * 4 + bvh_bytes
    roofline["hbm"] = {"bytes_per_launch": moved, "achieved_gbs": moved / (mean_dist_ms * 1e-3) / 1e9,
                       "peak_gbs": hbm_peak, "frac": moved / (mean_dist_ms * 1e-3) / 1e9 / hbm_peak,
                       "peak_source": hbm_src}
    tr = traffic_record(args.workload)
    if tr is not None:
        # measured DRAM bytes of the pass-A launch (pass B is ~3% of the stage)
        roofline["traffic"] = tr["bytes"]
        roofline["traffic_source"] = f"ncu capture of {tr['kernel']} (profiles/traffic.json)"
        roofline["hbm"]["measured_bytes_per_launch"] = tr["bytes"]

    served = None
    if not args.no_serve and args.workload == "batch64" and world == 1:
        served, reqs = serve_stream(sdfb, ctx, torch, meshes, args.serve_seconds)
        stage(f"served: {served['completed']}/{served['requests']} in {served['seconds']:.1f} s")
        served["plain"] = plain_stream(sdfb, ctx, meshes, reqs, min(10.0, args.serve_seconds))
        stage("plain stream done")
        # the same kind of stream at a rate one GPU keeps up with, for latency without a queue
        light, _ = serve_stream(sdfb, ctx, torch, meshes, min(30.0, args.serve_seconds), seed=78, rate=60.0)
        served["light"] = {k: light[k] for k in ("requests", "completed", "voxels_per_s", "p50_ms", "p99_ms",
                                                 "mean_ms", "rate_per_s")}
        stage(f"light stream: p50 {light['p50_ms']:.0f} ms, p99 {light['p99_ms']:.0f} ms")
        sat, _ = serve_stream(sdfb, ctx, torch, meshes, min(20.0, args.serve_seconds), seed=79, rate=1000.0,
                              closed_loop=True)
        served["saturation"] = {k: sat[k] for k in ("requests", "completed", "dropped", "voxels_per_s", "p50_ms",
                                                    "p99_ms", "mean_ms", "seconds")}
        served["saturation"]["note"] = ("closed loop: 128 clients, each submits its next request when the last "
                                        "one returns; latency from submission")
        stage(f"saturation: {sat['voxels_per_s'] / 1e6:.0f} M voxels/s")

    configs = None
    cpu = precision = None
    if args.workload == "batch64":
        if not args.no_configs:
            configs = {}
            for name in ("c1", "c2", "c3"):
                configs[name] = config_record(name, sdfb, ctx, torch, stream, flush, cpu=not args.no_cpu_baseline)
                stage(f"{name}: {configs[name]['gpu_ms']:.2f} ms"
                      + (f", max error {configs[name]['max_err_over_diag']:.3g} x diag"
                         if 'max_err_over_diag' in configs[name] else ""))
        cpu = None if args.no_cpu_baseline else cpu_baseline(meshes, gpu_grids=hd)
        precision = cpu.pop("precision") if cpu else None
    elif not args.no_cpu_baseline:
        v, i, n, sgn = config_mesh(args.workload)
        # the line's own grid: hd / ho from the e2e leg (a batch of one)
        chk = cpu_check(args.workload, v, i, n, sgn, hd[0], ho[0])
        c = chk.pop("cpu")
        cpu = {"value": c["voxels_per_s"], "unit": "voxels/s", "cores": c["cores"], "kind": c["kind"],
               "sample": c["what"]}
        precision = chk
    stage("CPU baseline done" + (f": max error {precision['max_err_over_diag']:.3g} x diag" if precision else ""))
    cfg = {"workload": args.workload, "meshes": len(meshes), "triangles": int(sum(len(i) for _, i, _ in meshes)),
           "voxels": int(total_cells), "grids": sorted({n for _, _, n in meshes}), "sign": sign,
           "parallelism": f"replicas x{world}",
           "l2": "512 MB L2 flush before every timed step (outputs alone exceed L2)"}
    cfg["seed"] = {"batch64": 2024, "c2": 1234, "c3": 4321}.get(args.workload)
    if args.workload != "batch64":
        cfg["description"] = CONFIG_NAMES[args.workload]
    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(step_ms) / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes generated in-process)",
        "config": cfg,
        "plain": {"value": plain_value, "unit": "voxels/s", "ms_per_step": statistics.mean(plain_ms),
                  "batched_over_plain": value / plain_value},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "voxels/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(total_cells * 5), "ms_per_step": 1e3 * statistics.mean(e2e_s),
                "device_ms_per_step": statistics.mean(e2e_dev_ms)},
        "clocks": clk,
        "gpu_launches": int(sum(launches)),
        "graph_replayed_steps": int(sum(replayed)),
        "precision": precision,
        "served": served,
        "configs": configs,
        "batch_classes": classes,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
