#!/usr/bin/env python
"""Benchmark of the GB300 mesh -> SDF bake.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batch64|displaced-sphere-256] [--serve-seconds S] [--no-serve]

Workloads (seeded synthetic meshes generated in-process; no dataset is involved):

* ``batch64`` (default): 64 meshes, triangle counts log-uniform in [1e3, 1e6] (displaced icospheres
  and tori), grids drawn uniformly from {32, 64, 128, 256}^3 over [-0.5, 0.5]^3, exact parity sign,
  occupancy on. One step = the whole batch baked by one call (sdfb_bake_batch_device: one BVH
  build, one persistent distance launch over every mesh's tiles, replayed from a CUDA graph).
  ``value`` is voxels/s of that step with meshes and outputs in HBM; ``plain`` times the same 64
  meshes through 64 single-mesh calls (sdfb_bake_device) in the same run.
* ``displaced-sphere-256``: the level-6 displaced icosphere (81,920 triangles) on a 256^3 grid, one
  single-mesh bake per step.

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
    ap.add_argument("--workload", default="batch64", choices=["batch64", "displaced-sphere-256"])
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args(argv)


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


def run_reference(args, rank, world):
    """The reference arm: the CPU bake of the workload (the reference's own bake of this path is an
    OptiX ray-cast estimate and the OptiX SDK is absent, so its CPU occupancy code and the FP64
    oracle stand in). Each step bakes meshes of the workload in a seeded order for a bounded time."""
    if rank != 0:
        return
    meshes = batch64_meshes() if args.workload == "batch64" else [sphere256()]
    orc, ref, kind = cpu_tools()
    budget = max(5.0, min(25.0, 150.0 / max(args.steps, 1)))
    for w in range(min(args.warmup, 1)):
        cpu_sample(meshes, 1.0, 1000 + w, orc, ref)
    vox, secs, used = 0, 0.0, 0
    for step in range(args.steps):
        a, b, c = cpu_sample(meshes, budget, step, orc, ref)
        vox, secs, used = vox + a, secs + b, used + c
    value = vox / secs if secs else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload},
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": orc.threads(), "kind": kind,
                             "sample": f"{used} mesh bakes over {args.steps} steps of ~{budget:.0f} s, {vox} voxels"},
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


def serve_stream(sdfb, ctx, torch, base_meshes, seconds, seed=77, rate=200.0, repeat=0.3, workers=64,
                 wave_log2=27, max_inflight=64):
    """The Poisson serving stream. Returns the served record and the request list (for plain)."""
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
    # pinned output slots, sized for the largest grid
    max_cells = 256 ** 3
    slots = queue.Queue()
    slot_bufs = []
    for k in range(workers):
        d = torch.empty(max_cells, dtype=torch.float32).pin_memory().numpy()
        o = torch.empty(max_cells, dtype=torch.uint8).pin_memory().numpy()
        slot_bufs.append((d, o))
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
    deadline[0] = t0 + seconds + max(60.0, seconds)
    for k, (arr, key, n) in enumerate(reqs):
        now = time.monotonic() - t0
        if arr > now:
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


def main(argv=None):
    args = parse(argv)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
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
    meshes = batch64_meshes() if args.workload == "batch64" else [sphere256()]
    stage(f"{len(meshes)} meshes, {sum(len(i) for _, i, _ in meshes)} triangles")
    grids = [unit_grid(sdfb, n) for _, _, n in meshes]
    cells = [g.cells for g in grids]
    total_cells = sum(cells)
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY)
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
    step_batch(cst, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, count_work=True))  # counting build (untimed)
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

    # ---- the single-mesh 256^3 bake (configs' plain single-mesh GPU bake) ----
    single = None
    if args.workload == "batch64":
        sv, si, sn = sphere256()
        sg = unit_grid(sdfb, sn)
        sdv, sdi = torch.from_numpy(sv).cuda(), torch.from_numpy(si.astype(np.int32)).cuda()
        sdd = torch.empty(sg.cells, dtype=torch.float32, device="cuda")
        sdo = torch.empty(sg.cells, dtype=torch.uint8, device="cuda")
        for _ in range(3):
            ctx.bake_device(sdv.data_ptr(), len(sv), sdi.data_ptr(), len(si), sg, opts, sdd.data_ptr(), sdo.data_ptr(),
                            stream.cuda_stream)
        ms = []
        for _ in range(5):
            flush.fill_(1.0)
            st = new_stats(sdfb)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.bake_device(sdv.data_ptr(), len(sv), sdi.data_ptr(), len(si), sg, opts, sdd.data_ptr(), sdo.data_ptr(),
                            stream.cuda_stream, st)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        single = {"workload": "displaced-sphere-256 (81,920 triangles, 256^3)", "ms": statistics.median(ms),
                  "voxels_per_s": sg.cells / (statistics.median(ms) * 1e-3), "ms_distance": st.ms_distance,
                  "ms_build": st.ms_build, "ms_occupancy": st.ms_occupancy, "ms_sign": st.ms_sign}

    stage("single mesh done" if single else "no single-mesh leg")
    # ---- roofline of the distance kernel ----
    peak = sgemm_peak(torch)
    stage(f"SGEMM peak {peak:.1f} TFLOP/s")
    flops = cst.flops_distance
    mean_dist_ms = statistics.mean(dist_ms)
    achieved = flops / (mean_dist_ms * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": "k_distance (+ k_distance_deferred)", "flops_per_launch": flops,
                "box_tests": int(cst.box_tests), "tri_tests": int(cst.tri_tests),
                "plane_tests": int(cst.plane_tests), "tiles_deferred": int(cst.tiles_deferred), "kernel_ms": mean_dist_ms,
                "peak_source": "cuBLAS SGEMM 8192^3 FP32 (TF32 off), best of 5, measured in this run",
                "algorithmic_bytes_per_launch": total_cells * 4}
    # the memory side beside it: distance writes plus one read of every mesh's hierarchy
    hbm_peak, hbm_src = hbm_peak_gbs()
    bvh_bytes = sum(len(i) * (64 + 64) for _, i, _ in meshes)  # triangle records + nodes
    moved = total_cells * 4 + bvh_bytes
    roofline["hbm"] = {"bytes_per_launch": moved, "achieved_gbs": moved / (mean_dist_ms * 1e-3) / 1e9,
                       "peak_gbs": hbm_peak, "frac": moved / (mean_dist_ms * 1e-3) / 1e9 / hbm_peak,
                       "peak_source": hbm_src}

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
    cpu = None if args.no_cpu_baseline else cpu_baseline(meshes, gpu_grids=hd)
    precision = cpu.pop("precision") if cpu else None
    stage("CPU baseline done" + (f": max error {precision['max_err_over_diag']:.3g} x diag" if precision else ""))
    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(step_ms) / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes generated in-process)",
        "config": {"workload": args.workload, "meshes": len(meshes), "triangles": int(sum(len(i) for _, i, _ in meshes)),
                   "voxels": int(total_cells), "grids": sorted({n for _, _, n in meshes}), "sign": "parity",
                   "seed": 2024 if args.workload == "batch64" else 1234, "parallelism": f"replicas x{world}",
                   "l2": "512 MB L2 flush before every timed step (outputs alone exceed L2)"},
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
        "single_mesh": single,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
