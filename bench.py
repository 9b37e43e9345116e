#!/usr/bin/env python
"""Benchmark of the GB300 mesh -> SDF bake.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workload (default ``displaced-sphere-256``): the level-6 displaced icosphere (81,920 triangles,
radius 0.35, 8 seeded sinusoids of total amplitude 0.05) baked onto a 256^3 FP32 grid over
[-0.5, 0.5]^3 with occupancy and exact parity sign. One step = one full bake (BVH build,
occupancy, parity crossings, distance + sign) of that mesh. Seeded synthetic input.

``value``  voxels/s with the mesh already in HBM (sdfb_bake_device), CUDA events on the bake's
           stream, L2 flushed (512 MB write) before every timed step.
``e2e``    the same metric through sdfb_bake with pinned host buffers: mesh upload, bake and the
           read-back of the distance and occupancy grids inside the timed region.
``roofline`` FP32 (the distance kernel is CUDA-core FMA work, no contraction): algorithmic flops
           per launch from the counting build of the same kernel / the kernel's mean CUDA-event
           time in the timed steps, against an SGEMM (cuBLAS, FP32, no TF32) measured in this run.
``cpu_baseline`` the CPU bake of the same mesh and grid on this host: occupancy by the reference's
           own SAT code where it was compiled (oracle/_ref) else by the oracle's restatement, FP64
           distance and exact parity sign from the oracle, all host threads.

Multi-GPU (torchrun): every rank bakes its own copy (replicas; the bake has no exchange step);
``value`` sums all ranks' voxels over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="displaced-sphere-256")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------------------------
# Workloads


def workload(name: str):
    from sdfb import meshgen as mg
    if name == "displaced-sphere-256":
        v, i = mg.displaced_sphere_mesh(seed=1234)
        origin, voxel, n = mg.unit_grid(256)
        cfg = {"workload": name, "mesh": "icosphere L6 displaced (8 sinusoids, amp 0.05), r=0.35",
               "triangles": int(len(i)), "grid": list(n), "bounds": [[-0.5] * 3, [0.5] * 3], "sign": "parity",
               "seed": 1234}
        return v, i, origin, voxel, n, cfg
    if name == "uv-sphere-64":
        v, i = mg.uv_sphere_mesh(0.4, 64, 32)
        origin, voxel, n = mg.unit_grid(64)
        cfg = {"workload": name, "mesh": "UV sphere r=0.4, 64 lon x 32 lat", "triangles": int(len(i)),
               "grid": list(n), "bounds": [[-0.5] * 3, [0.5] * 3], "sign": "parity"}
        return v, i, origin, voxel, n, cfg
    raise SystemExit(f"unknown workload {name}")


# ---------------------------------------------------------------------------------------------
# Clocks


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# CPU baseline (the reference's CPU occupancy code + the FP64 oracle)


def cpu_bake(v, i, origin, voxel, n, threads=0):
    """One CPU bake of the workload; returns (seconds, kind)."""
    from oracle.oracle import Oracle, soup_of
    orc = Oracle()
    kind = "port"
    ref = None
    try:
        from oracle import build_oracle
        if os.path.exists(build_oracle.REF_SO):
            from oracle.oracle import Reference
            ref = Reference(build_oracle.REF_SO)
            kind = "reference"
    except Exception:
        ref = None
    soup = soup_of(v, i) if ref is not None else None
    t0 = time.perf_counter()
    if ref is not None:
        occ = ref.occupancy(soup, origin, voxel, n)
    else:
        occ = orc.occupancy(v, i, origin, voxel, n)
    d = orc.distance(v, i, origin, voxel, n, threads=threads)
    s = orc.sign_parity(v, i, origin, voxel, n, axis=2, threads=threads)
    dist = (d * s).astype("float32")
    sec = time.perf_counter() - t0
    del occ, dist
    return sec, kind, orc.threads() if threads <= 0 else threads


def cpu_baseline(v, i, origin, voxel, n, budget_s=20.0):
    cells = n[0] * n[1] * n[2]
    secs = []
    kind = "port"
    cores = 1
    t_start = time.perf_counter()
    while True:
        s, kind, cores = cpu_bake(v, i, origin, voxel, n)
        secs.append(s)
        if time.perf_counter() - t_start > budget_s * 0.5 or len(secs) >= 3:
            break
    best = min(secs)
    return {"value": cells / best, "unit": "voxels/s", "cores": cores, "kind": kind,
            "sample": f"{len(secs)} full CPU bake(s) of the same mesh and {n[0]}x{n[1]}x{n[2]} grid "
                      f"(occupancy {'reference triBoxOverlap, 1 thread' if kind == 'reference' else 'oracle port, 1 thread'};"
                      f" FP64 distance + exact parity, {cores} threads); best {best:.2f} s"}


def run_reference(args, rank, world):
    """The reference arm: the CPU bake (the reference's own code path for this bake has no GPU
    implementation that can run here; its OptiX estimate needs the OptiX SDK)."""
    if rank != 0:
        return
    v, i, origin, voxel, n, cfg = workload(args.workload)
    cells = n[0] * n[1] * n[2]
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_bake(v, i, origin, voxel, n)
    times = []
    kind, cores = "port", 1
    for _ in range(args.steps):
        s, kind, cores = cpu_bake(v, i, origin, voxel, n)
        times.append(s)
        if sum(times) > 150:
            break
    tot = sum(times)
    value = cells * len(times) / tot
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": 1000 * tot / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": cores, "kind": kind,
                             "sample": f"{len(times)} full CPU bakes of the workload"},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU arm


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


def main():
    args = parse()
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
    lib_path = sdfb.LIB_PATH
    if not os.path.exists(lib_path):
        import build as pkg_build
        pkg_build.build()
    ctx = sdfb.Context(local)
    v, i, origin, voxel, n, cfg = workload(args.workload)
    cells = n[0] * n[1] * n[2]
    grid = sdfb.make_grid(origin, voxel, n)
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY)
    stream = torch.cuda.current_stream()
    dv = torch.from_numpy(v).cuda()
    di = torch.from_numpy(i.astype(np.int32)).cuda()
    dd = torch.empty(cells, dtype=torch.float32, device="cuda")
    do = torch.empty(cells, dtype=torch.uint8, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def bake_dev(stats=None):
        ctx.bake_device(dv.data_ptr(), len(v), di.data_ptr(), len(i), grid, opts, dd.data_ptr(), do.data_ptr(),
                        stream.cuda_stream, stats)

    def new_stats():
        st = sdfb.Stats()
        st.struct_size = sdfb.C.sizeof(sdfb.Stats)
        return st

    for _ in range(max(args.warmup, 3)):
        bake_dev()
    torch.cuda.synchronize()

    # counting build (untimed): exact traversal work of one launch
    cst = new_stats()
    ctx.bake_device(dv.data_ptr(), len(v), di.data_ptr(), len(i), grid, sdfb.make_opts(
        sign_mode=sdfb.SIGN_PARITY, count_work=True), dd.data_ptr(), do.data_ptr(), stream.cuda_stream, cst)

    # timed region
    clocks = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    step_ms, dist_ms, launches = [], [], []
    for _ in range(args.steps):
        flush.fill_(1.0)
        st = new_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bake_dev(st)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        dist_ms.append(st.ms_distance)
        launches.append(st.kernel_launches)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clk = clocks.stop()
    total_ms = sum(step_ms)
    if pg:
        t = torch.tensor([total_ms], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * cells * args.steps / (total_ms * 1e-3)

    # e2e through the host-buffer entry point (pinned host memory both ways)
    hv = torch.from_numpy(v).pin_memory().numpy()
    hi = torch.from_numpy(i).pin_memory().numpy() if i.dtype == np.uint32 else None
    if hi is None:
        hi = torch.from_numpy(i.astype(np.int32)).pin_memory().numpy().view(np.uint32)
    hd = torch.empty(cells, dtype=torch.float32).pin_memory().numpy().reshape(grid.shape)
    ho = torch.empty(cells, dtype=torch.uint8).pin_memory().numpy().reshape(grid.shape)
    lib = ctx.lib

    def bake_host():
        stt = lib.sdfb_bake(ctx.h, hv.ctypes.data_as(sdfb.C.c_void_p), len(hv), hi.ctypes.data_as(sdfb.C.c_void_p),
                            len(hi), sdfb.C.byref(grid), sdfb.C.byref(opts), hd.ctypes.data_as(sdfb.C.c_void_p),
                            ho.ctypes.data_as(sdfb.C.c_void_p), None)
        if stt != 0:
            raise sdfb.SdfbError(stt, ctx.error())

    for _ in range(2):
        bake_host()
    e2e_s = []
    for _ in range(max(3, args.steps // 2)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bake_host()
        e2e_s.append(time.perf_counter() - t0)
    e2e_total = sum(e2e_s)
    if pg:
        t = torch.tensor([e2e_total], device="cuda")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = world * cells * len(e2e_s) / e2e_total

    if rank != 0:
        if pg:
            pg.barrier()
            pg.destroy_process_group()
        return

    # roofline of the distance kernel
    peak = sgemm_peak(torch)
    flops = cst.flops_distance
    mean_dist_ms = statistics.mean(dist_ms)
    achieved = flops / (mean_dist_ms * 1e-3) / 1e12
    roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": "k_distance", "flops_per_launch": flops,
                "box_tests": int(cst.box_tests), "tri_tests": int(cst.tri_tests),
                "kernel_ms": mean_dist_ms,
                "peak_source": "cuBLAS SGEMM 8192^3 FP32 (TF32 off), best of 5, measured in this run",
                "algorithmic_bytes_per_launch": cells * 4}

    # precision against FP64 on a seeded sample
    from oracle.oracle import Oracle
    orc = Oracle()
    rng = np.random.default_rng(0)
    samp = np.sort(rng.choice(cells, min(cells, 20000), replace=False)).astype(np.int64)
    d64 = orc.distance(v, i, origin, voxel, n, samples=samp)
    got = np.abs(hd.reshape(-1)[samp].astype(np.float64))
    diagv = float(voxel) * float(np.sqrt(n[0] ** 2 + n[1] ** 2 + n[2] ** 2))
    err = np.abs(got - d64) / diagv

    cpu = None if args.no_cpu_baseline else cpu_baseline(v, i, origin, voxel, n)
    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded meshes generated in-process)",
        "config": {**cfg, "plain_single_mesh": True, "parallelism": f"replicas x{world}",
                   "l2": "512 MB L2 flush before every timed step"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "voxels/s", "h2d_bytes_per_step": int(v.nbytes + i.nbytes),
                "d2h_bytes_per_step": int(cells * 5), "ms_per_step": 1000 * e2e_total / len(e2e_s)},
        "clocks": clk,
        "gpu_launches": int(sum(launches)),
        "precision": {"max_err_over_diag": float(err.max()), "rms_err_over_diag": float(np.sqrt((err ** 2).mean())),
                      "samples": int(len(samp)), "reference": "FP64 oracle"},
        "stages_ms": {"distance": mean_dist_ms},
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
