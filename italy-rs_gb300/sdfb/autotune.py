"""Autotuner for the bake's launch parameters on the GPU it runs on.

Three parameters of the distance pass trade against each other with the mesh and the grid:
  * leaf size (triangles per BVH leaf, 1..16): small leaves test fewer triangles per visit but add
    node tests and stack traffic;
  * tile shape (the cells one warp walks the BVH for, ids 1..6 = 4x4x2, 8x4x1, 4x4x4, 8x4x2,
    4x4x8, 8x4x4 cells with 1, 1, 2, 2, 4, 4 cells per lane): bigger tiles share one traversal
    among more cells but visit the union of their candidates;
  * traversal stack depth (32 or 64 entries): the shallow stack needs fewer registers but a deep
    tree overflows it (the bake then reruns that launch with 64);
  * step budget (traversal steps before a tile is handed to the block-per-tile second pass, or
    never): a small budget moves more tiles into the pass that splits a tile's walk over a block,
    which pays on small grids (fewer tiles than the GPU holds warps).

For each (log2 triangles, log2 grid edge) bucket of a sweep of displaced spheres and grids, the tuner
times whole device-buffer bakes (CUDA events on the bake's stream, median of `reps`) under a
coordinate descent over the four parameters, then fills every bucket of the table from the
nearest measured one and writes "tri_bucket grid_bucket leaf tile stack budget" lines (tile
0-based, budget 0 = never) that
the library reads at context creation (tuning/gb300.tsv beside lib/, or the file SDFB_TUNING names).

A batch takes its tile shape, stack depth and budget from the bucket of its mesh with the most
cells. The batch mode (--batch) times a 64-mesh batch (1e3..1e6 triangles, 32^3..256^3 grids) with
those choices and under a coordinate descent over batch-wide (tile, stack, budget) settings; when
the best beats the table's choice by more than BATCH_GAIN it writes a "batch tile stack budget"
line into the table, which the library then uses for every bake of more than one mesh, and
otherwise it records the comparison as a comment.

    python italy-rs_gb300/sdfb/autotune.py [--out PATH] [--quick]
    python italy-rs_gb300/sdfb/autotune.py --batch [--out PATH]
"""
from __future__ import annotations

import argparse
import datetime
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(os.path.dirname(HERE), "tuning", "gb300.tsv")

TILES = (1, 2, 3, 4, 5, 6)
LEAVES = (1, 2, 3, 4, 6, 8, 12, 16)
STACKS = (32, 64)
BUDGETS = (-1, 32, 128, 512, 1024, 2048, 4096)
START = (4, 3, 64, 1024)  # leaf, tile id (1-based), stack, step budget: the built-in defaults

# (mesh, grid edge): displaced icospheres of levels 3..7 (1,280 .. 327,680 triangles) on 32^3 .. 512^3
# grids, and displaced tori of 131,072 and 1,048,576 triangles (thin tubes; the largest meshes a
# batch holds) on 128^3 and 256^3 grids
SWEEP = [(3, 32), (3, 64), (3, 128), (3, 256), (4, 64), (4, 128), (4, 256), (5, 32), (5, 64), (5, 128),
         (5, 256), (5, 512), (6, 32), (6, 64), (6, 128), (6, 256), (6, 512), (7, 32), (7, 64), (7, 128),
         (7, 256), (7, 512), ("torus128k", 128), ("torus128k", 256), ("torus1m", 128), ("torus1m", 256)]
QUICK = [(4, 128), (6, 256), (7, 256)]
BATCH_GAIN = 0.02  # a batch-wide line is written only when it saves more than this fraction
TORI = {"torus128k": (512, 128), "torus1m": (1024, 512)}  # nu x nv quads, 2 nu nv triangles


def sweep_mesh(meshgen, key):
    if key in TORI:
        nu, nv = TORI[key]
        return meshgen.displaced_torus(nu, nv, 0.3, 0.1, 90 + nu)
    return meshgen.displaced_icosphere(key, 0.4, 100 + key)


def bucket_tris(t: int) -> int:
    """floor(log2 t), at most 31 (the library's own bucketing of triangle counts)."""
    b = 0
    while b < 31 and (2 << b) <= t:
        b += 1
    return b


def bucket_grid(n: int) -> int:
    """floor(log2 n) - 4, clamped to 0..7 (the library's own bucketing of the longest grid edge)."""
    b = 0
    while b < 20 and (2 << b) <= n:
        b += 1
    return max(0, min(7, b - 4))


def fill_table(measured: dict) -> dict:
    """Every (tri bucket 0..31, grid bucket 0..7) from the nearest measured bucket: distance
    |d tri| + 2 |d grid| (the grid edge moves the work per tile more than the triangle count does),
    ties to the larger bucket."""
    table = {}
    keys = sorted(measured)
    for tb in range(32):
        for nb in range(8):
            best = min(keys, key=lambda k: (abs(k[0] - tb) + 2 * abs(k[1] - nb), -k[0], -k[1]))
            table[(tb, nb)] = measured[best]
    return table


def write_table(path: str, table: dict, measured: dict, times: dict, header: list[str]):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        for h in header:
            f.write(f"# {h}\n")
        f.write("# tri_bucket grid_bucket leaf tile(0-based) stack budget(0 = never)\n")
        for (tb, nb), (leaf, tile, stack, budget) in sorted(table.items()):
            note = f"  # measured {times[(tb, nb)]:.3f} ms" if (tb, nb) in measured else ""
            f.write(f"{tb} {nb} {leaf} {tile - 1} {stack} {max(budget, 0)}{note}\n")


def write_batch_line(path: str, params, note: str):
    """Replaces the table's batch line (and batch comments) by `params` = (tile 1-based, stack,
    budget) or, when params is None, by the comment `note` alone."""
    lines = []
    if os.path.exists(path):
        with open(path) as f:
            lines = [l for l in f.read().splitlines() if not l.startswith("batch ") and not l.startswith("# batch:")]
    if params is None:
        lines.append(f"# batch: {note}")
    else:
        tile, stack, budget = params
        lines.append(f"batch {tile - 1} {stack} {max(budget, 0)}  # {note}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def tune_batch(time_batch, log=print):
    """Coordinate descent over batch-wide (tile, stack, budget) from the table's own choice.
    time_batch(params or None) -> ms. Returns (best params or None, best ms, table ms)."""
    cache = {}

    def t(p):
        if p not in cache:
            cache[p] = time_batch(p)
        return cache[p]

    table_ms = t(None)
    best, best_ms = None, table_ms
    cur = (START[1], START[2], START[3])
    for axis, values in ((0, TILES), (1, STACKS), (2, BUDGETS), (0, TILES)):
        for v in values:
            p = list(cur)
            p[axis] = v
            p = tuple(p)
            if t(p) < t(cur):
                cur = p
    if t(cur) < best_ms:
        best, best_ms = cur, t(cur)
    log(f"    batch: {len(cache)} configurations, table {table_ms:.3f} ms, best batch-wide {cur} {t(cur):.3f} ms")
    return best, best_ms, table_ms


def _time_batch(ctx, torch, sdfb, devm, grids, outs, params, reps: int) -> float:
    tile, stack, budget = params if params is not None else (0, 0, 0)
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, tile=tile, stack_depth=stack, step_budget=budget)
    stream = torch.cuda.current_stream()
    flush = torch.empty(128 << 20, dtype=torch.float32, device="cuda")  # 512 MB > L2

    def step():
        ctx.bake_batch_device(devm, grids, opts, outs[0], outs[1], stream.cuda_stream)

    step()
    step()
    times = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def _time_bake(ctx, torch, sdfb, dev, grid, params, reps: int) -> float:
    leaf, tile, stack, budget = params
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, leaf_size=leaf, tile=tile, stack_depth=stack,
                          step_budget=budget)
    stream = torch.cuda.current_stream()
    dv, nv, di, nt, dd, do = dev
    ctx.bake_device(dv, nv, di, nt, grid, opts, dd, do, stream.cuda_stream)  # warm-up
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.bake_device(dv, nv, di, nt, grid, opts, dd, do, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def tune_case(ctx, torch, sdfb, dev, grid, reps: int, log=print):
    """Coordinate descent: tile, leaf, stack, budget, then tile again. Returns (params, ms)."""
    cache = {}

    def t(p):
        if p not in cache:
            cache[p] = _time_bake(ctx, torch, sdfb, dev, grid, p, reps)
        return cache[p]

    best = START
    for axis, values in ((1, TILES), (0, LEAVES), (2, STACKS), (3, BUDGETS), (1, TILES)):
        for v in values:
            p = list(best)
            p[axis] = v
            p = tuple(p)
            if t(p) < t(best):
                best = p
    log(f"    {len(cache)} configurations, best leaf {best[0]} tile {best[1]} stack {best[2]} budget {best[3]}: "
        f"{t(best):.3f} ms "
        f"(defaults {t(START):.3f} ms)")
    return best, t(best)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--quick", action="store_true", help="three buckets only")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--batch", action="store_true", help="tune batch-wide settings against the table at --out")
    args = ap.parse_args(argv)

    sys.path.insert(0, os.path.dirname(HERE))
    import numpy as np
    import torch

    import sdfb
    from sdfb import meshgen

    if args.batch:
        os.environ["SDFB_TUNING"] = args.out  # the batch is timed against this table's choices
        write_batch_line(args.out, None, "being tuned")  # no batch line while timing
        ctx = sdfb.Context(0)
        meshes = meshgen.batch_meshes(64, seed=2024)
        grids = [sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n)) for _, _, n in meshes]
        dv = [torch.from_numpy(np.ascontiguousarray(v, np.float32)).cuda() for v, _, _ in meshes]
        di = [torch.from_numpy(np.ascontiguousarray(f, np.int32)).cuda() for _, f, _ in meshes]
        dd = [torch.empty(g.cells, dtype=torch.float32, device="cuda") for g in grids]
        do = [torch.empty(g.cells, dtype=torch.uint8, device="cuda") for g in grids]
        devm = [(a.data_ptr(), len(v), b.data_ptr(), len(f)) for a, b, (v, f, _) in zip(dv, di, meshes)]
        outs = ([d.data_ptr() for d in dd], [o.data_ptr() for o in do])
        best, best_ms, table_ms = tune_batch(
            lambda p: _time_batch(ctx, torch, sdfb, devm, grids, outs, p, args.reps))
        stamp = f"{torch.cuda.get_device_name(0)}, {datetime.date.today().isoformat()}, 64-mesh batch"
        if best is not None and best_ms < (1.0 - BATCH_GAIN) * table_ms:
            write_batch_line(args.out, best, f"{stamp}: {best_ms:.1f} ms against {table_ms:.1f} ms per mesh bucket")
        else:
            write_batch_line(args.out, None, f"{stamp}: the per-bucket choice kept ({table_ms:.1f} ms; best "
                                             f"batch-wide {best_ms:.1f} ms)")
        print(f"wrote {args.out}")
        ctx.close()
        return

    os.environ["SDFB_TUNING"] = os.devnull  # tune from the built-in defaults, not an older table
    ctx = sdfb.Context(0)
    measured, times = {}, {}
    meshes = {}
    for level, n in (QUICK if args.quick else SWEEP):
        if level not in meshes:
            meshes[level] = sweep_mesh(meshgen, level)
        v, f = meshes[level]
        grid = sdfb.make_grid((-0.5, -0.5, -0.5), 1.0 / n, (n, n, n))
        dv = torch.from_numpy(np.ascontiguousarray(v, np.float32)).cuda()
        di = torch.from_numpy(np.ascontiguousarray(f, np.int32)).cuda()
        dd = torch.empty(grid.cells, dtype=torch.float32, device="cuda")
        do = torch.empty(grid.cells, dtype=torch.uint8, device="cuda")
        key = (bucket_tris(len(f)), bucket_grid(n))
        print(f"  {len(f):>7} triangles, {n}^3 grid -> bucket {key}", flush=True)
        params, ms = tune_case(ctx, torch, sdfb, (dv.data_ptr(), len(v), di.data_ptr(), len(f),
                                                  dd.data_ptr(), do.data_ptr()), grid, args.reps)
        if key not in measured or ms < times[key]:
            measured[key], times[key] = params, ms
        del dv, di, dd, do
    table = fill_table(measured)
    header = [f"written by italy-rs_gb300/sdfb/autotune.py{' --quick' if args.quick else ''} on "
              f"{torch.cuda.get_device_name(0)}, {datetime.date.today().isoformat()}",
              f"{len(measured)} buckets measured (displaced icospheres and tori, parity sign, median of {args.reps}); "
              f"the rest filled from the nearest"]
    write_table(args.out, table, measured, times, header)
    print(f"wrote {args.out}")
    ctx.close()


if __name__ == "__main__":
    main()
