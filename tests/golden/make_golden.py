"""Generates the golden fixtures in tests/golden/ (run here, where the reference tree exists).

Occupancy, sparse cell lists, grid sizing, weld indices and watertight verdicts come from the
reference's OWN code, compiled from its sources into oracle/_ref (oracle/build_oracle.py):
triBoxOverlap driven by the bakePerCellMaterial candidate loop, voxelizeMesh, weldPositions,
isWatertight. Distances and signs come from the FP64 oracle (the reference has no exact distance;
its OptiX estimate is not reproducible here). Every fixture stores its input mesh, so the tests do
not depend on regenerating meshes bit-identically on another machine.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "italy-rs_gb300"))

from oracle.oracle import Oracle, Reference, soup_of  # noqa: E402
from sdfb import meshgen as mg  # noqa: E402


def quad(a, b, c, d):
    return [a, b, c, a, c, d]


def cube_soup(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)) -> np.ndarray:
    """The reference tests' unit cube (tests/voxelize_test.cpp:22-37, mesh_validate_test.cpp:21-36)."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    p = []
    p += quad((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0))
    p += quad((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1))
    p += quad((x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1))
    p += quad((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0))
    p += quad((x0, y0, z0), (x0, y0, z1), (x1, y0, z1), (x1, y0, z0))
    p += quad((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1))
    return np.asarray(p, np.float32)


def random_soup(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.45, 0.45, size=(n, 1, 3))
    s = rng.lognormal(mean=-3.0, sigma=1.0, size=(n, 1, 1))
    tri = c + s * rng.normal(size=(n, 3, 3))
    # a few triangles snapped to the grid lattice to exercise ties
    tri[: n // 8] = np.round(tri[: n // 8] * 32.0) / 32.0
    return tri.reshape(-1, 3).astype(np.float32)


def main():
    O, R = Oracle(), Reference()
    out = {}

    # 1. Cube shell, res 8: sparse cells in insertion order (voxelize_test.cpp:37-58) + dense grid.
    cube = cube_soup()
    cells, org, vox = R.voxelize(cube, (0, 0, 0), (1, 1, 1), 8)
    out["cube_soup"] = cube
    out["cube_sparse_cells"] = cells
    out["cube_sparse_origin"] = org
    out["cube_sparse_voxel"] = np.float32(vox)
    go, gv, gn = R.grid_from_bounds((0, 0, 0), (1, 1, 1), 8)
    out["cube_grid"] = np.array([*go, gv, *gn], np.float64)
    out["cube_occ"] = np.packbits(R.occupancy(cube, go, gv, gn))
    # grid-aligned faces: the cube on a lattice whose cell boundaries hit its faces exactly
    out["cube_aligned_occ"] = np.packbits(R.occupancy(cube, (0.0, 0.0, 0.0), 0.125, (8, 8, 8)))
    out["cube_aligned_occ_shift"] = np.packbits(R.occupancy(cube, (-0.0625, -0.0625, -0.0625), 0.125, (10, 10, 10)))

    # 2. Watertight gate (mesh_validate_test.cpp:37-63).
    ok, msg = R.is_watertight(cube, (0, 0, 0), (1, 1, 1))
    out["cube_watertight"] = np.int8(ok)
    ok2, msg2 = R.is_watertight(cube[:-6], (0, 0, 0), (1, 1, 1))
    out["holey_watertight"] = np.int8(ok2)

    # 3. The sign test's UV sphere r = 1, 32 lon x 16 lat, res 24 (sdf_sign_test.cpp:46-83).
    s1 = mg.uv_sphere_soup(1.0, 32, 16)
    w1, n1 = R.weld(s1, (-1, -1, -1), (1, 1, 1))
    out["sphere1_soup"] = s1
    out["sphere1_weld"] = w1
    out["sphere1_watertight"] = np.int8(R.is_watertight(s1, (-1, -1, -1), (1, 1, 1))[0])
    g1o, g1v, g1n = R.grid_from_bounds((-1, -1, -1), (1, 1, 1), 24)
    out["sphere1_grid"] = np.array([*g1o, g1v, *g1n], np.float64)
    out["sphere1_occ"] = np.packbits(R.occupancy(s1, g1o, g1v, g1n))
    # indexed form (unique first-occurrence positions + welded indices) for the GPU API
    uniq = np.zeros((n1, 3), np.float32)
    first = {}
    for i, k in enumerate(w1):
        if k not in first:
            first[k] = i
    for k, i in first.items():
        uniq[k] = s1[i]
    idx1 = w1.reshape(-1, 3)
    out["sphere1_verts"] = uniq
    out["sphere1_idx"] = idx1
    out["sphere1_dist64"] = O.distance(uniq, idx1, g1o, g1v, g1n)
    out["sphere1_sign"] = O.sign_parity(uniq, idx1, g1o, g1v, g1n, axis=2)

    # 4. Plain-bake sphere: r = 0.4, 64 lon x 32 lat, over [-0.5, 0.5]^3 at 64^3.
    s4 = mg.uv_sphere_soup(0.4, 64, 32)
    w4, n4 = R.weld(s4, (-0.4,) * 3, (0.4,) * 3)
    v4, i4 = mg.weld(s4, (-0.4,) * 3, (0.4,) * 3)
    assert np.array_equal(w4.reshape(-1, 3), i4)
    out["c1_verts"] = v4
    out["c1_idx"] = i4
    org4, vox4, n4g = (-0.5, -0.5, -0.5), 1.0 / 64, (64, 64, 64)
    out["c1_occ"] = np.packbits(R.occupancy(s4, org4, vox4, n4g))
    out["c1_sign"] = np.packbits(O.sign_parity(v4, i4, org4, vox4, n4g, axis=2) < 0)
    rng = np.random.default_rng(7)
    samp = np.sort(rng.choice(64 ** 3, 4096, replace=False)).astype(np.int64)
    out["c1_samples"] = samp
    out["c1_dist64_samples"] = O.distance(v4, i4, org4, vox4, n4g, samples=samp)
    out["c1_grid_from_bounds_res64"] = np.array([*R.grid_from_bounds((-0.4,) * 3, (0.4,) * 3, 64)[0],
                                                 R.grid_from_bounds((-0.4,) * 3, (0.4,) * 3, 64)[1],
                                                 *R.grid_from_bounds((-0.4,) * 3, (0.4,) * 3, 64)[2]], np.float64)

    # 5. Random soup with grid-snapped triangles on a 32^3 grid (ties in the SAT test).
    rs = random_soup(300, 11)
    out["rsoup"] = rs
    out["rsoup_occ"] = np.packbits(R.occupancy(rs, (-0.5, -0.5, -0.5), 1.0 / 32, (32, 32, 32)))
    rc, ro, rv = R.voxelize(rs, rs.min(0), rs.max(0), 40)
    out["rsoup_sparse_cells"] = rc
    out["rsoup_sparse_bounds"] = np.stack([rs.min(0), rs.max(0)])

    # 6. Grid sizing for awkward bounds and resolutions.
    gs = []
    rng = np.random.default_rng(3)
    for k in range(64):
        lo = rng.uniform(-3, 3, 3).astype(np.float32)
        hi = (lo + rng.uniform(1e-7, 4, 3)).astype(np.float32)
        res = int(rng.integers(1, 300))
        o, v, n = R.grid_from_bounds(lo, hi, res)
        gs.append([*lo, *hi, res, *o, v, *n])
    out["grid_sizing_cases"] = np.array(gs, np.float64)

    # 7. Materials: a random soup with a seeded material set (two textures, one sRGB; triangle
    # material indices past the end; uvs outside [0, 1)). Sparse colours come from the
    # reference's own voxelizeMesh; the dense per-cell averages of bakePerCellMaterial from its
    # restatement in the reference driver (that function sits in the OptiX translation unit).
    ms = random_soup(400, 21)
    mm = mg.random_materials(len(ms) // 3, 21)
    out["mat_soup"] = ms
    out["mat_f"] = mm["mat_f"]
    out["mat_tex"] = mm["mat_tex"]
    out["mat_tri"] = mm["tri_mat"]
    out["mat_uvs"] = mm["uvs"]
    out["mat_tex0"], out["mat_tex1"] = mm["textures"][0][0], mm["textures"][1][0]
    out["mat_tex_srgb"] = np.array([1 if t[1] else 0 for t in mm["textures"]], np.int32)
    mc, mcol = R.voxelize_colors(ms, ms.min(0), ms.max(0), 40, mm)
    out["mat_sparse_cells"] = mc
    out["mat_sparse_colors"] = mcol
    mo, mv, mn = R.grid_from_bounds(ms.min(0), ms.max(0), 24)
    col, met, rou = R.materials_dense(ms, mo, mv, mn, mm)
    hit = np.flatnonzero(np.any(col != 1.0, axis=1) | (met != 0.0) | (rou != 1.0)).astype(np.int64)
    out["mat_dense_grid"] = np.array([*mo, mv, *mn], np.float64)
    out["mat_dense_cells"] = hit
    out["mat_dense_values"] = np.concatenate([col[hit], met[hit, None], rou[hit, None]], axis=1)

    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes;", msg2)


if __name__ == "__main__":
    main()
