"""Per-cell materials on the device (sdfb_bake_materials, sdfb_voxelize_sparse_colors) against the
reference's fixtures and the oracle, bit for bit: every operation of the material path is an IEEE
FP32 operation in the reference's order, and the sums add each cell's triangles in triangle order."""
from __future__ import annotations

import numpy as np
import pytest

from test_oracle_golden import golden_materials

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def soup_of_mesh(v, f):
    return np.ascontiguousarray(v[f.reshape(-1)], np.float32)


def test_golden_materials(ctx, golden):
    import sdfb
    soup, m = golden["mat_soup"], golden_materials(golden)
    cells, cols, _, _ = ctx.voxelize_sparse_colors(soup, soup.min(0), soup.max(0), 40, m)
    assert np.array_equal(cells, golden["mat_sparse_cells"])
    assert np.array_equal(bits(cols), bits(golden["mat_sparse_colors"]))
    g = golden["mat_dense_grid"]
    grid = sdfb.make_grid(g[0:3].astype(np.float32), np.float32(g[3]), tuple(int(x) for x in g[4:7]))
    col, met, rou = ctx.bake_materials(soup, grid, m)
    col, met, rou = col.reshape(-1, 3), met.reshape(-1), rou.reshape(-1)
    hit = golden["mat_dense_cells"]
    got = np.concatenate([col[hit], met[hit, None], rou[hit, None]], axis=1)
    assert np.array_equal(bits(got), bits(golden["mat_dense_values"]))
    rest = np.ones(len(met), bool)
    rest[hit] = False
    assert (col[rest] == 1.0).all() and (met[rest] == 0.0).all() and (rou[rest] == 1.0).all()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_materials_match_oracle(ctx, oracle, seed):
    import sdfb
    from sdfb import meshgen as mg
    rng = np.random.default_rng(seed)
    n = int(rng.integers(200, 3000))
    c = rng.uniform(-0.45, 0.45, size=(n, 1, 3))
    s = rng.lognormal(mean=-3.0, sigma=1.0, size=(n, 1, 1))
    soup = (c + s * rng.normal(size=(n, 3, 3))).reshape(-1, 3).astype(np.float32)
    soup[: 3 * (n // 8)] = np.round(soup[: 3 * (n // 8)] * 32) / 32  # lattice-snapped: SAT ties
    m = mg.random_materials(n, seed, num_materials=int(rng.integers(1, 7)))
    res = int(rng.integers(8, 96))
    lo, hi = soup.min(0), soup.max(0)
    cells, cols, _, _ = ctx.voxelize_sparse_colors(soup, lo, hi, res, m)
    oc, ok = oracle.voxelize_colors(soup, lo, hi, res, m)
    assert np.array_equal(cells, oc) and np.array_equal(bits(cols), bits(ok))
    g = sdfb.grid_from_bounds_res(lo, hi, res)
    col, met, rou = ctx.bake_materials(soup, g, m)
    ocol, omet, orou = oracle.materials_dense(soup, g.origin[:], g.voxel_size, (g.nx, g.ny, g.nz), m)
    assert np.array_equal(bits(col.reshape(-1, 3)), bits(ocol))
    assert np.array_equal(bits(met.reshape(-1)), bits(omet))
    assert np.array_equal(bits(rou.reshape(-1)), bits(orou))


def test_materials_full_size_sphere(ctx, oracle):
    """The displaced sphere (81,920 triangles) as a soup on its 256-resolution bake grid, every
    cell against the oracle."""
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_sphere_mesh()
    soup = soup_of_mesh(v, f)
    m = mg.random_materials(len(f), 9, num_materials=5, tex_sizes=((256, 128), (64, 64)))
    g = sdfb.grid_from_bounds_res(soup.min(0), soup.max(0), 256)
    col, met, rou = ctx.bake_materials(soup, g, m)
    ocol, omet, orou = oracle.materials_dense(soup, g.origin[:], g.voxel_size, (g.nx, g.ny, g.nz), m)
    assert np.array_equal(bits(col.reshape(-1, 3)), bits(ocol))
    assert np.array_equal(bits(met.reshape(-1)), bits(omet)) and np.array_equal(bits(rou.reshape(-1)), bits(orou))
    assert (met.reshape(-1) != 0).sum() > 100000


def test_material_edge_cases(ctx, oracle):
    import sdfb
    from sdfb import meshgen as mg
    rng = np.random.default_rng(4)
    soup = rng.uniform(-0.5, 0.5, (60 * 3, 3)).astype(np.float32)
    g = sdfb.grid_from_bounds_res(soup.min(0), soup.max(0), 16)
    n = (g.nx, g.ny, g.nz)
    # one material, no per-triangle list, no uvs, no textures
    m = {"mat_f": np.array([[0.2, 0.4, 0.6, 0.3, 0.7]], np.float32), "mat_tex": np.array([-1], np.int32)}
    got = ctx.bake_materials(soup, g, m)
    ref = oracle.materials_dense(soup, g.origin[:], g.voxel_size, n, m)
    for a, b in zip(got, ref):
        assert np.array_equal(bits(a).reshape(-1), bits(b).reshape(-1))
    # textured material but too few uvs: the factor alone
    m2 = mg.random_materials(60, 5)
    m2["uvs"] = m2["uvs"][:30]
    got = ctx.bake_materials(soup, g, m2)
    ref = oracle.materials_dense(soup, g.origin[:], g.voxel_size, n, m2)
    for a, b in zip(got, ref):
        assert np.array_equal(bits(a).reshape(-1), bits(b).reshape(-1))
    # no triangles: every cell keeps the defaults
    col, met, rou = ctx.bake_materials(np.zeros((0, 3), np.float32), g, m)
    assert (col == 1).all() and (met == 0).all() and (rou == 1).all()
    # no material is an error
    st = ctx.lib.sdfb_bake_materials(ctx.h, None, 0, sdfb.C.byref(g), None, None, None, None)
    assert st == sdfb.ERR_INVALID_ARGUMENT
