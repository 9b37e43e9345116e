"""The CPU oracle, pinned: against fixtures produced by the reference's own code (oracle/_ref),
against the reference's known-answer tests, and against analytic geometry. No GPU needed."""
from __future__ import annotations

from fractions import Fraction

import numpy as np
import pytest

from conftest import grid_of, unpack


def test_grid_sizing_matches_reference(golden, oracle):
    # bakeSdf grid sizing, src/convert/sdf_baker.cpp:138-148
    for row in golden["grid_sizing_cases"]:
        lo, hi, res = row[0:3].astype(np.float32), row[3:6].astype(np.float32), int(row[6])
        o, v, n = oracle.grid_from_bounds(lo, hi, res)
        assert np.array_equal(o, row[7:10].astype(np.float32))
        assert np.float32(v) == np.float32(row[10])
        assert n == tuple(int(x) for x in row[11:14])


@pytest.mark.parametrize("name,grid", [
    ("cube_occ", None), ("cube_aligned_occ", ((0.0, 0.0, 0.0), 0.125, (8, 8, 8))),
    ("cube_aligned_occ_shift", ((-0.0625,) * 3, 0.125, (10, 10, 10)))])
def test_cube_occupancy_matches_reference(golden, oracle, name, grid):
    o, v, n = grid_of(golden["cube_grid"]) if grid is None else grid
    occ = oracle.occupancy(golden["cube_soup"], None, o, v, n)
    assert np.array_equal(occ, unpack(golden[name], occ.size))


def test_sphere_occupancy_matches_reference(golden, oracle):
    o, v, n = grid_of(golden["sphere1_grid"])
    occ = oracle.occupancy(golden["sphere1_soup"], None, o, v, n)
    assert np.array_equal(occ, unpack(golden["sphere1_occ"], occ.size))
    # the indexed (welded) form gives the same occupancy: welding keeps first-occurrence positions
    occ2 = oracle.occupancy(golden["sphere1_verts"], golden["sphere1_idx"], o, v, n)
    assert np.array_equal(occ, occ2)


def test_c1_and_random_soup_occupancy(golden, oracle):
    occ = oracle.occupancy(golden["c1_verts"], golden["c1_idx"], (-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    assert np.array_equal(occ, unpack(golden["c1_occ"], occ.size))
    occ = oracle.occupancy(golden["rsoup"], None, (-0.5,) * 3, 1.0 / 32, (32, 32, 32))
    assert np.array_equal(occ, unpack(golden["rsoup_occ"], occ.size))


def test_sparse_voxelize_matches_reference_order(golden, oracle):
    # tests/voxelize_test.cpp:37-58 plus the exact insertion order of voxelizeMesh
    cells, org, vox = oracle.voxelize_sparse(golden["cube_soup"], (0, 0, 0), (1, 1, 1), 8)
    assert np.array_equal(cells, golden["cube_sparse_cells"])
    assert 0 < len(cells) <= 6 * 8 * 8
    assert any((c == [0, 0, 0]).all() for c in cells)
    assert not any((c == [4, 4, 4]).all() for c in cells)
    b = golden["rsoup_sparse_bounds"]
    cells, _, _ = oracle.voxelize_sparse(golden["rsoup"], b[0], b[1], 40)
    assert np.array_equal(cells, golden["rsoup_sparse_cells"])


def test_weld_and_watertight(golden, oracle):
    w, n = oracle.weld(golden["sphere1_soup"], (-1,) * 3, (1,) * 3)
    assert np.array_equal(w, golden["sphere1_weld"])
    ok, b, m = oracle.watertight(w)
    assert ok == bool(golden["sphere1_watertight"]) and b == 0 and m == 0
    cube = golden["cube_soup"]
    wc, _ = oracle.weld(cube, (0, 0, 0), (1, 1, 1))
    assert oracle.watertight(wc)[0] == bool(golden["cube_watertight"])
    wh, _ = oracle.weld(cube[:-6], (0, 0, 0), (1, 1, 1))
    ok, b, m = oracle.watertight(wh)
    assert ok == bool(golden["holey_watertight"]) and not ok and b == 4
    # an empty mesh is not watertight (mesh_validate_test.cpp:58-62)
    assert oracle.watertight(np.zeros(0, np.uint32))[0] is False


def test_distance_sign_against_analytic_sphere(golden, oracle):
    """tests/sdf_sign_test.cpp:46-83 on the oracle: sign exact where |analytic| > 1.5 voxel and
    |error| < 3 voxel, and far tighter: the error is bounded by the tessellation gap."""
    o, v, n = grid_of(golden["sphere1_grid"])
    d = golden["sphere1_dist64"]
    s = golden["sphere1_sign"]
    xs = [(np.float32(o[a]) + (np.arange(n[a], dtype=np.float32) + np.float32(0.5)) * np.float32(v)) for a in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    an = np.sqrt(X.astype(np.float64) ** 2 + Y ** 2 + Z ** 2).reshape(-1) - 1.0
    far = np.abs(an) > 1.5 * v
    assert far.sum() > 0
    assert np.all((an[far] < 0) == (s[far] < 0))
    err = np.abs(s * d - an)[far]
    assert err.max() < 3 * v
    # chord sag of a 32 x 16 UV sphere of radius 1 bounds the distance error (about 0.02)
    assert err.max() < 1 - np.cos(np.pi / 16) + 1e-9


def test_parity_axes_agree_and_match_golden(golden, oracle):
    v4, i4 = golden["c1_verts"], golden["c1_idx"]
    g = ((-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    sz = oracle.sign_parity(v4, i4, *g, axis=2)
    assert np.array_equal(sz < 0, unpack(golden["c1_sign"], sz.size).astype(bool))
    d = oracle.distance(v4, i4, *g)
    far = d > 1.0 / 64
    for ax in (0, 1):
        s = oracle.sign_parity(v4, i4, *g, axis=ax)
        assert np.array_equal(s[far], sz[far])
    samp = golden["c1_samples"]
    assert np.allclose(d[samp], golden["c1_dist64_samples"], rtol=0, atol=1e-12)


def test_gwn_agrees_with_parity_on_closed_mesh(golden, oracle):
    v4, i4 = golden["c1_verts"], golden["c1_idx"]
    g = ((-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    samp = golden["c1_samples"][:1024]
    w = oracle.gwn(v4, i4, *g, samples=samp)
    s = oracle.sign_parity(v4, i4, *g, axis=2)[samp]
    assert np.array_equal(np.abs(w) > 0.5, s < 0)
    # a closed mesh has winding number 0 or +-1 away from the surface
    d = golden["c1_dist64_samples"][:1024]
    far = d > 1.0 / 64
    assert np.all(np.minimum(np.abs(np.abs(w[far]) - 1), np.abs(w[far])) < 1e-6)


def _orient_exact(a, b, p):
    F = Fraction
    return (F(b[0]) - F(a[0])) * (F(p[1]) - F(a[1])) - (F(b[1]) - F(a[1])) * (F(p[0]) - F(a[0]))


def test_orient_predicate_is_exact(oracle):
    """Nearly collinear float triples: the oracle's sign equals the rational sign (ties broken by
    the (eps, eps^2) perturbation rule)."""
    rng = np.random.default_rng(5)
    f = np.float32
    for k in range(2000):
        a = rng.uniform(-1, 1, 2).astype(f)
        b = rng.uniform(-1, 1, 2).astype(f)
        t = f(rng.uniform(-0.5, 1.5))
        p = (a + t * (b - a)).astype(f)  # on the line up to rounding
        if k % 3 == 0:
            p = np.nextafter(p, f(2) * np.sign(rng.normal(size=2)).astype(f))
        if k % 7 == 0:  # exact ties on axis-aligned lines
            p = np.array([a[0], rng.uniform(-1, 1)], f)
            b = np.array([a[0], b[1]], f)
        s = oracle.orient2_sos(*[float(x) for x in (a[0], a[1], b[0], b[1], p[0], p[1])])
        ex = _orient_exact([float(x) for x in a], [float(x) for x in b], [float(x) for x in p])
        if ex != 0:
            assert s == (1 if ex > 0 else -1)
        else:
            exp = (1 if a[1] > b[1] else -1) if a[1] != b[1] else ((1 if b[0] > a[0] else -1) if b[0] != a[0] else 0)
            assert s == exp


def test_shared_edge_counted_once(oracle):
    """A column through the shared edge (and the shared vertex) of a closed fan crosses it once."""
    f = np.float32
    top = np.array([0, 0, 1], f)
    ring = [np.array([np.cos(t), np.sin(t), 0], f) for t in np.linspace(0, 2 * np.pi, 7)[:-1]]
    ring[0] = np.array([1, 0, 0], f)
    hits = 0
    for k in range(6):
        a, b = ring[k], ring[(k + 1) % 6]
        hit, _ = oracle.column_crossing(a, b, top, 2, 0.0, 0.0)  # through the apex
        hits += hit
    assert hits == 1
    hits = 0
    for k in range(6):
        a, b = ring[k], ring[(k + 1) % 6]
        hit, _ = oracle.column_crossing(a, b, top, 2, float(ring[0][0]) * 0.5, 0.0)  # on edge apex-ring[0]
        hits += hit
    assert hits == 1


def test_oracle_matches_live_reference_occupancy(reference, oracle):
    rng = np.random.default_rng(99)
    for seed in range(4):
        n = int(rng.integers(50, 400))
        c = rng.uniform(-0.45, 0.45, size=(n, 1, 3))
        s = rng.lognormal(mean=-3.0, sigma=1.0, size=(n, 1, 1))
        tri = (c + s * rng.normal(size=(n, 3, 3))).reshape(-1, 3).astype(np.float32)
        tri[: n // 4] = np.round(tri[: n // 4] * 16) / 16
        res = int(rng.integers(8, 48))
        o = rng.uniform(-0.6, -0.4, 3).astype(np.float32)
        v = float(np.float32(1.0 / res))
        occ_r = reference.occupancy(tri, o, v, (res, res, res))
        occ_o = oracle.occupancy(tri, None, o, v, (res, res, res))
        assert np.array_equal(occ_r, occ_o)
        lo, hi = tri.min(0), tri.max(0)
        cr, _, _ = reference.voxelize(tri, lo, hi, res)
        co, _, _ = oracle.voxelize_sparse(tri, lo, hi, res)
        assert np.array_equal(cr, co)


def test_degenerate_triangles_are_their_edges(oracle):
    """Zero-area triangles (collinear, two coincident vertices, a point) measure as the union of
    their edges."""
    v = np.array([[0, 0, 0], [0.2, 0.1, 0.0], [0.4, 0.2, 0.0], [0.1, 0.3, 0.2], [0.1, 0.3, 0.2]], np.float32)
    i = np.array([[0, 1, 2], [3, 4, 0], [2, 2, 2]], np.uint32)
    n = (12, 12, 12)
    o = np.float32(-0.2)
    vox = np.float32(0.05)
    d = oracle.distance(v, i, (o,) * 3, vox, n)
    c = (o + (np.arange(12, dtype=np.float32) + np.float32(0.5)) * vox).astype(np.float32)
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    P = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float64)

    def seg(a, b):
        ab = b - a
        l2 = ab @ ab
        t = np.clip(((P - a) @ ab) / l2, 0, 1) if l2 > 0 else np.zeros(len(P))
        return np.linalg.norm(P - a - t[:, None] * ab, axis=1)

    V = v.astype(np.float64)
    bf = np.minimum.reduce([seg(V[0], V[2]), seg(V[3], V[0]), seg(V[2], V[2])])
    assert np.abs(bf - d).max() < 1e-12


def golden_materials(golden):
    return {"mat_f": golden["mat_f"], "mat_tex": golden["mat_tex"], "tri_mat": golden["mat_tri"],
            "uvs": golden["mat_uvs"],
            "textures": [(golden["mat_tex0"], bool(golden["mat_tex_srgb"][0])),
                         (golden["mat_tex1"], bool(golden["mat_tex_srgb"][1]))]}


def test_material_colors_match_reference(golden, oracle):
    """voxelizeMesh's per-cell colours (voxelize.cpp:78-104, textures sampled nearest with wrap,
    sRGB decoded) and bakePerCellMaterial's dense averages (sdf_baker.cpp:76-128), bit for bit."""
    soup, m = golden["mat_soup"], golden_materials(golden)
    cells, cols = oracle.voxelize_colors(soup, soup.min(0), soup.max(0), 40, m)
    assert np.array_equal(cells, golden["mat_sparse_cells"])
    assert np.array_equal(cols.view(np.uint32), golden["mat_sparse_colors"].view(np.uint32))
    # the same cell list as the plain voxelizer
    plain, _, _ = oracle.voxelize_sparse(soup, soup.min(0), soup.max(0), 40)
    assert np.array_equal(plain, cells)
    g = golden["mat_dense_grid"]
    col, met, rou = oracle.materials_dense(soup, g[0:3].astype(np.float32), np.float32(g[3]),
                                           tuple(int(x) for x in g[4:7]), m)
    hit = golden["mat_dense_cells"]
    got = np.concatenate([col[hit], met[hit, None], rou[hit, None]], axis=1)
    assert np.array_equal(got.view(np.uint32), golden["mat_dense_values"].view(np.uint32))
    rest = np.ones(len(met), bool)
    rest[hit] = False
    assert (col[rest] == 1.0).all() and (met[rest] == 0.0).all() and (rou[rest] == 1.0).all()
    # textures matter: some cells average textured colours, which differ from every factor
    assert len(np.unique(cols[:, 0])) > len(golden["mat_f"])


def test_oracle_matches_live_reference_materials(reference, oracle):
    from sdfb import meshgen as mg
    rng = np.random.default_rng(17)
    for seed in range(3):
        n = int(rng.integers(40, 300))
        c = rng.uniform(-0.45, 0.45, size=(n, 1, 3))
        s = rng.lognormal(mean=-2.5, sigma=0.8, size=(n, 1, 1))
        tri = (c + s * rng.normal(size=(n, 3, 3))).reshape(-1, 3).astype(np.float32)
        m = mg.random_materials(n, 100 + seed, num_materials=int(rng.integers(1, 6)))
        lo, hi = tri.min(0), tri.max(0)
        res = int(rng.integers(6, 40))
        cr, kr = reference.voxelize_colors(tri, lo, hi, res, m)
        co, ko = oracle.voxelize_colors(tri, lo, hi, res, m)
        assert np.array_equal(cr, co) and np.array_equal(kr.view(np.uint32), ko.view(np.uint32))
        o, v, nn = reference.grid_from_bounds(lo, hi, res)
        for a, b in zip(reference.materials_dense(tri, o, v, nn, m), oracle.materials_dense(tri, o, v, nn, m)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
