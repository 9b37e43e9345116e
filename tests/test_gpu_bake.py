"""GPU bake parity against the oracle and the reference's fixtures (needs an sm_103 device).

Bars: occupancy bit-exact; unsigned distance within 1e-5 of the grid diagonal of the FP64
oracle; sign bit-exact for every cell farther than one voxel from the surface.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import grid_of, unpack

pytestmark = pytest.mark.gpu

DIST_TOL = 1e-5  # of the grid diagonal


def diag(voxel, n):
    return float(voxel) * float(np.sqrt(sum(float(x) ** 2 for x in n)))


def check_bake(oracle, verts, idx, origin, voxel, n, dist, occ, occ_ref=None, sign_axis=2, samples=None):
    """Asserts the three bars; returns (max err / diag, out-of-band sign mismatches, in-band ones)."""
    flat = dist.reshape(-1)
    if occ_ref is None:
        occ_ref = oracle.occupancy(verts, idx, origin, voxel, n)
    assert np.array_equal(occ.reshape(-1), occ_ref.reshape(-1)), "occupancy differs from the reference rule"
    if samples is None:
        d64 = oracle.distance(verts, idx, origin, voxel, n)
        got = flat
    else:
        d64 = oracle.distance(verts, idx, origin, voxel, n, samples=samples)
        got = flat[samples]
    err = np.abs(np.abs(got.astype(np.float64)) - d64)
    tol = DIST_TOL * diag(voxel, n)
    assert err.max() <= tol, f"max distance error {err.max()} > {tol}"
    sgn = oracle.sign_parity(verts, idx, origin, voxel, n, axis=sign_axis)
    if samples is not None:
        sgn = sgn[samples]
    far = d64 > voxel
    bad_far = int(np.count_nonzero((got[far] < 0) != (sgn[far] < 0)))
    assert bad_far == 0, f"{bad_far} sign mismatches outside the band"
    bad_near = int(np.count_nonzero((got[~far] < 0) != (sgn[~far] < 0)))
    return err.max() / diag(voxel, n), bad_far, bad_near


def test_c1_plain_bake(ctx, oracle, golden):
    import sdfb
    v, i = golden["c1_verts"], golden["c1_idx"]
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dist, occ = ctx.bake(v, i, g, sdfb.make_opts(), stats=st)
    assert st.sign_mode_used == sdfb.SIGN_PARITY and st.watertight == 1
    check_bake(oracle, v, i, (-0.5,) * 3, 1.0 / 64, (64, 64, 64), dist, occ,
               occ_ref=unpack(golden["c1_occ"], 64 ** 3))
    # the committed FP64 samples too
    s = golden["c1_samples"]
    assert np.abs(np.abs(dist.reshape(-1)[s]) - golden["c1_dist64_samples"]).max() <= DIST_TOL * np.sqrt(3)
    far = np.abs(dist.reshape(-1)) > (1.0 / 64) * (1 + 1e-3)
    assert np.array_equal(dist.reshape(-1)[far] < 0, unpack(golden["c1_sign"], 64 ** 3).astype(bool)[far])


def test_sign_test_sphere(ctx, oracle, golden):
    """tests/sdf_sign_test.cpp:46-83 through the soup entry point (bakeSdf sizing, res 24)."""
    import sdfb
    soup = golden["sphere1_soup"]
    g, dist, occ = ctx.bake_soup(soup, (-1, -1, -1), (1, 1, 1), 24)
    o, vx, n = grid_of(golden["sphere1_grid"])
    assert (g.nx, g.ny, g.nz) == n and np.float32(g.voxel_size) == np.float32(vx)
    assert np.array_equal(occ.reshape(-1), unpack(golden["sphere1_occ"], occ.size))
    d64 = golden["sphere1_dist64"]
    assert np.abs(np.abs(dist.reshape(-1)) - d64).max() <= DIST_TOL * diag(vx, n)
    xs = [np.float32(o[a]) + (np.arange(n[a], dtype=np.float32) + np.float32(0.5)) * np.float32(vx) for a in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    an = (np.sqrt(X.astype(np.float64) ** 2 + Y ** 2 + Z ** 2) - 1.0).reshape(-1)
    far = np.abs(an) > 1.5 * vx
    assert far.sum() > 0
    assert np.all((an[far] < 0) == (dist.reshape(-1)[far] < 0))
    assert np.abs(dist.reshape(-1)[far] - an[far]).max() < 2.0 * 1.5 * vx
    sg = golden["sphere1_sign"]
    out = d64 > vx
    assert np.array_equal(dist.reshape(-1)[out] < 0, sg[out] < 0)


@pytest.mark.parametrize("name,grid", [
    ("cube_aligned_occ", ((0.0, 0.0, 0.0), 0.125, (8, 8, 8))),
    ("cube_aligned_occ_shift", ((-0.0625,) * 3, 0.125, (10, 10, 10)))])
def test_cube_occupancy_ties(ctx, golden, name, grid):
    import sdfb
    soup = golden["cube_soup"]
    idx = np.arange(len(soup), dtype=np.uint32).reshape(-1, 3)
    g = sdfb.make_grid(*grid)
    _, occ = ctx.bake(soup, idx, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE), want_dist=False)
    assert np.array_equal(occ.reshape(-1), unpack(golden[name], occ.size))


def test_cube_soup_bake_and_watertight_gate(ctx, oracle, golden):
    import sdfb
    soup = golden["cube_soup"]
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    g, dist, occ = ctx.bake_soup(soup, (0, 0, 0), (1, 1, 1), 8, stats=st)
    assert st.watertight == 1 and st.sign_mode_used == sdfb.SIGN_PARITY
    o, v, n = grid_of(golden["cube_grid"])
    assert np.array_equal(occ.reshape(-1), unpack(golden["cube_occ"], occ.size))
    idx = np.arange(len(soup), dtype=np.uint32).reshape(-1, 3)
    check_bake(oracle, soup, idx, o, v, n, dist, occ)


def test_sparse_voxelize_order(ctx, golden):
    """The reference's voxelizeMesh cell list, in its insertion order."""
    cells, org, vox = ctx.voxelize_sparse(golden["cube_soup"], (0, 0, 0), (1, 1, 1), 8)
    assert np.array_equal(cells, golden["cube_sparse_cells"])
    assert np.float32(vox) == np.float32(golden["cube_sparse_voxel"])
    b = golden["rsoup_sparse_bounds"]
    cells, _, _ = ctx.voxelize_sparse(golden["rsoup"], b[0], b[1], 40)
    assert np.array_equal(cells, golden["rsoup_sparse_cells"])


def test_random_soup_unsigned(ctx, oracle, golden):
    import sdfb
    soup = golden["rsoup"]
    idx = np.arange(len(soup), dtype=np.uint32).reshape(-1, 3)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 32, (32, 32, 32))
    dist, occ = ctx.bake(soup, idx, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
    assert np.array_equal(occ.reshape(-1), unpack(golden["rsoup_occ"], occ.size))
    d64 = oracle.distance(soup, idx, (-0.5,) * 3, 1.0 / 32, (32, 32, 32))
    assert np.all(dist >= 0)
    assert np.abs(dist.reshape(-1) - d64).max() <= DIST_TOL * np.sqrt(3)


@pytest.mark.parametrize("leaf", [1, 2, 4, 8, 16])
def test_leaf_sizes_and_tiles_agree(ctx, golden, leaf):
    import sdfb
    v, i = golden["c1_verts"], golden["c1_idx"]
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 48, (48, 40, 36))
    ref_d, ref_o = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, leaf_size=1, tile=1))
    for tile in range(1, 7):
        d, o = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, leaf_size=leaf, tile=tile))
        assert np.array_equal(o, ref_o)
        # the same nearest triangle whichever way the tree is walked (a culling decision taken on an
        # FP32 box bound may only differ by rounding)
        assert np.abs(d - ref_d).max() <= 4e-7 and np.array_equal(d < 0, ref_d < 0)


def test_displaced_sphere_full_size(ctx, oracle):
    """Level-6 displaced icosphere (81,920 triangles) at 256^3: occupancy and sign on every cell,
    distance on a seeded sample of 20,000 cells against FP64."""
    import sdfb
    from sdfb import meshgen as mg
    v, i = mg.displaced_sphere_mesh()
    n = (256, 256, 256)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 256, n)
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dist, occ = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY), stats=st)
    occ_ref = oracle.occupancy(v, i, (-0.5,) * 3, 1.0 / 256, n)
    assert np.array_equal(occ.reshape(-1), occ_ref)
    rng = np.random.default_rng(12)
    samp = np.sort(rng.choice(256 ** 3, 20000, replace=False)).astype(np.int64)
    d64 = oracle.distance(v, i, (-0.5,) * 3, 1.0 / 256, n, samples=samp)
    flat = dist.reshape(-1)
    assert np.abs(np.abs(flat[samp]) - d64).max() <= DIST_TOL * np.sqrt(3)
    # sign on all 16.8M cells against the oracle's exact parity, outside the band
    sgn = oracle.sign_parity(v, i, (-0.5,) * 3, 1.0 / 256, n, axis=2)
    far = np.abs(flat) > (1.0 / 256) * (1 + 1e-3)
    assert np.array_equal(flat[far] < 0, sgn[far] < 0)
    # size-independent property: inside cells are exactly the cells below an odd number of crossings
    # of the +z column; the interior is one connected blob around the centre
    assert flat[(128 * 256 + 128) * 256 + 128] < 0 and flat[0] > 0


def test_million_triangle_torus_every_cell(ctx, oracle):
    """The heaviest meshes of the batch are 1M-triangle tori: one (1,048,576 triangles) at 128^3
    against FP64 on every cell -- occupancy bit-exact, distance within 1e-5 of the diagonal, sign
    exact outside one voxel -- through the single-mesh path and inside a batch with a small mesh."""
    import sdfb
    from sdfb import meshgen as mg
    v, i = mg.displaced_torus(1024, 512, 0.3, 0.1, 1114)
    assert len(i) == 1 << 20
    n = (128, 128, 128)
    origin, voxel = (-0.5,) * 3, 1.0 / 128
    g = sdfb.make_grid(origin, voxel, n)
    dist, occ = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY))
    err, _, _ = check_bake(oracle, v, i, origin, voxel, n, dist, occ)
    assert err <= DIST_TOL
    small_v, small_i = mg.displaced_icosphere(3, 0.3, 5)
    gs = sdfb.make_grid(origin, 1.0 / 32, (32, 32, 32))
    (bd, _), (bo, _) = ctx.bake_batch([(v, i), (small_v, small_i)], [g, gs],
                                      sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY))
    assert np.array_equal(bo, occ)
    assert np.abs(bd - dist).max() <= DIST_TOL * np.sqrt(3)


def test_grid_edge_cases(ctx, oracle):
    import sdfb
    tri_v = np.array([[0.1, 0.1, 0.1], [0.3, 0.1, 0.2], [0.1, 0.35, 0.3]], np.float32)
    tri_i = np.array([[0, 1, 2]], np.uint32)
    for origin, voxel, n in [((0, 0, 0), 0.05, (1, 1, 1)), ((0, 0, 0), 0.05, (7, 5, 3)),
                             ((0.5, 0.5, 0.5), 0.1, (9, 9, 9)), ((-1, -1, -1), 0.013, (33, 17, 65))]:
        g = sdfb.make_grid(origin, voxel, n)
        dist, occ = ctx.bake(tri_v, tri_i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
        occ_ref = oracle.occupancy(tri_v, tri_i, origin, np.float32(voxel), n)
        assert np.array_equal(occ.reshape(-1), occ_ref)
        d64 = oracle.distance(tri_v, tri_i, origin, np.float32(voxel), n)
        assert np.abs(dist.reshape(-1) - d64).max() <= DIST_TOL * diag(np.float32(voxel), n)


def test_degenerate_triangles(ctx, oracle):
    """Zero-area triangles (collinear and repeated vertices, as at the UV sphere's poles)."""
    import sdfb
    v = np.array([[0, 0, 0], [0.2, 0.1, 0.0], [0.4, 0.2, 0.0], [0.1, 0.3, 0.2], [0.1, 0.3, 0.2]], np.float32)
    i = np.array([[0, 1, 2], [3, 4, 0], [2, 2, 2]], np.uint32)
    n = (16, 16, 16)
    g = sdfb.make_grid((-0.2,) * 3, 0.05, n)
    dist, occ = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
    d64 = oracle.distance(v, i, (-0.2,) * 3, np.float32(0.05), n)
    assert np.abs(dist.reshape(-1) - d64).max() <= DIST_TOL * diag(np.float32(0.05), n)
    assert np.array_equal(occ.reshape(-1), oracle.occupancy(v, i, (-0.2,) * 3, np.float32(0.05), n))


def test_hard_triangles(ctx, oracle):
    """Slivers, needles, nearly collinear and mixed-scale triangles (each distance record holds
    its triangle in a frame along the longest edge), then the same soup and grid moved to 1000 on
    every axis, where FP32 coordinates keep only about 4 decimals: unsigned distances against the
    FP64 oracle on the same FP32 inputs."""
    import sdfb
    rng = np.random.default_rng(11)
    tris = []
    for k in range(250):
        a = rng.uniform(-0.4, 0.4, 3)
        b = a + rng.normal(0.0, 0.15, 3)
        kind = k % 5
        if kind == 0:  # sliver: C within 1e-7 .. 1e-3 of the segment AB
            c = a + 0.5 * (b - a) + rng.normal(0.0, 1.0, 3) * 10.0 ** rng.uniform(-7, -3)
        elif kind == 1:  # needle: C next to B
            c = b + rng.normal(0.0, 1.0, 3) * 1e-6
        elif kind == 2:  # collinear up to rounding, C anywhere on the line
            c = a + rng.uniform(-1.0, 2.0) * (b - a)
        elif kind == 3:  # one short edge AB, C far away
            b = a + (b - a) * 1e-3
            c = a + rng.normal(0.0, 0.3, 3)
        else:
            c = a + rng.normal(0.0, 0.15, 3)
        tris.append([a, b, c])
    v = np.asarray(tris, np.float64).reshape(-1, 3)
    i = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
    n = (24, 24, 24)
    voxel = np.float32(1.0 / 24)
    for shift in (0.0, 1000.0):
        vv = (v + shift).astype(np.float32)
        origin = (np.float32(-0.5 + shift),) * 3
        g = sdfb.make_grid(origin, voxel, n)
        dist, _ = ctx.bake(vv, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
        d64 = oracle.distance(vv, i, origin, voxel, n)
        err = np.abs(dist.reshape(-1).astype(np.float64) - d64).max()
        assert err <= DIST_TOL * diag(voxel, n), (shift, err)


def test_error_paths(ctx):
    import sdfb
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    g = sdfb.make_grid((0, 0, 0), 0.25, (4, 4, 4))
    st, msg = ctx.bake_status(v, np.array([[0, 1, 3]], np.uint32), g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
    assert st == sdfb.ERR_BAD_MESH and "index" in msg
    vn = v.copy()
    vn[1, 0] = np.nan
    st, msg = ctx.bake_status(vn, np.array([[0, 1, 2]], np.uint32), g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
    assert st == sdfb.ERR_BAD_MESH
    st, msg = ctx.bake_status(v, np.zeros((0, 3), np.uint32), g)
    assert st == sdfb.ERR_BAD_MESH
    bad = sdfb.make_grid((0, 0, 0), 0.0, (4, 4, 4))
    st, msg = ctx.bake_status(v, np.array([[0, 1, 2]], np.uint32), bad)
    assert st == sdfb.ERR_INVALID_ARGUMENT
    # the context is still usable after errors
    d, o = ctx.bake(v, np.array([[0, 1, 2]], np.uint32), g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE))
    assert np.isfinite(d).all()


def test_deterministic(ctx):
    import sdfb
    from sdfb import meshgen as mg
    v, i = mg.displaced_icosphere(4, 0.3, 77)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 96, (96, 96, 96))
    a = ctx.bake(v, i, g, sdfb.make_opts())
    b = ctx.bake(v, i, g, sdfb.make_opts())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_device_entry_point_matches_host(ctx):
    torch = pytest.importorskip("torch")
    import sdfb
    from sdfb import meshgen as mg
    v, i = mg.displaced_icosphere(3, 0.3, 9)
    n = (40, 48, 56)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 48, n)
    hd, ho = ctx.bake(v, i, g, sdfb.make_opts())
    dv = torch.from_numpy(v).cuda()
    di = torch.from_numpy(i.astype(np.int32)).cuda()
    dd = torch.empty(n[2] * n[1] * n[0], dtype=torch.float32, device="cuda")
    do = torch.empty(n[2] * n[1] * n[0], dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.bake_device(dv.data_ptr(), len(v), di.data_ptr(), len(i), g, sdfb.make_opts(), dd.data_ptr(), do.data_ptr())
    assert np.array_equal(dd.cpu().numpy().reshape(hd.shape), hd)
    assert np.array_equal(do.cpu().numpy().reshape(ho.shape), ho)


@pytest.mark.parametrize("tile", [1, 3, 6])
def test_deferred_tiles_agree(ctx, tile):
    """Tiles still walking when every tile has been handed out are finished by a block-per-tile
    pass that splits the tree into subtrees; the result must not depend on it. With a budget of 8
    steps nearly every tile in flight at the end is deferred; budget -1 defers none."""
    import sdfb
    from sdfb import meshgen as mg
    v, i = mg.displaced_icosphere(5, 0.4, 7)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 128, (128, 128, 128))
    out = {}
    for budget in (-1, 8):
        st = sdfb.Stats()
        st.struct_size = sdfb.C.sizeof(sdfb.Stats)
        d, o = ctx.bake(v, i, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, tile=tile, step_budget=budget), stats=st)
        out[budget] = (d, o, st.tiles_deferred)
    assert out[-1][2] == 0 and out[8][2] > 100
    assert np.array_equal(out[-1][1], out[8][1])
    # the same nearest triangle; a culling decision on an FP32 box bound may only differ by rounding
    assert np.abs(out[-1][0] - out[8][0]).max() <= 4e-7 and np.array_equal(out[-1][0] < 0, out[8][0] < 0)
