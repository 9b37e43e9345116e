"""Winding-number sign on meshes with holes (needs an sm_103 device).

The oracle sums every triangle's solid angle in FP64; the bake's sign must equal |w| > 0.5 for
every cell farther than one voxel from the surface whose oracle winding number is not within
1e-6 of 0.5 (such cells sit on the w = 0.5 level set and have no robust sign)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIST_TOL = 1e-5


def holey_soup(seed: int, sphere_level=3, torus=(48, 16), fraction=0.05):
    from sdfb import meshgen as mg
    rng = np.random.default_rng(seed)
    parts = [mg.displaced_icosphere(sphere_level, 0.22, int(rng.integers(1 << 30)), center=(-0.15, 0.05, 0.0)),
             mg.displaced_torus(torus[0], torus[1], 0.2, 0.07, int(rng.integers(1 << 30)), center=(0.18, -0.1, 0.05))]
    v, f = mg.concat(parts)
    return mg.delete_faces(v, f, fraction, int(rng.integers(1 << 30)))


@pytest.mark.parametrize("seed,n,dims", [(3, 40, None), (4, 56, None), (5, 44, (37, 41, 29))])
def test_gwn_sign_matches_fp64_oracle(ctx, oracle, seed, n, dims):
    """dims: a grid whose edges are not multiples of the winding-number tile (4 x 4 x 8 cells)."""
    import sdfb
    v, f = holey_soup(seed)
    origin, voxel = (-0.5,) * 3, 1.0 / n
    dims = dims or (n, n, n)
    grid = sdfb.make_grid(origin, voxel, dims)
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dist, occ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO), stats=st)
    assert st.watertight == 0 and st.sign_mode_used == sdfb.SIGN_GWN
    assert st.gwn_fp64_cells > 0
    flat = dist.reshape(-1)
    d64 = oracle.distance(v, f, origin, voxel, dims)
    assert np.abs(np.abs(flat.astype(np.float64)) - d64).max() <= DIST_TOL * np.sqrt(3)
    assert np.array_equal(occ.reshape(-1), oracle.occupancy(v, f, origin, voxel, dims))
    w = oracle.gwn(v, f, origin, voxel, dims)
    far = (d64 > voxel) & (np.abs(np.abs(w) - 0.5) > 1e-6)
    bad = np.count_nonzero((flat[far] < 0) != (np.abs(w[far]) > 0.5))
    assert bad == 0, f"{bad} winding-number sign mismatches outside the band"
    # in the band the FP64 pass decides; report, and require near-total agreement
    near = (d64 <= voxel) & (np.abs(np.abs(w) - 0.5) > 1e-6)
    bad_near = np.count_nonzero((flat[near] < 0) != (np.abs(w[near]) > 0.5))
    assert bad_near <= max(2, near.sum() // 1000)


def _holes_meeting_at_vertices(level=3, seed=8):
    """A displaced icosphere with (a) two holes that share exactly one vertex (a boundary vertex with
    two arriving and two leaving boundary half-edges, where the cap loops can be split either way),
    (b) every triangle around another vertex removed (one long loop), and (c) a second sphere
    inside the first, with one triangle removed."""
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(level, 0.3, seed)
    f = np.asarray(f, np.int64)
    # (a) two faces meeting only at vertex x
    x = int(f[0, 0])
    around = [t for t in range(len(f)) if x in f[t]]
    a = around[0]
    b = next(t for t in around[1:] if len(set(f[t]) & set(f[a])) == 1)
    # (b) the fan of the vertex farthest from x
    y = int(np.argmax(np.linalg.norm(np.asarray(v, np.float64) - np.asarray(v[x], np.float64), axis=1)))
    fan = [t for t in range(len(f)) if y in f[t]]
    drop = set([a, b] + fan)
    keep = np.array([t for t in range(len(f)) if t not in drop])
    outer_v, outer_f = v, f[keep]
    iv, ifc = mg.displaced_icosphere(2, 0.12, seed + 1, center=(0.05, 0.0, 0.02))
    ifc = np.asarray(ifc, np.int64)[1:]
    return mg.concat([(outer_v, outer_f), (iv, ifc)])


def test_device_caps_on_loops_that_share_vertices(ctx, oracle):
    """The caps built on the device close loops that meet at a vertex and long loops; every cell
    outside the band gets the FP64 winding number's sign."""
    import sdfb
    v, f = _holes_meeting_at_vertices()
    n = 48
    origin, voxel = (-0.5,) * 3, 1.0 / n
    grid = sdfb.make_grid(origin, voxel, (n, n, n))
    dist, _ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_GWN))
    flat = dist.reshape(-1)
    d64 = oracle.distance(v, f, origin, voxel, (n, n, n))
    w = oracle.gwn(v, f, origin, voxel, (n, n, n))
    far = (d64 > voxel) & (np.abs(np.abs(w) - 0.5) > 1e-6)
    assert far.sum() > 0.9 * flat.size
    bad = np.count_nonzero((flat[far] < 0) != (np.abs(w[far]) > 0.5))
    assert bad == 0, f"{bad} sign mismatches outside the band"
    # both spheres' interiors are inside (the holes do not open them)
    assert flat[(24 * n + 24) * n + 27] < 0


def test_gwn_equals_parity_on_closed_mesh(ctx):
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(4, 0.33, 21)
    grid = sdfb.make_grid((-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    dp, _ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY))
    dg, _ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_GWN))
    assert np.array_equal(np.abs(dp), np.abs(dg))
    far = np.abs(dp) > 1.0 / 64
    assert np.array_equal(dp[far] < 0, dg[far] < 0)
    near = ~far
    assert np.count_nonzero((dp[near] < 0) != (dg[near] < 0)) <= 2


def test_gwn_band_width_option(ctx):
    import sdfb
    v, f = holey_soup(7)
    grid = sdfb.make_grid((-0.5,) * 3, 1.0 / 40, (40, 40, 40))
    s1, s3 = sdfb.Stats(), sdfb.Stats()
    s1.struct_size = s3.struct_size = sdfb.C.sizeof(sdfb.Stats)
    d1, _ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_GWN, band_voxels=1.0), stats=s1)
    d3, _ = ctx.bake(v, f, grid, sdfb.make_opts(sign_mode=sdfb.SIGN_GWN, band_voxels=3.0), stats=s3)
    assert s3.gwn_fp64_cells > s1.gwn_fp64_cells
    assert np.array_equal(np.abs(d1), np.abs(d3))


def test_c3_soup_full_size(ctx, oracle):
    """The 500k-triangle soup with 2% of its faces deleted, on the 512^3 grid: occupancy on every
    cell, distance on a seeded 20,000-cell sample against FP64, winding-number sign on a seeded
    sample of 3,000 cells outside the band and 1,000 band cells against the FP64 direct sum."""
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.soup_with_holes()
    n = (512, 512, 512)
    origin, voxel = (-0.5,) * 3, 1.0 / 512
    g = sdfb.make_grid(origin, voxel, n)
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dist, occ = ctx.bake(v, f, g, sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO), stats=st)
    assert st.sign_mode_used == sdfb.SIGN_GWN and st.watertight == 0
    assert np.array_equal(occ.reshape(-1), oracle.occupancy(v, f, origin, voxel, n))
    flat = dist.reshape(-1)
    rng = np.random.default_rng(33)
    samp = np.sort(rng.choice(flat.size, 20000, replace=False)).astype(np.int64)
    d64 = oracle.distance(v, f, origin, voxel, n, samples=samp)
    assert np.abs(np.abs(flat[samp].astype(np.float64)) - d64).max() <= DIST_TOL * np.sqrt(3)
    far = samp[d64 > voxel][:3000]
    w = oracle.gwn(v, f, origin, voxel, n, samples=far)
    ok = np.abs(np.abs(w) - 0.5) > 1e-6
    assert np.count_nonzero((flat[far][ok] < 0) != (np.abs(w[ok]) > 0.5)) == 0
    band = np.flatnonzero(np.abs(flat) <= voxel)
    band = np.sort(rng.choice(band, min(1000, band.size), replace=False)).astype(np.int64)
    wb = oracle.gwn(v, f, origin, voxel, n, samples=band)
    okb = np.abs(np.abs(wb) - 0.5) > 1e-6
    assert np.count_nonzero((flat[band][okb] < 0) != (np.abs(wb[okb]) > 0.5)) <= 2
