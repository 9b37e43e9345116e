"""Batched bake (several meshes and grids in one launch sequence): every result equals the same
mesh baked alone, bit for bit, and the CUDA graph replay gives the same grids again."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(seed=5, count=7):
    from sdfb import meshgen as mg
    rng = np.random.default_rng(seed)
    meshes, grids = [], []
    import sdfb
    for k in range(count):
        if k % 2:
            v, f = mg.displaced_icosphere(int(rng.integers(1, 5)), 0.3, int(rng.integers(1 << 30)))
        else:
            v, f = mg.displaced_torus(int(rng.integers(8, 40)), int(rng.integers(4, 14)), 0.27, 0.1,
                                      int(rng.integers(1 << 30)))
        n = int(rng.choice([16, 24, 33, 40]))
        meshes.append((v, f))
        grids.append(sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n + (k % 3), n - (k % 2))))
    return meshes, grids


def test_batch_equals_single(ctx):
    import sdfb
    meshes, grids = small_batch()
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY)
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dists, occs = ctx.bake_batch(meshes, grids, opts, stats=st)
    assert st.voxels == sum(g.cells for g in grids)
    for (v, f), g, d, o in zip(meshes, grids, dists, occs):
        d1, o1 = ctx.bake(v, f, g, opts)
        assert np.array_equal(o, o1)
        assert np.array_equal(d, d1)
    # a second identical call replays the captured graph and gives the same grids
    st2 = sdfb.Stats()
    st2.struct_size = sdfb.C.sizeof(sdfb.Stats)
    dists2, occs2 = ctx.bake_batch(meshes, grids, opts, stats=st2)
    assert st2.graph_replayed == 1
    for a, b in zip(dists, dists2):
        assert np.array_equal(a, b)
    for a, b in zip(occs, occs2):
        assert np.array_equal(a, b)


def test_batch_mixed_signs_against_oracle(ctx, oracle):
    """A watertight mesh, a holey soup (winding number) and an unsigned request in one batch."""
    import sdfb
    from sdfb import meshgen as mg
    v1, f1 = mg.displaced_icosphere(3, 0.3, 3)
    v2, f2 = mg.delete_faces(*mg.displaced_torus(30, 10, 0.25, 0.09, 4), 0.06, 5)
    n = 28
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n))
    dists, occs = ctx.bake_batch([(v1, f1), (v2, f2)], [g, g], sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO))
    origin, voxel = (-0.5,) * 3, 1.0 / n
    for (v, f), d, o in zip([(v1, f1), (v2, f2)], dists, occs):
        assert np.array_equal(o.reshape(-1), oracle.occupancy(v, f, origin, voxel, (n, n, n)))
        d64 = oracle.distance(v, f, origin, voxel, (n, n, n))
        assert np.abs(np.abs(d.reshape(-1).astype(np.float64)) - d64).max() <= 1e-5 * np.sqrt(3)
    w = oracle.gwn(v2, f2, origin, voxel, (n, n, n))
    d64 = oracle.distance(v2, f2, origin, voxel, (n, n, n))
    far = (d64 > voxel) & (np.abs(np.abs(w) - 0.5) > 1e-6)
    assert np.array_equal(dists[1].reshape(-1)[far] < 0, np.abs(w[far]) > 0.5)
    sg = oracle.sign_parity(v1, f1, origin, voxel, (n, n, n))
    d64 = oracle.distance(v1, f1, origin, voxel, (n, n, n))
    far = d64 > voxel
    assert np.array_equal(dists[0].reshape(-1)[far] < 0, sg[far] < 0)


def test_batch_device_entry_point(ctx):
    torch = pytest.importorskip("torch")
    import sdfb
    meshes, grids = small_batch(seed=9, count=4)
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY)
    host_d, host_o = ctx.bake_batch(meshes, grids, opts)
    keep = []
    devm, dptr, optr = [], [], []
    for (v, f), g in zip(meshes, grids):
        dv = torch.from_numpy(v).cuda()
        di = torch.from_numpy(f.astype(np.int32)).cuda()
        dd = torch.empty(g.cells, dtype=torch.float32, device="cuda")
        do = torch.empty(g.cells, dtype=torch.uint8, device="cuda")
        keep += [dv, di, dd, do]
        devm.append((dv.data_ptr(), len(v), di.data_ptr(), len(f)))
        dptr.append(dd.data_ptr())
        optr.append(do.data_ptr())
    torch.cuda.synchronize()
    ctx.bake_batch_device(devm, grids, opts, dptr, optr)
    for k, g in enumerate(grids):
        assert np.array_equal(keep[4 * k + 2].cpu().numpy().reshape(g.shape), host_d[k])
        assert np.array_equal(keep[4 * k + 3].cpu().numpy().reshape(g.shape), host_o[k])


def test_pinned_outputs_are_written_in_place(ctx):
    """Pinned distance outputs are written by the distance kernel itself (no copy after the bake);
    the grids equal those returned through pageable buffers, for watertight meshes and for a
    winding-number soup in the same batch (whose distances still go through device memory), and
    for the single-mesh entry point."""
    torch = pytest.importorskip("torch")
    import sdfb
    from sdfb import meshgen as mg
    meshes, grids = small_batch(seed=9, count=5)
    meshes.append(mg.delete_faces(*mg.displaced_torus(30, 10, 0.25, 0.09, 14), 0.06, 15))
    grids.append(sdfb.make_grid((-0.5,) * 3, 1.0 / 28, (28, 29, 27)))
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO)
    ref_d, ref_o = ctx.bake_batch(meshes, grids, opts)

    def pinned(dtype, g):
        return torch.empty(g.cells, dtype=dtype).pin_memory().numpy().reshape(g.shape)

    for _ in range(2):  # the second call replays the captured launch sequence
        hd = [pinned(torch.float32, g) for g in grids]
        ho = [pinned(torch.uint8, g) for g in grids]
        for a in hd:
            a.fill(np.nan)
        ctx.bake_batch(meshes, grids, opts, out=(hd, ho))
        for a, b in zip(hd, ref_d):
            assert np.array_equal(a, b)
        for a, b in zip(ho, ref_o):
            assert np.array_equal(a, b)
    v, f = meshes[1]
    g = grids[1]
    d1, o1 = ctx.bake(v, f, g, opts)
    hd, ho = pinned(torch.float32, g), pinned(torch.uint8, g)
    hd.fill(np.nan)
    ctx.bake(v, f, g, opts, out=(hd, ho))
    assert np.array_equal(hd, d1) and np.array_equal(ho, o1)
    # the reference-shaped soup entry point
    soup = v[f.reshape(-1)].reshape(-1, 3)
    lo, hi = soup.min(axis=0), soup.max(axis=0)
    g0, d0, o0 = ctx.bake_soup(soup, lo, hi, 40, opts)
    tdt = {np.float32: torch.float32, np.uint8: torch.uint8}
    g2, d2, o2 = ctx.bake_soup(soup, lo, hi, 40, opts,
                               alloc=lambda shape, dt: torch.empty(int(np.prod(shape)), dtype=tdt[dt])
                               .pin_memory().numpy().reshape(shape))
    assert g2.shape == g0.shape and np.array_equal(d2, d0) and np.array_equal(o2, o0)


def test_batch_line_of_the_tuning_table(tmp_path, monkeypatch):
    """A "batch tile stack budget" line in the tuning table sets those for every bake of more than
    one mesh; single-mesh bakes keep the per-bucket rows; the grids match the context without it."""
    import sdfb
    table = tmp_path / "t.tsv"
    table.write_text("# test table\n0 0 4 0 64 1024\nbatch 1 32 0\n")
    monkeypatch.setenv("SDFB_TUNING", str(table))
    ctx_b = sdfb.Context(0)
    table.write_text("# test table\n0 0 4 0 64 1024\n")
    ctx_p = sdfb.Context(0)
    try:
        meshes, grids = small_batch(seed=9, count=4)
        opts = sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY)
        sts = []
        outs = []
        for c in (ctx_b, ctx_p):
            st = sdfb.Stats()
            st.struct_size = sdfb.C.sizeof(sdfb.Stats)
            outs.append(c.bake_batch(meshes, grids, opts, stats=st))
            sts.append(st)
        assert (sts[0].tile_used, sts[0].stack_used) == (2, 32)
        assert sts[1].tile_used == 3  # the built-in default (tile id 2 + 1) for buckets the table lacks
        (db, ob), (dp, op) = outs
        for a, b in zip(ob, op):
            assert np.array_equal(a, b)
        for a, b in zip(db, dp):
            assert np.abs(a - b).max() <= 4e-7 and np.array_equal(a < 0, b < 0)
        st = sdfb.Stats()
        st.struct_size = sdfb.C.sizeof(sdfb.Stats)
        ctx_b.bake(*meshes[0], grids[0], opts, stats=st)
        assert st.tile_used == 3  # one mesh: no batch line
    finally:
        ctx_b.close()
        ctx_p.close()


def test_winding_number_batch_replays_its_graph(ctx):
    """A batch holding a mesh with holes (winding-number sign, caps built on the device before the
    launch sequence) is captured once and replayed, with the same grids."""
    import sdfb
    from sdfb import meshgen as mg
    v1, f1 = mg.displaced_icosphere(3, 0.3, 13)
    v2, f2 = mg.delete_faces(*mg.displaced_torus(30, 10, 0.25, 0.09, 14), 0.06, 15)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 28, (28, 28, 28))
    opts = sdfb.make_opts(sign_mode=sdfb.SIGN_AUTO)
    runs = []
    for _ in range(2):
        st = sdfb.Stats()
        st.struct_size = sdfb.C.sizeof(sdfb.Stats)
        runs.append((ctx.bake_batch([(v1, f1), (v2, f2)], [g, g], opts, stats=st), st.graph_replayed))
    (d0, o0), _ = runs[0]
    (d1, o1), replayed = runs[1]
    assert replayed == 1
    for a, b in zip(d0 + o0, d1 + o1):
        assert np.array_equal(a, b)
    assert (d1[1] < 0).any()  # the holey torus has inside cells (winding-number sign)
