"""Serving loop: continuous batching over resident meshes. A served result equals the same
request alone, and the same bake run through the plain entry point, within the tolerance: occupancy
and signs identical, distances up to rounding (4e-7). A wave takes its launch parameters (tile
shape, stack depth, deferral budget) from its largest grid, the resident hierarchy is built with
the leaf size tuned for a 256^3 grid while a plain bake tunes for its own grid, and where two
triangles nearly tie with an FP32 box bound, walks in a different order may keep either. With the
same launch parameters the served result is bit-identical to the request alone."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def assert_same_bake(d, o, d1, o1):
    """Occupancy and signs identical; distances equal up to the last bits (the bound the
    leaf-size and tile-shape test uses)."""
    assert np.array_equal(o, o1)
    assert np.array_equal(np.signbit(d), np.signbit(d1))
    assert np.abs(d - d1).max() <= 4e-7


def test_served_equals_plain_in_the_mix(ctx):
    import sdfb
    from sdfb import meshgen as mg
    meshes = [mg.displaced_icosphere(3, 0.3, 1), mg.displaced_torus(40, 12, 0.27, 0.1, 2),
              mg.displaced_icosphere(4, 0.33, 3)]
    sizes = [24, 40, 56, 32, 48, 64, 24, 40, 72, 16]
    with sdfb.Server(ctx, max_inflight=6, wave_voxels_log2=17) as srv:
        ids = [srv.register(v, f) for v, f in meshes]
        assert srv.register(*meshes[1]) == ids[1]  # identical contents: the resident copy
        alone = []
        for k in range(3):  # each mesh alone in its wave first
            n = sizes[k]
            g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n + 1, n - 1))
            d = np.empty(g.shape, np.float32)
            o = np.empty(g.shape, np.uint8)
            assert srv.poll(srv.submit(ids[k], g, d, o), 60000)[0]
            alone.append((d, o))
        reqs = []
        for k, n in enumerate(sizes):
            g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n + 1, n - 1))
            d = np.empty(g.shape, np.float32)
            o = np.empty(g.shape, np.uint8)
            reqs.append((srv.submit(ids[k % 3], g, d, o), k % 3, g, d, o))
        infos = []
        for k, (rid, m, g, d, o) in enumerate(reqs):
            done, info = srv.poll(rid, 60000)
            assert done and info["status"] == 0
            infos.append(info)
            if k < 3:  # the same request in a mixed wave (here with its lone launch parameters)
                assert np.array_equal(d, alone[k][0]) and np.array_equal(o, alone[k][1])
            d1, o1 = ctx.bake(*meshes[m], g, sdfb.make_opts())
            assert_same_bake(d, o, d1, o1)
        assert all(i["t_submit_ms"] <= i["t_admit_ms"] <= i["t_done_ms"] for i in infos)


def test_served_gwn_mesh(ctx):
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.delete_faces(*mg.displaced_icosphere(3, 0.3, 8), 0.05, 9)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 36, (36, 36, 36))
    with sdfb.Server(ctx) as srv:
        mid = srv.register(v, f)
        d = np.empty(g.shape, np.float32)
        o = np.empty(g.shape, np.uint8)
        rid = srv.submit(mid, g, d, o)
        done, info = srv.poll(rid, 60000)
        assert done
    d1, o1 = ctx.bake(v, f, g, sdfb.make_opts())
    assert_same_bake(d, o, d1, o1)


def test_budget_evicts_least_recently_used(ctx):
    import sdfb
    from sdfb import meshgen as mg
    ms = [mg.displaced_icosphere(4, 0.3, s) for s in range(3)]  # 5,120 triangles each
    per_mesh = 5120 * 160
    with sdfb.Server(ctx, hbm_budget_bytes=int(per_mesh * 2.5)) as srv:
        a = srv.register(*ms[0])
        b = srv.register(*ms[1])
        srv.register(*ms[0])  # touch a: b is now the least recently used
        c = srv.register(*ms[2])  # evicts b
        g = sdfb.make_grid((-0.5,) * 3, 1.0 / 8, (8, 8, 8))
        d = np.empty(g.shape, np.float32)
        with pytest.raises(sdfb.SdfbError) as e:
            srv.submit(b, g, d, None)
        assert e.value.status == sdfb.ERR_NOT_FOUND
        for mid in (a, c):
            rid = srv.submit(mid, g, d, None)
            assert srv.poll(rid, 60000)[0]
        with pytest.raises(sdfb.SdfbError) as e:
            srv.register(*mg.displaced_icosphere(6, 0.3, 4))  # larger than the whole budget
        assert e.value.status == sdfb.ERR_OUT_OF_MEMORY


def test_pinned_outputs(ctx):
    torch = pytest.importorskip("torch")
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_torus(30, 10, 0.27, 0.1, 5)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 40, (40, 40, 40))
    d = torch.empty(g.cells, dtype=torch.float32).pin_memory().numpy().reshape(g.shape)
    o = torch.empty(g.cells, dtype=torch.uint8).pin_memory().numpy().reshape(g.shape)
    with sdfb.Server(ctx) as srv:
        rid = srv.submit(srv.register(v, f), g, d, o)
        assert srv.poll(rid, 60000)[0]
    d1, o1 = ctx.bake(v, f, g, sdfb.make_opts())
    assert_same_bake(d, o, d1, o1)


def test_concurrent_registration_of_the_same_mesh(ctx):
    """Many threads register a few meshes at once and submit right away (the serving stream's
    repeats): registrations of different meshes overlap in the registration slots, each mesh is
    built once, and every result equals the plain bake."""
    import threading

    import sdfb
    from sdfb import meshgen as mg
    meshes = [mg.displaced_icosphere(4, 0.3, 21), mg.displaced_torus(60, 20, 0.27, 0.1, 22),
              mg.displaced_icosphere(3, 0.35, 23), mg.displaced_torus(40, 16, 0.3, 0.08, 24)]
    n = 40
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n))
    ref = [ctx.bake(v, f, g, sdfb.make_opts()) for v, f in meshes]
    errors, results = [], []
    with sdfb.Server(ctx, max_inflight=8, wave_voxels_log2=18) as srv:
        start = threading.Barrier(16)

        def worker(k):
            try:
                v, f = meshes[k % 4]
                start.wait()
                mid = srv.register(v, f)
                d = np.empty(g.shape, np.float32)
                o = np.empty(g.shape, np.uint8)
                done, info = srv.poll(srv.submit(mid, g, d, o), 60000)
                results.append((k % 4, done, info["status"], d, o))
            except Exception as e:  # reported below
                errors.append(repr(e))

        threads = [threading.Thread(target=worker, args=(k,)) for k in range(16)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    assert not errors, errors[0]
    assert len(results) == 16
    for m, done, status, d, o in results:
        assert done and status == 0
        assert_same_bake(d, o, ref[m][0], ref[m][1])


def test_admission_evicts_and_always_progresses(ctx):
    """Registered meshes may fill the budget; admitting a request then evicts unreferenced meshes
    for its outputs, and a request larger than what is left is still admitted when nothing else
    is in flight."""
    import sdfb
    from sdfb import meshgen as mg
    ms = [mg.displaced_icosphere(4, 0.3, 40 + s) for s in range(2)]
    per_mesh = 5120 * 160
    with sdfb.Server(ctx, hbm_budget_bytes=int(per_mesh * 2.2)) as srv:
        a = srv.register(*ms[0])
        b = srv.register(*ms[1])
        for n in (40, 96):  # 40^3 outputs need an eviction; 96^3 outputs exceed the whole budget
            g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n))
            d = np.empty(g.shape, np.float32)
            o = np.empty(g.shape, np.uint8)
            done, info = srv.poll(srv.submit(b, g, d, o), 60000)
            assert done and info["status"] == 0
            d1, o1 = ctx.bake(*ms[1], g, sdfb.make_opts())
            assert_same_bake(d, o, d1, o1)
        del a


def test_close_with_requests_queued(ctx):
    """Closing the server cancels what is still queued and returns."""
    import threading

    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(4, 0.3, 50)
    srv = sdfb.Server(ctx, max_inflight=1, wave_voxels_log2=12)
    mid = srv.register(v, f)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 64, (64, 64, 64))
    bufs = [(np.empty(g.shape, np.float32), np.empty(g.shape, np.uint8)) for _ in range(20)]
    for d, o in bufs:
        srv.submit(mid, g, d, o)
    t = threading.Thread(target=srv.close, daemon=True)
    t.start()
    t.join(60)
    assert not t.is_alive()


def test_registration_while_waves_run(ctx):
    """New meshes registered while other threads keep waves in flight (registrations run on
    high-priority streams beside the waves; a wave holding a new mesh may take other launch
    parameters): every result of the resident mesh matches it alone within the tolerance, and each
    new mesh's result matches its plain bake."""
    import threading

    import sdfb
    from sdfb import meshgen as mg
    base = mg.displaced_torus(64, 24, 0.27, 0.1, 21)
    news = [mg.displaced_icosphere(4, 0.28, 30 + k) for k in range(4)]
    n = 48
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n))
    with sdfb.Server(ctx) as srv:
        mid = srv.register(*base)
        d0 = np.empty(g.shape, np.float32)
        o0 = np.empty(g.shape, np.uint8)
        assert srv.poll(srv.submit(mid, g, d0, o0), 60000)[0]
        outs, errors, stop = [], [], threading.Event()

        def busy():
            try:
                while not stop.is_set():
                    d = np.empty(g.shape, np.float32)
                    o = np.empty(g.shape, np.uint8)
                    done, info = srv.poll(srv.submit(mid, g, d, o), 60000)
                    assert done and info["status"] == 0
                    outs.append((d, o))
            except Exception as e:  # reported on the main thread
                errors.append(e)

        th = [threading.Thread(target=busy) for _ in range(3)]
        [t.start() for t in th]
        results = []
        for v, f in news:
            nid = srv.register(v, f)
            d = np.empty(g.shape, np.float32)
            o = np.empty(g.shape, np.uint8)
            assert srv.poll(srv.submit(nid, g, d, o), 60000)[0]
            results.append((v, f, d, o))
        stop.set()
        [t.join() for t in th]
        assert not errors, errors
        assert outs
        for d, o in outs:
            assert_same_bake(d, o, d0, o0)
    for v, f, d, o in results:
        d1, o1 = ctx.bake(v, f, g, sdfb.make_opts())
        assert_same_bake(d, o, d1, o1)
