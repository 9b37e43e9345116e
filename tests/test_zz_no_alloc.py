"""The allocation-free occupancy entry point (sdfb_occupancy_noalloc), for callers that may not
allocate device memory (plugins whose host owns all device memory, processes under a fixed memory
quota, latency-bound loops). Called through the C ABI twice in a row on different meshes and grids,
its occupancy must equal the context-based bake's, bit for bit (occupancy is exact)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).cuda()


def test_noalloc_occupancy_matches_bake_twice(ctx):
    torch = pytest.importorskip("torch")
    import sdfb
    from sdfb import meshgen as mg
    lib = sdfb.load()
    cases = [(mg.displaced_icosphere(4, 0.33, 11), 48), (mg.displaced_torus(60, 20, 0.27, 0.1, 12), 37)]
    grids, outs, keep = [], [], []
    for (v, f), n in cases:  # two calls in a row on torch's (legacy default) stream, no sync between them
        g = sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n + 3, n - 2))
        dv, di = _dev(torch, v, np.float32), _dev(torch, f.astype(np.int32), np.int32)
        docc = torch.full((g.cells,), 7, dtype=torch.uint8, device="cuda")  # stale contents must be cleared
        st = lib.sdfb_occupancy_noalloc(C.c_void_p(dv.data_ptr()), len(v), C.c_void_p(di.data_ptr()), len(f),
                                        C.byref(g), C.c_void_p(docc.data_ptr()), None)
        assert st == sdfb.OK
        grids.append(g)
        outs.append(docc)
        keep += [dv, di]
    torch.cuda.synchronize()
    for ((v, f), _), g, docc in zip(cases, grids, outs):
        _, ref = ctx.bake(v, f, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE), want_dist=False)
        assert ref.any()
        assert np.array_equal(docc.cpu().numpy().reshape(g.shape), ref)


def test_noalloc_at_the_triangle_limit_on_a_caller_stream(ctx):
    """A mesh of exactly 1,048,576 triangles (the documented maximum) on a non-blocking stream the
    caller created: the array must hold its counts and their scan, and the result must equal the
    context bake's, bit for bit."""
    torch = pytest.importorskip("torch")
    import sdfb
    from sdfb import meshgen as mg
    lib = sdfb.load()
    v, f = mg.displaced_torus(1024, 512, 0.3, 0.12, 21)
    assert len(f) == 1 << 20
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 96, (96, 96, 96))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dv, di = _dev(torch, v, np.float32), _dev(torch, f.astype(np.int32), np.int32)
        docc = torch.full((g.cells,), 3, dtype=torch.uint8, device="cuda")
    st = lib.sdfb_occupancy_noalloc(C.c_void_p(dv.data_ptr()), len(v), C.c_void_p(di.data_ptr()), len(f),
                                    C.byref(g), C.c_void_p(docc.data_ptr()), C.c_void_p(s.cuda_stream))
    assert st == sdfb.OK
    s.synchronize()
    _, ref = ctx.bake(v, f, g, sdfb.make_opts(sign_mode=sdfb.SIGN_NONE), want_dist=False)
    assert ref.any()
    assert np.array_equal(docc.cpu().numpy().reshape(g.shape), ref)


def test_noalloc_rejects_oversized_mesh(ctx):
    import sdfb
    lib = sdfb.load()
    g = sdfb.make_grid((0, 0, 0), 0.1, (4, 4, 4))
    st = lib.sdfb_occupancy_noalloc(C.c_void_p(16), 3, C.c_void_p(16), (1 << 20) + 1, C.byref(g), C.c_void_p(16),
                                    None)
    assert st == sdfb.ERR_INVALID_ARGUMENT
