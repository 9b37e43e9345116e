"""Failure paths of the bake (needs an sm_103 device), made to happen without faulting the GPU.

The reference only throws (src/render/optix_check.h:13-52); this library returns statuses. Each
test makes a wait or a limit that the kernels already bound run out on purpose, through the
testing-only sdfb_opts fields (fault_inject, alloc_cap_kib), and checks the status the bake
returns and that the context still bakes correctly afterwards:

* the bounded wait of a warp for its block's next chunk of distance tiles (no warp moves the
  block on) -> SDFB_ERR_INTERNAL;
* the traversal step limit -> SDFB_ERR_INTERNAL;
* a shallow traversal stack that overflows -> the bake reruns with 64 entries and returns the same
  grid; a stack that overflows at every depth -> SDFB_ERR_OVERFLOW;
* a workspace allocation over a cap -> SDFB_ERR_OUT_OF_MEMORY;
* a serving poll whose timeout runs out before the request is done -> not done, status OK.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mesh():
    from sdfb import meshgen as mg
    return mg.displaced_icosphere(5, 0.35, 7)  # 20,480 triangles


def grid(n):
    import sdfb
    return sdfb.make_grid((-0.5,) * 3, 1.0 / n, (n, n, n))


def plain(ctx, mesh, g, **kw):
    import sdfb
    return ctx.bake(mesh[0], mesh[1], g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, **kw))


def expect_status(ctx, mesh, g, status, words, **kw):
    import sdfb
    with pytest.raises(sdfb.SdfbError) as e:
        plain(ctx, mesh, g, **kw)
    assert e.value.status == status, str(e.value)
    assert words in str(e.value), str(e.value)


def test_dispatch_wait_runs_out(ctx, mesh):
    import sdfb
    g = grid(128)
    ref = plain(ctx, mesh, g)
    expect_status(ctx, mesh, g, sdfb.ERR_INTERNAL, "dispatch timed out", fault_inject=sdfb.FAULT_DISPATCH,
                  step_budget=-1)
    d, o = plain(ctx, mesh, g)  # the context is still usable
    assert np.array_equal(d, ref[0]) and np.array_equal(o, ref[1])


def test_step_limit(ctx, mesh):
    import sdfb
    g = grid(64)
    ref = plain(ctx, mesh, g)
    expect_status(ctx, mesh, g, sdfb.ERR_INTERNAL, "step limit", fault_inject=sdfb.FAULT_STEP_LIMIT)
    d, _ = plain(ctx, mesh, g)
    assert np.array_equal(d, ref[0])


def test_shallow_stack_reruns_with_64_entries(ctx, mesh):
    import sdfb
    g = grid(96)
    ref = plain(ctx, mesh, g, stack_depth=64, leaf_size=4, tile=5)
    st = sdfb.Stats()
    st.struct_size = sdfb.C.sizeof(sdfb.Stats)
    d, o = ctx.bake(mesh[0], mesh[1], g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY, stack_depth=32, leaf_size=4,
                                                        tile=5, fault_inject=sdfb.FAULT_SHALLOW_STACK), stats=st)
    assert st.stack_used == 64
    assert np.array_equal(d, ref[0]) and np.array_equal(o, ref[1])


def test_stack_overflow_status(ctx, mesh):
    import sdfb
    g = grid(64)
    expect_status(ctx, mesh, g, sdfb.ERR_OVERFLOW, "stack overflow", fault_inject=sdfb.FAULT_STACK_ALL)
    plain(ctx, mesh, g)


def test_allocation_cap_is_out_of_memory(ctx, mesh):
    import sdfb
    g = grid(64)
    ref = plain(ctx, mesh, g)
    expect_status(ctx, mesh, g, sdfb.ERR_OUT_OF_MEMORY, "cannot allocate", alloc_cap_kib=1)
    d, _ = plain(ctx, mesh, g)
    assert np.array_equal(d, ref[0])


def test_poll_timeout_returns_not_done(ctx, mesh):
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_torus(512, 256, 0.3, 0.12, 5)  # 262,144 triangles
    g = grid(256)
    srv = sdfb.Server(ctx)
    try:
        mid = srv.register(v, f)
        d = np.empty(g.cells, np.float32)
        rid = srv.submit(mid, g, d, None)
        done, _ = srv.poll(rid, 1)  # a 256^3 bake of this mesh takes far longer than 1 ms
        assert not done
        done, info = srv.poll(rid, 120000)
        assert done and info["status"] == sdfb.OK
        ref, _ = ctx.bake(v, f, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY), want_occ=False)
        assert np.abs(d.reshape(g.shape) - ref).max() <= 1e-5 * np.sqrt(3.0)
    finally:
        srv.close()
