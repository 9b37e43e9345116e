"""Device weld and watertight census (sdfb_weld_device, sdfb_is_watertight_device) against the
host implementations, which the CPU suite pins to the reference's weldPositions / isWatertight."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_weld(ctx, soup, bmin, bmax):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(soup, np.float32).reshape(-1)).cuda()
    w = torch.empty(len(soup), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    u = ctx.weld_device(d.data_ptr(), len(soup), bmin, bmax, w.data_ptr())
    torch.cuda.synchronize()
    ok, b, m = ctx.is_watertight_device(w.data_ptr(), len(soup) // 3)
    return w.cpu().numpy().view(np.uint32), u, (ok, b, m)


def cases():
    from sdfb import meshgen as mg
    yield "uv-sphere", mg.uv_sphere_soup(0.4, 64, 32)
    v, f = mg.displaced_icosphere(5, 0.4, 2)
    soup = v[f.reshape(-1)]
    yield "icosphere", soup
    yield "icosphere-holes", v[mg.delete_faces(v, f, 0.02, 3)[1].reshape(-1)]
    rng = np.random.default_rng(5)
    jitter = soup + rng.normal(scale=1e-7, size=soup.shape).astype(np.float32)  # within the weld lattice
    yield "jittered", jitter.astype(np.float32)
    t, tf = mg.displaced_torus(90, 30, 0.3, 0.1, 4)
    yield "torus+sphere", np.concatenate([t[tf.reshape(-1)], soup]).astype(np.float32)
    dup = np.concatenate([soup, soup[:300]]).astype(np.float32)  # 100 triangles used twice: non-manifold
    yield "non-manifold", dup


@pytest.mark.parametrize("idx", range(6))
def test_device_weld_matches_host(ctx, idx):
    import sdfb
    pytest.importorskip("torch")
    name, soup = list(cases())[idx]
    soup = np.ascontiguousarray(soup, np.float32).reshape(-1, 3)
    bmin, bmax = soup.min(0), soup.max(0)
    hw, hu = sdfb.weld(soup, bmin, bmax)
    dw, du, (ok, b, m) = _device_weld(ctx, soup, bmin, bmax)
    assert du == hu and np.array_equal(dw, hw), name
    hok, hb, hm = sdfb.is_watertight(hw)
    assert (ok, b, m) == (hok, hb, hm), name


def test_soup_bake_with_device_weld(ctx, oracle):
    """The soup bake welds on the device: a closed soup takes parity, a holed one the winding
    number, and occupancy stays bit-exact."""
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(4, 0.4, 6)
    for faces, mode in ((f, sdfb.SIGN_PARITY), (mg.delete_faces(v, f, 0.03, 1)[1], sdfb.SIGN_GWN)):
        soup = np.ascontiguousarray(v[faces.reshape(-1)], np.float32)
        st = sdfb.Stats()
        st.struct_size = sdfb.C.sizeof(sdfb.Stats)
        g, dist, occ = ctx.bake_soup(soup, soup.min(0), soup.max(0), 48, stats=st)
        assert st.sign_mode_used == mode
        occ_ref = oracle.occupancy(soup, None, g.origin[:], g.voxel_size, (g.nx, g.ny, g.nz))
        assert np.array_equal(occ.reshape(-1), occ_ref)
