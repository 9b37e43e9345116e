"""The consumer check: a baked grid read the way the renderer reads it -- trilinear sampleSdf and
the sphere-traced __intersection__sdf (src/render/kernels/pathtracer.cu:587-613,684-702,740-787).
Where the traced rays meet the zero level set is compared with exact FP64 ray/mesh intersections.
The oracle's restatement runs here; the device kernels are compared with it bit for bit on a GPU."""
from __future__ import annotations

import numpy as np
import pytest

HIT_TOL_VOXELS = 0.1  # head-on rays: traced zero crossing vs exact first hit


def head_on_rays(k, seed):
    rng = np.random.default_rng(seed)
    dirs = rng.normal(size=(k, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    orig = -dirs * 0.49 + rng.normal(scale=0.02, size=(k, 3))
    tgt = rng.normal(scale=0.05, size=(k, 3))
    d = tgt - orig
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([orig, d], 1).astype(np.float32)


def signed_grid(oracle, v, f, org, vox, n):
    d = oracle.distance(v, f, org, vox, n)
    s = oracle.sign_parity(v, f, org, vox, n)
    return np.where(s < 0, -d, d).astype(np.float32)


def test_oracle_trace_meets_mesh(oracle):
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(4, 0.4, 3)
    n, org, vox = (64, 64, 64), (-0.5,) * 3, 1 / 64
    sd = signed_grid(oracle, v, f, org, vox, n)
    rays = head_on_rays(1500, 0)
    ts = oracle.trace_sdf(sd, org, vox, n, rays)
    tm = oracle.ray_mesh(v, f, rays)
    assert (ts >= 0).all() and (tm >= 0).all()
    assert np.abs(ts - tm).max() <= HIT_TOL_VOXELS * vox
    # rays that start inside report the far wall, rays that miss the grid report nothing
    miss = np.array([[2, 2, 2, 1, 0, 0], [0, 0, 0.9, 0, 0, 1]], np.float32)
    assert (oracle.trace_sdf(sd, org, vox, n, miss) == -1).all()


def test_oracle_sample_interpolates(oracle):
    n, org, vox = (8, 9, 10), (-0.5, -0.4, -0.3), 0.1
    rng = np.random.default_rng(1)
    grid = rng.normal(size=n[::-1]).astype(np.float32)
    # a linear field is reproduced exactly up to rounding by trilinear interpolation
    z, y, x = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    lin = (0.3 * x - 0.2 * y + 0.1 * z).astype(np.float32)
    p = rng.uniform(0.1, 0.6, (500, 3)).astype(np.float32) + np.float32([-0.5, -0.4, -0.3]) + 0.05
    got = oracle.sample_sdf(lin, org, vox, n, p)
    loc = (p - np.float32(org)) / np.float32(vox) - 0.5
    want = 0.3 * loc[:, 0] - 0.2 * loc[:, 1] + 0.1 * loc[:, 2]
    assert np.abs(got - want).max() < 1e-5
    assert np.isfinite(oracle.sample_sdf(grid, org, vox, n, p)).all()


@pytest.mark.gpu
def test_device_consumer_matches_oracle(ctx, oracle):
    """On a device bake of the displaced sphere: device sample and trace equal the oracle's bit for
    bit on the same grid, and the traced hits meet the exact mesh within 0.1 voxel."""
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(5, 0.4, 8)
    g = sdfb.make_grid((-0.5,) * 3, 1.0 / 128, (128, 128, 128))
    dist, _ = ctx.bake(v, f, g, sdfb.make_opts(sign_mode=sdfb.SIGN_PARITY))
    org, vox, n = (-0.5,) * 3, np.float32(1.0 / 128), (128, 128, 128)
    rng = np.random.default_rng(2)
    pts = rng.uniform(-0.6, 0.6, (20000, 3)).astype(np.float32)
    assert np.array_equal(ctx.sample_sdf(g, dist, pts).view(np.uint32),
                          oracle.sample_sdf(dist, org, vox, n, pts).view(np.uint32))
    rays = head_on_rays(4000, 3)
    td = ctx.trace_sdf(g, dist, rays)
    to = oracle.trace_sdf(dist, org, vox, n, rays)
    assert np.array_equal(td.view(np.uint32), to.view(np.uint32))
    tm = oracle.ray_mesh(v, f, rays)
    assert (td >= 0).all() and (tm >= 0).all()
    assert np.abs(td - tm).max() <= HIT_TOL_VOXELS * vox
