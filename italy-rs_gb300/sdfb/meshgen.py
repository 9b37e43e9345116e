"""Seeded synthetic meshes for the bake workloads (no datasets are involved).

Every generator returns ``(verts, idx)``: ``float32[V, 3]`` vertex positions and
``uint32[T, 3]`` triangle indices, or, for the reference's soup layout, ``float32[3T, 3]``.

* ``uv_sphere_soup`` follows the UV sphere of the reference's sign test
  (tests/sdf_sign_test.cpp:18-42): quads split ``a,b,c, a,c,d`` in FP32, so the pole rows
  contain degenerate triangles and the seam repeats positions. ``weld`` turns it into an
  indexed mesh the way ``weldPositions`` (src/io/mesh_weld.cpp:26-48) does.
* ``icosphere`` subdivides an icosahedron ``level`` times (20 * 4**level triangles) and
  projects to a sphere; ``displace`` pushes vertices radially by a sum of seeded sinusoids.
* ``torus`` is a watertight (nu x nv) quad torus; ``soup_with_holes`` concatenates meshes and
  deletes a seeded fraction of faces; ``batch_meshes`` draws the 64-mesh batch workload.
"""
from __future__ import annotations

import math

import numpy as np

# --------------------------------------------------------------------------------------------
# The reference's UV sphere, in FP32 like the C++ test.


def uv_sphere_soup(r: float, lon_segs: int, lat_segs: int) -> np.ndarray:
    """float32[6 * lon * lat, 3] soup, vertex order a,b,c, a,c,d per quad (sdf_sign_test.cpp:25-36)."""
    f = np.float32
    lat = np.arange(lat_segs + 1, dtype=np.int64)
    lon = np.arange(lon_segs + 1, dtype=np.int64)
    theta = (lat.astype(f) / f(lat_segs)) * f(math.pi)
    phi = ((lon.astype(f) / f(lon_segs)) * f(2.0)) * f(math.pi)
    st = np.sin(theta.astype(np.float64)).astype(f)
    ct = np.cos(theta.astype(np.float64)).astype(f)
    sp = np.sin(phi.astype(np.float64)).astype(f)
    cp = np.cos(phi.astype(np.float64)).astype(f)
    rr = f(r)
    # vertex(lat, lon) = (r sin(theta) cos(phi), r cos(theta), r sin(theta) sin(phi)), FP32 left to right
    vx = (rr * st)[:, None] * cp[None, :]
    vy = np.broadcast_to((rr * ct)[:, None], vx.shape)
    vz = (rr * st)[:, None] * sp[None, :]
    V = np.stack([vx, vy, vz], axis=-1).astype(f)  # [lat+1, lon+1, 3]
    la, lo = np.meshgrid(np.arange(lat_segs), np.arange(lon_segs), indexing="ij")
    a = V[la, lo]
    b = V[la + 1, lo]
    c = V[la + 1, lo + 1]
    d = V[la, lo + 1]
    quads = np.stack([a, b, c, a, c, d], axis=2)  # [lat, lon, 6, 3]
    return np.ascontiguousarray(quads.reshape(-1, 3))


def weld(positions: np.ndarray, bmin, bmax) -> tuple[np.ndarray, np.ndarray]:
    """Indexed mesh from a soup: lattice max(|extent| * 1e-5, 1e-6) in FP32, keys lround(p / cell),
    first occurrence kept (src/io/mesh_weld.cpp:26-48). Returns (unique float32[U, 3], uint32[T, 3])."""
    f = np.float32
    pos = np.ascontiguousarray(positions, dtype=f)
    ext = (np.asarray(bmax, f) - np.asarray(bmin, f)).astype(f)
    diag = np.sqrt(f(f(ext[0] * ext[0]) + f(ext[1] * ext[1])) + f(ext[2] * ext[2]))
    cell = max(f(diag * f(1e-5)), f(1e-6))
    q = pos / f(cell)
    keys = np.where(q >= 0, np.floor(q.astype(np.float64) + 0.5), np.ceil(q.astype(np.float64) - 0.5)).astype(np.int64)
    _, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    inverse = inverse.reshape(-1)
    # renumber in first-occurrence order
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    welded = rank[inverse].astype(np.uint32)
    uniq = pos[np.sort(first)]
    return np.ascontiguousarray(uniq), np.ascontiguousarray(welded.reshape(-1, 3))


# --------------------------------------------------------------------------------------------
# Icospheres, tori, displacement.


def icosahedron() -> tuple[np.ndarray, np.ndarray]:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere in FP64: (verts[V, 3], faces[T, 3]) with outward (counter-clockwise) winding."""
    v, f = icosahedron()
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e_sorted = np.sort(e, axis=1)
        uniq, inv = np.unique(e_sorted, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid], axis=0)
        nT = len(f)
        m01 = base + inv[0:nT]
        m12 = base + inv[nT:2 * nT]
        m20 = base + inv[2 * nT:3 * nT]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f


def torus(R: float, r: float, nu: int, nv: int) -> tuple[np.ndarray, np.ndarray]:
    """Watertight torus around the y axis in FP64, 2 * nu * nv triangles, outward winding."""
    u = np.arange(nu) * (2.0 * math.pi / nu)
    w = np.arange(nv) * (2.0 * math.pi / nv)
    U, W = np.meshgrid(u, w, indexing="ij")
    x = (R + r * np.cos(W)) * np.cos(U)
    z = (R + r * np.cos(W)) * np.sin(U)
    y = r * np.sin(W)
    verts = np.stack([x, y, z], axis=-1).reshape(-1, 3)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    faces = np.concatenate([np.stack([a, d, c], -1).reshape(-1, 3), np.stack([a, c, b], -1).reshape(-1, 3)], 0)
    return verts, faces


def displace(verts: np.ndarray, center: np.ndarray, rng: np.random.Generator, amplitude: float = 0.05,
             terms: int = 8) -> np.ndarray:
    """Push each vertex radially about `center`: p' = c + (p - c) * (1 + sum_k a_k sin(f_k (d . u_k) + phi_k)),
    with d the unit direction, u_k seeded unit vectors, f_k ~ U[2, 12], phi_k ~ U[0, 2 pi) and
    a_k >= 0 summing to `amplitude`."""
    u = rng.normal(size=(terms, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    freq = rng.uniform(2.0, 12.0, size=terms)
    phase = rng.uniform(0.0, 2.0 * math.pi, size=terms)
    a = rng.uniform(0.0, 1.0, size=terms)
    a = a / a.sum() * amplitude
    rel = verts - center
    nrm = np.linalg.norm(rel, axis=1, keepdims=True)
    d = rel / np.maximum(nrm, 1e-300)
    s = np.sin(d @ (u.T * freq) + phase) @ a
    return center + rel * (1.0 + s)[:, None]


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _f32(v: np.ndarray, f: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    return np.ascontiguousarray(v, dtype=np.float32), np.ascontiguousarray(f, dtype=np.uint32)


def displaced_icosphere(level: int, radius: float, seed: int, center=(0.0, 0.0, 0.0),
                        amplitude: float = 0.05) -> tuple[np.ndarray, np.ndarray]:
    """Icosphere of `level`, radius `radius`, displaced radially by 8 seeded sinusoids whose
    amplitudes sum to `amplitude` (relative to the radius)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    c = np.asarray(center, dtype=np.float64)
    v = c + v * radius
    v = displace(v, c, rng, amplitude)
    return _f32(v, f)


def displaced_torus(nu: int, nv: int, R: float, r: float, seed: int, center=(0.0, 0.0, 0.0),
                    amplitude: float = 0.05) -> tuple[np.ndarray, np.ndarray]:
    """Seeded-rotation torus displaced along its tube normal by 8 seeded sinusoids."""
    rng = np.random.default_rng(seed)
    v, f = torus(R, r, nu, nv)
    # displace along the tube: about the nearest point of the core circle
    ring = v.copy()
    ring[:, 1] = 0.0
    ring *= (R / np.maximum(np.linalg.norm(ring, axis=1, keepdims=True), 1e-300))
    rel = v - ring
    u = rng.normal(size=(8, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    freq = rng.uniform(2.0, 12.0, size=8)
    phase = rng.uniform(0.0, 2.0 * math.pi, size=8)
    a = rng.uniform(0.0, 1.0, size=8)
    a = a / a.sum() * amplitude
    d = v / np.maximum(np.linalg.norm(v, axis=1, keepdims=True), 1e-300)
    s = np.sin(d @ (u.T * freq) + phase) @ a
    v = ring + rel * (1.0 + s)[:, None]
    v = v @ random_rotation(rng).T + np.asarray(center, dtype=np.float64)
    return _f32(v, f)


def concat(meshes: list[tuple[np.ndarray, np.ndarray]]) -> tuple[np.ndarray, np.ndarray]:
    vs, fs, off = [], [], 0
    for v, f in meshes:
        vs.append(v)
        fs.append(f.astype(np.int64) + off)
        off += len(v)
    return _f32(np.concatenate(vs, 0), np.concatenate(fs, 0))


def delete_faces(verts: np.ndarray, faces: np.ndarray, fraction: float, seed: int) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    n = len(faces)
    k = int(round(fraction * n))
    drop = rng.choice(n, size=k, replace=False)
    keep = np.ones(n, dtype=bool)
    keep[drop] = False
    return verts, np.ascontiguousarray(faces[keep])


# --------------------------------------------------------------------------------------------
# The workloads.

UNIT_BOUNDS = ((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))


def unit_grid(n: int) -> tuple[tuple[float, float, float], float, tuple[int, int, int]]:
    """Grid over [-0.5, 0.5]^3 with n^3 cells: (origin, voxel, (n, n, n))."""
    return (-0.5, -0.5, -0.5), 1.0 / n, (n, n, n)


def uv_sphere_mesh(r: float = 0.4, lon: int = 64, lat: int = 32) -> tuple[np.ndarray, np.ndarray]:
    """The plain-bake sphere: the reference's UV sphere (lon 64 x lat 32, 4096 triangles, 128 of them
    degenerate at the poles), welded to an indexed mesh."""
    soup = uv_sphere_soup(r, lon, lat)
    return weld(soup, (-r, -r, -r), (r, r, r))


def displaced_sphere_mesh(seed: int = 1234) -> tuple[np.ndarray, np.ndarray]:
    """Level-6 icosphere (81,920 triangles), radius 0.35, 8 seeded sinusoids of total amplitude 0.05."""
    return displaced_icosphere(6, 0.35, seed)


def soup_with_holes(seed: int = 4321, spheres: int = 5, sphere_level: int = 6, torus_nu: int = 224,
                    torus_nv: int = 75, fraction: float = 0.02) -> tuple[np.ndarray, np.ndarray]:
    """Non-watertight soup: `spheres` displaced icospheres and 3 displaced tori at seeded placements in
    [-0.5, 0.5]^3, then `fraction` of the faces deleted uniformly at random. Defaults give
    5 * 81,920 + 3 * 33,600 = 510,400 triangles before and 500,192 after deletion."""
    rng = np.random.default_rng(seed)
    parts = []
    for i in range(spheres):
        r = rng.uniform(0.12, 0.22)
        c = rng.uniform(-0.5 + r * 1.1, 0.5 - r * 1.1, size=3)
        parts.append(displaced_icosphere(sphere_level, r, int(rng.integers(1 << 30)), center=c))
    for i in range(3):
        R = rng.uniform(0.15, 0.25)
        r = rng.uniform(0.04, 0.07)
        ext = R + r
        c = rng.uniform(-0.5 + ext * 1.1, 0.5 - ext * 1.1, size=3)
        parts.append(displaced_torus(torus_nu, torus_nv, R, r, int(rng.integers(1 << 30)), center=c))
    v, f = concat(parts)
    return delete_faces(v, f, fraction, int(rng.integers(1 << 30)))


def mesh_for_count(target: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """A displaced icosphere or torus (seeded coin) with about `target` triangles in [-0.5, 0.5]^3.
    Icospheres take the level whose count 20 * 4**L is nearest in log scale, kept within levels 3..7
    (1,280 .. 327,680 triangles); tori take nu x nv (aspect 3:1) with 2 nu nv ~= target."""
    rng = np.random.default_rng(seed)
    if rng.uniform() < 0.5:
        level = int(round(math.log(max(target, 20) / 20.0, 4)))
        level = max(3, min(level, 7))  # 1,280 .. 327,680 triangles: inside [1e3, 1e6]
        return displaced_icosphere(level, 0.35, int(rng.integers(1 << 30)))
    nv = max(3, int(round(math.sqrt(target / 6.0))))
    nu = max(3, int(round(target / (2.0 * nv))))
    return displaced_torus(nu, nv, 0.28, 0.1, int(rng.integers(1 << 30)))


def batch_meshes(count: int = 64, seed: int = 2024, tri_lo: float = 1e3, tri_hi: float = 1e6,
                 resolutions=(32, 64, 128, 256)):
    """The batched workload: `count` meshes with log-uniform triangle counts in [tri_lo, tri_hi] and
    grids drawn uniformly from `resolutions` (cubed, over [-0.5, 0.5]^3). Mesh i uses seed + i.
    Returns a list of (verts, idx, n)."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        target = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        n = int(resolutions[int(rng.integers(len(resolutions)))])
        v, f = mesh_for_count(target, seed + i + 7919)
        out.append((v, f, n))
    return out


def random_materials(ntris: int, seed: int, num_materials: int = 4, tex_sizes=((16, 8), (5, 7)),
                     short_tri_mat: bool = True) -> dict:
    """A seeded material set for a soup of `ntris` triangles, in the layout of MeshAsset's
    materials (src/io/mesh_asset.h:33-54): per material a base colour factor, metallic, roughness
    and a base colour texture (-1 = none); per triangle a material index (some past the end, which
    the bake maps to material 0, and the list one short so the last triangle uses the default);
    one uv pair per soup vertex, spread over [-2, 3) so texture wrapping is exercised; RGBA8
    textures, the first sRGB-encoded and the second linear."""
    rng = np.random.default_rng(seed)
    mat_f = np.empty((num_materials, 5), np.float32)
    mat_f[:, :3] = rng.uniform(0.0, 1.2, (num_materials, 3))
    mat_f[:, 3] = rng.uniform(0.0, 1.0, num_materials)
    mat_f[:, 4] = rng.uniform(0.0, 1.0, num_materials)
    mat_tex = np.array([(i % (len(tex_sizes) + 1)) - 1 for i in range(num_materials)], np.int32)
    if num_materials > 1:
        mat_tex[1] = len(tex_sizes) + 3  # an index past the texture list: no texture
    tri_mat = rng.integers(0, num_materials + 2, ntris).astype(np.uint32)
    if short_tri_mat and ntris > 0:
        tri_mat = tri_mat[:-1]
    uvs = rng.uniform(-2.0, 3.0, (3 * ntris, 2)).astype(np.float32)
    textures = [(rng.integers(0, 256, (h, w, 4)).astype(np.uint8), k == 0) for k, (w, h) in enumerate(tex_sizes)]
    return {"mat_f": mat_f, "mat_tex": mat_tex, "tri_mat": tri_mat, "uvs": uvs, "textures": textures}
