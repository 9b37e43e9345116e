"""ctypes binding of libsdfb.so, the GB300 mesh -> SDF bake (C ABI in include/sdfb.h).

This is the Python face of the same entry points a C, C++ or FFI caller binds; tests and the
benchmark go through it. Loading fails loudly when the library has not been built: there is no
CPU fallback. Build it with ``python italy-rs_gb300/build.py`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libsdfb.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_OUT_OF_MEMORY = 2
ERR_CUDA = 3
ERR_BAD_MESH = 4
ERR_OVERFLOW = 5
ERR_BUSY = 6
ERR_TIMEOUT = 7
ERR_NOT_FOUND = 8
ERR_NO_DEVICE = 9
ERR_INTERNAL = 10

# sdfb_opts.fault_inject bits (testing only; see include/sdfb.h)
FAULT_DISPATCH = 1
FAULT_STEP_LIMIT = 2
FAULT_SHALLOW_STACK = 4
FAULT_STACK_ALL = 8

SIGN_AUTO, SIGN_PARITY, SIGN_GWN, SIGN_NONE = 0, 1, 2, 3


class SdfbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"sdfb status {status}: {message}")
        self.status = status


class GridDesc(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("voxel_size", C.c_float), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nz", C.c_int32)]

    @property
    def shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def cells(self) -> int:
        return int(self.nx) * int(self.ny) * int(self.nz)


class Opts(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("sign_mode", C.c_int32), ("band_voxels", C.c_float),
                ("leaf_size", C.c_int32), ("tile", C.c_int32), ("no_occupancy", C.c_int32),
                ("no_distance", C.c_int32), ("count_work", C.c_int32), ("stack_depth", C.c_int32),
                ("step_budget", C.c_int32), ("fault_inject", C.c_int32), ("alloc_cap_kib", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class Stats(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("sign_mode_used", C.c_int32), ("watertight", C.c_int32),
                ("leaf_size_used", C.c_int32), ("tile_used", C.c_int32), ("stack_used", C.c_int32),
                ("ms_total", C.c_double), ("ms_prepare", C.c_double), ("ms_build", C.c_double),
                ("ms_occupancy", C.c_double), ("ms_sign", C.c_double), ("ms_distance", C.c_double),
                ("voxels", C.c_uint64), ("triangles", C.c_uint64), ("sat_tests", C.c_uint64),
                ("crossings", C.c_uint64), ("box_tests", C.c_uint64), ("tri_tests", C.c_uint64),
                ("flops_distance", C.c_double), ("kernel_launches", C.c_uint64), ("gwn_fp64_cells", C.c_uint64),
                ("graph_replayed", C.c_uint64), ("tiles_deferred", C.c_uint64),
                ("plane_tests", C.c_uint64), ("rect_tests", C.c_uint64), ("gwn_direct_cells", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k not in ("reserved", "struct_size")}


class MeshDesc(C.Structure):
    _fields_ = [("verts", C.c_void_p), ("idx", C.c_void_p), ("num_verts", C.c_uint32), ("num_tris", C.c_uint32)]


class ServerOpts(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("hbm_budget_bytes", C.c_uint64), ("max_inflight", C.c_int32),
                ("wave_voxels_log2", C.c_int32), ("reserved", C.c_int32 * 8)]


class RequestInfo(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("status", C.c_int32), ("t_submit_ms", C.c_double),
                ("t_admit_ms", C.c_double), ("t_done_ms", C.c_double), ("voxels", C.c_uint64),
                ("mesh_was_resident", C.c_int32), ("pad", C.c_int32)]


class Texture(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("srgb", C.c_int32),
                ("reserved", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("base_color", C.c_float * 3), ("metallic", C.c_float), ("roughness", C.c_float),
                ("base_color_texture", C.c_int32)]


class Materials(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("num_materials", C.c_uint32), ("materials", C.c_void_p),
                ("triangle_material", C.c_void_p), ("num_triangle_material", C.c_uint64), ("uvs", C.c_void_p),
                ("num_uvs", C.c_uint64), ("textures", C.c_void_p), ("num_textures", C.c_uint32),
                ("reserved", C.c_uint32)]


def make_materials(m: dict):
    """(Materials, keep-alive list) from {"mat_f": (M, 5) base colour rgb, metallic, roughness;
    "mat_tex": (M,) texture index or -1; "tri_mat": per-triangle indices; "uvs": (3T, 2);
    "textures": [(rgba uint8 (h, w, 4), srgb), ...]} (the layout meshgen.random_materials makes)."""
    mf = np.ascontiguousarray(m["mat_f"], np.float32).reshape(-1, 5)
    mt = np.ascontiguousarray(m["mat_tex"], np.int32).reshape(-1)
    mats = (Material * len(mt))()
    for i in range(len(mt)):
        mats[i].base_color[:] = [float(x) for x in mf[i, :3]]
        mats[i].metallic, mats[i].roughness, mats[i].base_color_texture = float(mf[i, 3]), float(mf[i, 4]), int(mt[i])
    tri = np.ascontiguousarray(m.get("tri_mat", np.zeros(0)), np.uint32).reshape(-1)
    uvs = np.ascontiguousarray(m.get("uvs", np.zeros((0, 2))), np.float32).reshape(-1, 2)
    texs = [(np.ascontiguousarray(t[0], np.uint8), bool(t[1])) for t in m.get("textures", [])]
    tarr = (Texture * max(len(texs), 1))()
    for k, (px, srgb) in enumerate(texs):
        tarr[k].rgba = px.ctypes.data
        tarr[k].width, tarr[k].height, tarr[k].srgb = px.shape[1], px.shape[0], int(srgb)
    out = Materials()
    out.struct_size = C.sizeof(Materials)
    out.num_materials = len(mt)
    out.materials = C.cast(mats, C.c_void_p)
    out.triangle_material = tri.ctypes.data if len(tri) else None
    out.num_triangle_material = len(tri)
    out.uvs = uvs.ctypes.data if len(uvs) else None
    out.num_uvs = len(uvs)
    out.textures = C.cast(tarr, C.c_void_p) if texs else None
    out.num_textures = len(texs)
    return out, [mats, tri, uvs, texs, tarr]


_P = C.c_void_p
_u32, _i32, _u64 = C.c_uint32, C.c_int32, C.c_uint64

# name -> (restype, argtypes)
SIGNATURES = {
    "sdfb_abi_version": (_i32, []),
    "sdfb_ctx_create": (_i32, [_i32, C.POINTER(_P)]),
    "sdfb_ctx_destroy": (None, [_P]),
    "sdfb_last_error": (C.c_char_p, [_P]),
    "sdfb_ctx_trim": (_i32, [_P]),
    "sdfb_ctx_device_bytes": (_u64, [_P]),
    "sdfb_grid_from_bounds_res": (_i32, [_P, _P, _i32, C.POINTER(GridDesc)]),
    "sdfb_bake": (_i32, [_P, _P, _u32, _P, _u32, C.POINTER(GridDesc), C.POINTER(Opts), _P, _P, C.POINTER(Stats)]),
    "sdfb_bake_device": (_i32, [_P, _P, _u32, _P, _u32, C.POINTER(GridDesc), C.POINTER(Opts), _P, _P, _P,
                                C.POINTER(Stats)]),
    "sdfb_bake_soup": (_i32, [_P, _P, _u32, _P, _P, _i32, C.POINTER(Opts), C.POINTER(GridDesc), _P, _P,
                              C.POINTER(Stats)]),
    "sdfb_voxelize_sparse": (_i32, [_P, _P, _u32, _P, _P, _i32, _P, _u64, C.POINTER(_u64), _P, C.POINTER(C.c_float)]),
    "sdfb_weld": (_i32, [_P, _P, _u32, _P, _P, _P, C.POINTER(_u32)]),
    "sdfb_is_watertight": (_i32, [_P, _P, _u32, C.POINTER(_i32), C.POINTER(_u64), C.POINTER(_u64)]),
    "sdfb_bake_batch": (_i32, [_P, _u32, C.POINTER(MeshDesc), C.POINTER(GridDesc), C.POINTER(Opts), _P, _P,
                               C.POINTER(Stats)]),
    "sdfb_bake_batch_device": (_i32, [_P, _u32, C.POINTER(MeshDesc), C.POINTER(GridDesc), C.POINTER(Opts), _P, _P,
                                      _P, C.POINTER(Stats)]),
    "sdfb_server_create": (_i32, [_P, C.POINTER(ServerOpts), C.POINTER(_P)]),
    "sdfb_server_destroy": (None, [_P]),
    "sdfb_mesh_register": (_i32, [_P, _P, _u32, _P, _u32, C.POINTER(_u64)]),
    "sdfb_submit": (_i32, [_P, _u64, C.POINTER(GridDesc), C.POINTER(Opts), _P, _P, C.POINTER(_u64)]),
    "sdfb_poll": (_i32, [_P, _u64, _i32, C.POINTER(_i32), C.POINTER(RequestInfo)]),
    "sdfb_server_last_error": (C.c_char_p, [_P]),
    "sdfb_bake_materials": (_i32, [_P, _P, _u32, C.POINTER(GridDesc), C.POINTER(Materials), _P, _P, _P]),
    "sdfb_voxelize_sparse_colors": (_i32, [_P, _P, _u32, _P, _P, _i32, C.POINTER(Materials), _P, _P, _u64,
                                           C.POINTER(_u64), _P, C.POINTER(C.c_float)]),
    "sdfb_weld_device": (_i32, [_P, _P, _u32, _P, _P, _P, C.POINTER(_u32), _P]),
    "sdfb_is_watertight_device": (_i32, [_P, _P, _u32, C.POINTER(_i32), C.POINTER(_u64), C.POINTER(_u64), _P]),
    "sdfb_sample_sdf": (_i32, [_P, C.POINTER(GridDesc), _P, _P, _u64, _P]),
    "sdfb_trace_sdf": (_i32, [_P, C.POINTER(GridDesc), _P, _P, _u64, C.c_float, C.c_float, _P]),
    "sdfb_occupancy_noalloc": (_i32, [_P, _u32, _P, _u32, C.POINTER(GridDesc), _P, _P]),
}

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Loads libsdfb.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is not built; run italy-rs_gb300/build.py")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32a(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def make_grid(origin, voxel, n) -> GridDesc:
    g = GridDesc()
    for i in range(3):
        g.origin[i] = float(origin[i])
    g.voxel_size = float(np.float32(voxel))
    g.nx, g.ny, g.nz = (int(x) for x in n)
    return g


def make_opts(sign_mode: int = SIGN_AUTO, band_voxels: float = 1.0, leaf_size: int = 0, tile: int = 0,
              no_occupancy: bool = False, no_distance: bool = False, count_work: bool = False,
              stack_depth: int = 0, step_budget: int = 0, fault_inject: int = 0, alloc_cap_kib: int = 0) -> Opts:
    """tile: shape 1..6 (0 = tuned); leaf_size 1..16 (0 = tuned); stack_depth 32 or 64 (0 = tuned);
    step_budget: traversal steps before a distance tile is deferred (0 = tuned, -1 = never);
    fault_inject / alloc_cap_kib: testing only (FAULT_* bits; a workspace allocation cap)."""
    o = Opts()
    o.struct_size = C.sizeof(Opts)
    o.sign_mode = sign_mode
    o.band_voxels = band_voxels
    o.leaf_size = leaf_size
    o.tile = tile
    o.no_occupancy = int(no_occupancy)
    o.no_distance = int(no_distance)
    o.count_work = int(count_work)
    o.stack_depth = stack_depth
    o.step_budget = step_budget
    o.fault_inject = fault_inject
    o.alloc_cap_kib = alloc_cap_kib
    return o


def grid_from_bounds_res(bmin, bmax, resolution: int) -> GridDesc:
    g = GridDesc()
    st = load().sdfb_grid_from_bounds_res(_ptr(_f32(bmin)), _ptr(_f32(bmax)), int(resolution), C.byref(g))
    if st != OK:
        raise SdfbError(st, "grid too large")
    return g


def weld(positions, bmin, bmax):
    p = _f32(positions).reshape(-1, 3)
    out = np.empty(len(p), np.uint32)
    n = C.c_uint32()
    st = load().sdfb_weld(None, _ptr(p), len(p), _ptr(_f32(bmin)), _ptr(_f32(bmax)), _ptr(out), C.byref(n))
    if st != OK:
        raise SdfbError(st, "weld failed")
    return out, int(n.value)


def is_watertight(welded_idx):
    w = _u32a(welded_idx).reshape(-1)
    ok, b, m = C.c_int32(), C.c_uint64(), C.c_uint64()
    st = load().sdfb_is_watertight(None, _ptr(w), len(w) // 3, C.byref(ok), C.byref(b), C.byref(m))
    if st != OK:
        raise SdfbError(st, "watertight test failed")
    return bool(ok.value), int(b.value), int(m.value)


class Context:
    """One device context (streams, device memory, resident meshes)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.sdfb_ctx_create(int(device), C.byref(h))
        if st != OK:
            raise SdfbError(st, "cannot create a context (no sm_103 device?)")
        self.h = h

    def close(self):
        if self.h:
            self.lib.sdfb_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self) -> str:
        return (self.lib.sdfb_last_error(self.h) or b"").decode()

    def _check(self, st: int):
        if st != OK:
            raise SdfbError(st, self.error())

    def bake(self, verts, idx, grid: GridDesc, opts: Opts | None = None, want_dist=True, want_occ=True,
             stats: Stats | None = None, out=None):
        """Host-buffer bake. Returns (dist float32[nz, ny, nx] or None, occ uint8[nz, ny, nx] or None);
        `out` may pass preallocated (dist, occ) arrays (a pinned distance array is written in place
        by the bake's kernels)."""
        v = _f32(verts).reshape(-1, 3)
        i = _u32a(idx).reshape(-1, 3)
        if out is not None:
            dist, occ = out
        else:
            dist = np.empty(grid.shape, np.float32) if want_dist else None
            occ = np.empty(grid.shape, np.uint8) if want_occ else None
        st = self.lib.sdfb_bake(self.h, _ptr(v), len(v), _ptr(i), len(i), C.byref(grid),
                                C.byref(opts) if opts is not None else None, _ptr(dist), _ptr(occ),
                                C.byref(stats) if stats is not None else None)
        self._check(st)
        return dist, occ

    def bake_status(self, verts, idx, grid: GridDesc, opts: Opts | None = None) -> tuple[int, str]:
        """Runs a bake and returns (status, message) instead of raising (for error-path tests)."""
        v = _f32(verts).reshape(-1, 3)
        i = _u32a(idx).reshape(-1, 3)
        dist = np.empty(grid.shape, np.float32)
        occ = np.empty(grid.shape, np.uint8)
        st = self.lib.sdfb_bake(self.h, _ptr(v), len(v), _ptr(i), len(i), C.byref(grid),
                                C.byref(opts) if opts is not None else None, _ptr(dist), _ptr(occ), None)
        return st, self.error()

    def bake_device(self, d_verts: int, num_verts: int, d_idx: int, num_tris: int, grid: GridDesc,
                    opts: Opts | None, d_dist: int, d_occ: int, stream: int = 0, stats: Stats | None = None):
        st = self.lib.sdfb_bake_device(self.h, C.c_void_p(d_verts), num_verts, C.c_void_p(d_idx), num_tris,
                                       C.byref(grid), C.byref(opts) if opts is not None else None,
                                       C.c_void_p(d_dist), C.c_void_p(d_occ), C.c_void_p(stream),
                                       C.byref(stats) if stats is not None else None)
        self._check(st)

    def bake_soup(self, positions, bmin, bmax, resolution: int, opts: Opts | None = None, stats: Stats | None = None,
                  alloc=None):
        """The reference's bakeSdf(MeshAsset, resolution): returns (grid, dist, occ). `alloc(shape,
        dtype)` may supply the output arrays (pinned ones are written in place)."""
        p = _f32(positions).reshape(-1, 3)
        g = GridDesc()
        st = self.lib.sdfb_bake_soup(self.h, _ptr(p), len(p) // 3, _ptr(_f32(bmin)), _ptr(_f32(bmax)),
                                     int(resolution), C.byref(opts) if opts is not None else None, C.byref(g), None,
                                     None, None)
        self._check(st)
        alloc = alloc or (lambda shape, dtype: np.empty(shape, dtype))
        dist = alloc(g.shape, np.float32)
        occ = alloc(g.shape, np.uint8)
        st = self.lib.sdfb_bake_soup(self.h, _ptr(p), len(p) // 3, _ptr(_f32(bmin)), _ptr(_f32(bmax)),
                                     int(resolution), C.byref(opts) if opts is not None else None, C.byref(g),
                                     _ptr(dist), _ptr(occ), C.byref(stats) if stats is not None else None)
        self._check(st)
        return g, dist, occ

    def bake_materials(self, positions, grid: GridDesc, materials: dict):
        """bakePerCellMaterial on the device: (base colour float32[nz, ny, nx, 3], metallic, roughness)."""
        p = _f32(positions).reshape(-1, 9)
        m, keep = make_materials(materials)
        col = np.empty(grid.shape + (3,), np.float32)
        met = np.empty(grid.shape, np.float32)
        rou = np.empty(grid.shape, np.float32)
        self._check(self.lib.sdfb_bake_materials(self.h, _ptr(p), len(p), C.byref(grid), C.byref(m), _ptr(col),
                                                 _ptr(met), _ptr(rou)))
        del keep
        return col, met, rou

    def voxelize_sparse_colors(self, positions, bmin, bmax, resolution: int, materials: dict):
        """voxelizeMesh with colours: (cells int32[n, 3], colours float32[n, 3], origin, voxel)."""
        p = _f32(positions).reshape(-1, 9)
        m, keep = make_materials(materials)
        cap = 1 << 16
        while True:
            cells = np.empty((cap, 3), np.int32)
            cols = np.empty((cap, 3), np.float32)
            cnt = _u64()
            origin = np.empty(3, np.float32)
            vox = C.c_float()
            self._check(self.lib.sdfb_voxelize_sparse_colors(
                self.h, _ptr(p), len(p), _ptr(_f32(bmin).reshape(3)), _ptr(_f32(bmax).reshape(3)), int(resolution),
                C.byref(m), _ptr(cells), _ptr(cols), cap, C.byref(cnt), _ptr(origin), C.byref(vox)))
            if cnt.value <= cap:
                del keep
                return cells[:cnt.value].copy(), cols[:cnt.value].copy(), origin, vox.value
            cap = int(cnt.value)

    def weld_device(self, d_positions: int, num_positions: int, bmin, bmax, d_welded_out: int, stream: int = 0) -> int:
        """Device weld; returns the unique count (welded indices are written to d_welded_out)."""
        u = _u32()
        self._check(self.lib.sdfb_weld_device(self.h, C.c_void_p(d_positions), num_positions,
                                              _ptr(_f32(bmin).reshape(3)), _ptr(_f32(bmax).reshape(3)),
                                              C.c_void_p(d_welded_out), C.byref(u), C.c_void_p(stream)))
        return u.value

    def is_watertight_device(self, d_welded: int, num_tris: int, stream: int = 0):
        """Device watertight census: (watertight, boundary edges, non-manifold edges)."""
        w, b, m = _i32(), _u64(), _u64()
        self._check(self.lib.sdfb_is_watertight_device(self.h, C.c_void_p(d_welded), num_tris, C.byref(w), C.byref(b),
                                                       C.byref(m), C.c_void_p(stream)))
        return bool(w.value), b.value, m.value

    def sample_sdf(self, grid: GridDesc, dist, points) -> np.ndarray:
        """The renderer's trilinear sample (sampleSdf) of a baked grid at points (n, 3)."""
        d = _f32(dist).reshape(-1)
        p = _f32(points).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        self._check(self.lib.sdfb_sample_sdf(self.h, C.byref(grid), _ptr(d), _ptr(p), len(p), _ptr(out)))
        return out

    def trace_sdf(self, grid: GridDesc, dist, rays, tmin: float = 0.0, tmax: float = 1e30) -> np.ndarray:
        """The renderer's SDF intersection per ray (n, 6): hit distance or -1."""
        d = _f32(dist).reshape(-1)
        r = _f32(rays).reshape(-1, 6)
        out = np.empty(len(r), np.float32)
        self._check(self.lib.sdfb_trace_sdf(self.h, C.byref(grid), _ptr(d), _ptr(r), len(r), float(tmin),
                                            float(tmax), _ptr(out)))
        return out

    def voxelize_sparse(self, positions, bmin, bmax, resolution: int):
        p = _f32(positions).reshape(-1, 3)
        cap = max(1024, 4 * len(p))
        while True:
            cells = np.empty((cap, 3), np.int32)
            cnt = C.c_uint64()
            o = np.zeros(3, np.float32)
            v = C.c_float()
            st = self.lib.sdfb_voxelize_sparse(self.h, _ptr(p), len(p) // 3, _ptr(_f32(bmin)), _ptr(_f32(bmax)),
                                               int(resolution), _ptr(cells), cap, C.byref(cnt), _ptr(o), C.byref(v))
            self._check(st)
            if cnt.value <= cap:
                return cells[:cnt.value].copy(), o, float(np.float32(v.value))
            cap = int(cnt.value)

    def bake_batch(self, meshes, grids, opts: Opts | None = None, want_dist=True, want_occ=True,
                   stats: Stats | None = None, out=None):
        """Host-buffer batched bake of [(verts, idx), ...] onto [GridDesc, ...]. Returns
        ([dist], [occ]); `out` may pass preallocated (dists, occs) lists (pinned memory is fastest)."""
        n = len(meshes)
        vs = [_f32(v).reshape(-1, 3) for v, _ in meshes]
        fs = [_u32a(f).reshape(-1, 3) for _, f in meshes]
        descs = (MeshDesc * n)()
        for k in range(n):
            descs[k].verts = vs[k].ctypes.data
            descs[k].idx = fs[k].ctypes.data
            descs[k].num_verts = len(vs[k])
            descs[k].num_tris = len(fs[k])
        gs = (GridDesc * n)(*grids)
        if out is not None:
            dists, occs = out
        else:
            dists = [np.empty(g.shape, np.float32) for g in grids] if want_dist else None
            occs = [np.empty(g.shape, np.uint8) for g in grids] if want_occ else None
        dp = (C.c_void_p * n)(*[d.ctypes.data for d in dists]) if dists is not None else None
        op = (C.c_void_p * n)(*[o.ctypes.data for o in occs]) if occs is not None else None
        st = self.lib.sdfb_bake_batch(self.h, n, descs, gs, C.byref(opts) if opts is not None else None, dp, op,
                                      C.byref(stats) if stats is not None else None)
        self._check(st)
        return dists, occs

    def bake_batch_device(self, dev_meshes, grids, opts: Opts | None, dist_ptrs, occ_ptrs, stream: int = 0,
                          stats: Stats | None = None):
        """dev_meshes: [(verts_ptr, num_verts, idx_ptr, num_tris)]; pointers are device addresses."""
        n = len(dev_meshes)
        descs = (MeshDesc * n)()
        for k, (vp, nv, ip, nt) in enumerate(dev_meshes):
            descs[k].verts = vp
            descs[k].idx = ip
            descs[k].num_verts = nv
            descs[k].num_tris = nt
        gs = (GridDesc * n)(*grids)
        dp = (C.c_void_p * n)(*dist_ptrs) if dist_ptrs is not None else None
        op = (C.c_void_p * n)(*occ_ptrs) if occ_ptrs is not None else None
        st = self.lib.sdfb_bake_batch_device(self.h, n, descs, gs, C.byref(opts) if opts is not None else None, dp, op,
                                             C.c_void_p(stream), C.byref(stats) if stats is not None else None)
        self._check(st)

    def device_bytes(self) -> int:
        return int(self.lib.sdfb_ctx_device_bytes(self.h))


class Server:
    """Continuous-batching bake server over device-resident meshes (sdfb_server_*)."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int = 0, max_inflight: int = 0, wave_voxels_log2: int = 0):
        self.lib = ctx.lib
        o = ServerOpts()
        o.struct_size = C.sizeof(ServerOpts)
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.max_inflight = int(max_inflight)
        o.wave_voxels_log2 = int(wave_voxels_log2)
        h = C.c_void_p()
        st = self.lib.sdfb_server_create(ctx.h, C.byref(o), C.byref(h))
        if st != OK:
            raise SdfbError(st, ctx.error())
        self.h = h
        self._keep = {}

    def close(self):
        if self.h:
            self.lib.sdfb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def error(self) -> str:
        return (self.lib.sdfb_server_last_error(self.h) or b"").decode()

    def register(self, verts, idx) -> int:
        v = _f32(verts).reshape(-1, 3)
        i = _u32a(idx).reshape(-1, 3)
        mid = C.c_uint64()
        st = self.lib.sdfb_mesh_register(self.h, _ptr(v), len(v), _ptr(i), len(i), C.byref(mid))
        if st != OK:
            raise SdfbError(st, self.error())
        return int(mid.value)

    def submit(self, mesh_id: int, grid: GridDesc, dist: np.ndarray | None, occ: np.ndarray | None,
               opts: Opts | None = None) -> int:
        """Queues a bake; dist / occ are caller-owned arrays of grid.cells elements that must stay
        alive until poll reports the request done."""
        rid = C.c_uint64()
        st = self.lib.sdfb_submit(self.h, C.c_uint64(mesh_id), C.byref(grid), C.byref(opts) if opts else None,
                                  _ptr(dist), _ptr(occ), C.byref(rid))
        if st != OK:
            raise SdfbError(st, self.error())
        self._keep[int(rid.value)] = (dist, occ)
        return int(rid.value)

    def poll(self, request_id: int, timeout_ms: int = -1):
        """Returns (done, info dict); raises if the finished request failed."""
        done = C.c_int32()
        info = RequestInfo()
        info.struct_size = C.sizeof(RequestInfo)
        st = self.lib.sdfb_poll(self.h, C.c_uint64(request_id), int(timeout_ms), C.byref(done), C.byref(info))
        if done.value:
            self._keep.pop(request_id, None)
        if st != OK:
            raise SdfbError(st, self.error())
        d = {k: getattr(info, k) for k, _ in RequestInfo._fields_ if k not in ("struct_size", "pad")}
        return bool(done.value), d
