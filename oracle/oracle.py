"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference legs use this
module, and only as the reference for comparisons or the timed CPU baseline; the product library
never imports it.

``Oracle`` wraps ``oracle/_build/liboracle.so`` (this project's restatement, see sdf_oracle.c).
``Reference`` wraps ``oracle/_ref/libitaly_ref.so``, the reference's own CPU sources compiled
here (absent on machines without the reference tree).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle as _b

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _grid_args(origin, voxel, n):
    return _f32(origin).reshape(3), C.c_float(voxel), int(n[0]), int(n[1]), int(n[2])


def flat_materials(m: dict) -> dict:
    """Flattens a material set -- {"mat_f": (M, 5) base colour rgb, metallic, roughness;
    "mat_tex": (M,) texture index or -1; "tri_mat": per-triangle material index; "uvs": (N, 2) one
    pair per soup vertex; "textures": [(rgba uint8 (h, w, 4), srgb bool), ...]} -- into the C
    arrays the oracle and the reference driver take."""
    tex = m.get("textures", [])
    pix = [np.ascontiguousarray(t[0], np.uint8).reshape(-1) for t in tex]
    off = np.zeros(max(len(tex), 1), np.int64)
    if tex:
        off[1:len(tex)] = np.cumsum([len(p) for p in pix])[:-1]
    return {
        "mat_f": np.ascontiguousarray(m["mat_f"], np.float32).reshape(-1),
        "mat_tex": np.ascontiguousarray(m["mat_tex"], np.int32).reshape(-1),
        "nmat": len(m["mat_tex"]),
        "tri_mat": np.ascontiguousarray(m.get("tri_mat", np.zeros(0)), np.uint32).reshape(-1),
        "uvs": np.ascontiguousarray(m.get("uvs", np.zeros((0, 2))), np.float32).reshape(-1),
        "pixels": np.concatenate(pix) if pix else np.zeros(1, np.uint8),
        "tex_off": off,
        "tex_w": np.array([t[0].shape[1] for t in tex] or [0], np.int32),
        "tex_h": np.array([t[0].shape[0] for t in tex] or [0], np.int32),
        "tex_srgb": np.array([1 if t[1] else 0 for t in tex] or [0], np.int32),
        "ntex": len(tex),
    }


class _OrcMaterials(C.Structure):
    _fields_ = [("mat_f", C.c_void_p), ("mat_tex", C.c_void_p), ("nmat", C.c_int64), ("tri_mat", C.c_void_p),
                ("ntri_mat", C.c_int64), ("uvs", C.c_void_p), ("nuv", C.c_int64), ("pixels", C.c_void_p),
                ("tex_off", C.c_void_p), ("tex_w", C.c_void_p), ("tex_h", C.c_void_p), ("tex_srgb", C.c_void_p),
                ("ntex", C.c_int64)]


def _orc_materials(f: dict) -> _OrcMaterials:
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    return _OrcMaterials(p(f["mat_f"]), p(f["mat_tex"]), f["nmat"], p(f["tri_mat"]), len(f["tri_mat"]), p(f["uvs"]),
                         len(f["uvs"]) // 2, p(f["pixels"]), p(f["tex_off"]), p(f["tex_w"]), p(f["tex_h"]),
                         p(f["tex_srgb"]), f["ntex"])


def _ref_material_args(f: dict):
    return (f["mat_f"], f["mat_tex"], f["nmat"], f["tri_mat"], len(f["tri_mat"]), f["uvs"], len(f["uvs"]) // 2,
            f["pixels"], f["tex_off"], f["tex_w"], f["tex_h"], f["tex_srgb"], f["ntex"])


_REF_MAT_TYPES = [_f32p, _i32p, C.c_int64, _u32p, C.c_int64, _f32p, C.c_int64, _u8p, _i64p, _i32p, _i32p, _i32p,
                  C.c_int64]


class Oracle:
    def __init__(self, path: str | None = None):
        path = path or _b.build_oracle()
        L = C.CDLL(path)
        self.lib = L
        L.orc_grid_from_bounds.argtypes = [_f32p, _f32p, C.c_int32, _f32p, C.POINTER(C.c_float), _i32p]
        L.orc_grid_from_bounds.restype = None
        L.orc_occupancy_dense.argtypes = [_f32p, C.c_int64, C.c_void_p, C.c_int64, _f32p, C.c_float, C.c_int32,
                                          C.c_int32, C.c_int32, _u8p]
        L.orc_occupancy_dense.restype = C.c_int32
        L.orc_tri_box_overlap.argtypes = [_f32p] * 5
        L.orc_tri_box_overlap.restype = C.c_int32
        L.orc_voxelize_sparse.argtypes = [_f32p, C.c_int64, _f32p, _f32p, C.c_int32, _i32p, C.c_int64, _f32p,
                                          C.POINTER(C.c_float)]
        L.orc_voxelize_sparse.restype = C.c_int64
        L.orc_weld.argtypes = [_f32p, C.c_int64, _f32p, _f32p, _u32p]
        L.orc_weld.restype = C.c_int64
        L.orc_watertight.argtypes = [_u32p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_watertight.restype = C.c_int32
        L.orc_distance.argtypes = [_f32p, C.c_void_p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32,
                                   C.c_void_p, C.c_int64, _f64p, C.c_void_p, C.c_int32]
        L.orc_distance.restype = C.c_int32
        L.orc_sign_parity.argtypes = [_f32p, C.c_void_p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32,
                                      C.c_int32, C.c_int32, _i8p, C.c_int32]
        L.orc_sign_parity.restype = C.c_int32
        L.orc_gwn.argtypes = [_f32p, C.c_void_p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32,
                              C.c_void_p, C.c_int64, _f64p, C.c_int32]
        L.orc_gwn.restype = C.c_int32
        L.orc_column_crossing.argtypes = [_f32p, _f32p, _f32p, C.c_int32, C.c_float, C.c_float,
                                          C.POINTER(C.c_double)]
        L.orc_column_crossing.restype = C.c_int32
        L.orc_orient2_sos.argtypes = [C.c_float] * 6
        L.orc_orient2_sos.restype = C.c_int32
        L.orc_default_threads.restype = C.c_int32
        L.orc_sample_sdf.argtypes = [_f32p, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32, _f32p, C.c_int64,
                                     _f32p]
        L.orc_sample_sdf.restype = None
        L.orc_trace_sdf.argtypes = [_f32p, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32, _f32p, C.c_int64,
                                    C.c_float, C.c_float, _f32p]
        L.orc_trace_sdf.restype = None
        L.orc_ray_mesh.argtypes = [_f32p, C.c_void_p, C.c_int64, _f32p, C.c_int64, _f64p]
        L.orc_ray_mesh.restype = None
        L.orc_triangle_material.argtypes = [C.POINTER(_OrcMaterials), C.c_int64, _f32p]
        L.orc_triangle_material.restype = None
        L.orc_materials_dense.argtypes = [_f32p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32,
                                          C.POINTER(_OrcMaterials), _f32p, _f32p, _f32p]
        L.orc_materials_dense.restype = C.c_int32
        L.orc_voxelize_colors.argtypes = [_f32p, C.c_int64, _f32p, _f32p, C.c_int32, C.POINTER(_OrcMaterials), _i32p,
                                          _f32p, C.c_int64, _f32p, C.POINTER(C.c_float)]
        L.orc_voxelize_colors.restype = C.c_int64

    @staticmethod
    def _mesh(verts, idx):
        v = _f32(verts).reshape(-1, 3)
        if idx is None:
            return v, None, len(v) // 3, None
        i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        return v, i, len(i), i.ctypes.data_as(C.c_void_p)

    def threads(self) -> int:
        return int(self.lib.orc_default_threads())

    def grid_from_bounds(self, bmin, bmax, res):
        o = np.zeros(3, np.float32)
        v = C.c_float()
        n = np.zeros(3, np.int32)
        self.lib.orc_grid_from_bounds(_f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res), o, C.byref(v), n)
        return o, float(np.float32(v.value)), tuple(int(x) for x in n)

    def tri_box_overlap(self, center, half, t0, t1, t2) -> bool:
        return bool(self.lib.orc_tri_box_overlap(*(_f32(a).reshape(3) for a in (center, half, t0, t1, t2))))

    def occupancy(self, verts, idx, origin, voxel, n) -> np.ndarray:
        v, i, T, ip = self._mesh(verts, idx)
        occ = np.empty(int(n[0]) * int(n[1]) * int(n[2]), np.uint8)
        rc = self.lib.orc_occupancy_dense(v, len(v), ip, T, *_grid_args(origin, voxel, n), occ)
        if rc != 0:
            raise ValueError("triangle index out of range")
        return occ

    def voxelize_sparse(self, soup, bmin, bmax, res):
        s = _f32(soup).reshape(-1, 3)
        cap = 1 << 16
        while True:
            cells = np.empty((cap, 3), np.int32)
            o = np.zeros(3, np.float32)
            v = C.c_float()
            n = self.lib.orc_voxelize_sparse(s, len(s) // 3, _f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res),
                                             cells, cap, o, C.byref(v))
            if n < 0:
                raise MemoryError
            if n <= cap:
                return cells[:n].copy(), o, float(np.float32(v.value))
            cap = int(n)

    def sample_sdf(self, dist, origin, voxel, n, points) -> np.ndarray:
        """The renderer's trilinear sample of a baked grid (sampleSdf) at points (k, 3)."""
        p = _f32(points).reshape(-1, 3)
        out = np.empty(len(p), np.float32)
        self.lib.orc_sample_sdf(_f32(dist).reshape(-1), *_grid_args(origin, voxel, n), p.reshape(-1), len(p), out)
        return out

    def trace_sdf(self, dist, origin, voxel, n, rays, tmin=0.0, tmax=1e30) -> np.ndarray:
        """The renderer's SDF ray march per ray (k, 6): reported hit distance or -1."""
        r = _f32(rays).reshape(-1, 6)
        out = np.empty(len(r), np.float32)
        self.lib.orc_trace_sdf(_f32(dist).reshape(-1), *_grid_args(origin, voxel, n), r.reshape(-1), len(r),
                               float(tmin), float(tmax), out)
        return out

    def ray_mesh(self, verts, idx, rays) -> np.ndarray:
        """Exact FP64 first hit t > 0 of each ray with the mesh, or -1."""
        v, i, T, ip = self._mesh(verts, idx)
        r = _f32(rays).reshape(-1, 6)
        out = np.empty(len(r), np.float64)
        self.lib.orc_ray_mesh(v, ip, T, r.reshape(-1), len(r), out)
        return out

    def triangle_materials(self, ntris, materials) -> np.ndarray:
        f = flat_materials(materials)
        om = _orc_materials(f)
        out = np.empty((ntris, 5), np.float32)
        row = np.empty(5, np.float32)
        for t in range(ntris):
            self.lib.orc_triangle_material(C.byref(om), t, row)
            out[t] = row
        return out

    def materials_dense(self, soup, origin, voxel, n, materials):
        """bakePerCellMaterial over an explicit grid: (base colour (cells, 3), metallic, roughness)."""
        s = _f32(soup).reshape(-1, 3)
        f = flat_materials(materials)
        cells = int(n[0]) * int(n[1]) * int(n[2])
        col = np.empty((cells, 3), np.float32)
        met = np.empty(cells, np.float32)
        rou = np.empty(cells, np.float32)
        rc = self.lib.orc_materials_dense(s, len(s) // 3, *_grid_args(origin, voxel, n), C.byref(_orc_materials(f)),
                                          col.reshape(-1), met, rou)
        if rc != 0:
            raise MemoryError
        return col, met, rou

    def voxelize_colors(self, soup, bmin, bmax, res, materials):
        """voxelizeMesh with colours: (cells (n, 3) int32, colours (n, 3) float32)."""
        s = _f32(soup).reshape(-1, 3)
        f = flat_materials(materials)
        om = _orc_materials(f)
        cap = 1 << 16
        while True:
            cells = np.empty((cap, 3), np.int32)
            cols = np.empty((cap, 3), np.float32)
            o = np.zeros(3, np.float32)
            v = C.c_float()
            n = self.lib.orc_voxelize_colors(s, len(s) // 3, _f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res),
                                             C.byref(om), cells, cols.reshape(-1), cap, o, C.byref(v))
            if n < 0:
                raise MemoryError
            if n <= cap:
                return cells[:n].copy(), cols[:n].copy()
            cap = int(n)

    def weld(self, positions, bmin, bmax):
        p = _f32(positions).reshape(-1, 3)
        out = np.empty(len(p), np.uint32)
        n = self.lib.orc_weld(p, len(p), _f32(bmin).reshape(3), _f32(bmax).reshape(3), out)
        return out, int(n)

    def watertight(self, welded_idx):
        w = np.ascontiguousarray(welded_idx, dtype=np.uint32).reshape(-1)
        b, m = C.c_int64(), C.c_int64()
        rc = self.lib.orc_watertight(w, len(w) // 3, C.byref(b), C.byref(m))
        return rc == 1, int(b.value), int(m.value)

    def distance(self, verts, idx, origin, voxel, n, samples=None, threads=0, want_tri=False):
        v, i, T, ip = self._mesh(verts, idx)
        if samples is None:
            cnt = int(n[0]) * int(n[1]) * int(n[2])
            sp = None
        else:
            s = np.ascontiguousarray(samples, dtype=np.int64)
            cnt = len(s)
            sp = s.ctypes.data_as(C.c_void_p)
        out = np.empty(cnt, np.float64)
        tri = np.empty(cnt, np.int64) if want_tri else None
        rc = self.lib.orc_distance(v, ip, T, *_grid_args(origin, voxel, n), sp, cnt, out,
                                   tri.ctypes.data_as(C.c_void_p) if want_tri else None, int(threads))
        if rc != 0:
            raise MemoryError
        return (out, tri) if want_tri else out

    def sign_parity(self, verts, idx, origin, voxel, n, axis=2, threads=0) -> np.ndarray:
        v, i, T, ip = self._mesh(verts, idx)
        out = np.empty(int(n[0]) * int(n[1]) * int(n[2]), np.int8)
        rc = self.lib.orc_sign_parity(v, ip, T, *_grid_args(origin, voxel, n), int(axis), out, int(threads))
        if rc != 0:
            raise MemoryError
        return out

    def gwn(self, verts, idx, origin, voxel, n, samples=None, threads=0) -> np.ndarray:
        v, i, T, ip = self._mesh(verts, idx)
        if samples is None:
            cnt = int(n[0]) * int(n[1]) * int(n[2])
            sp = None
        else:
            s = np.ascontiguousarray(samples, dtype=np.int64)
            cnt = len(s)
            sp = s.ctypes.data_as(C.c_void_p)
        out = np.empty(cnt, np.float64)
        self.lib.orc_gwn(v, ip, T, *_grid_args(origin, voxel, n), sp, cnt, out, int(threads))
        return out

    def column_crossing(self, a, b, c, axis, pu, pv):
        t = C.c_double()
        hit = self.lib.orc_column_crossing(_f32(a), _f32(b), _f32(c), int(axis), float(pu), float(pv), C.byref(t))
        return bool(hit), t.value

    def orient2_sos(self, au, av, bu, bv, pu, pv) -> int:
        return int(self.lib.orc_orient2_sos(au, av, bu, bv, pu, pv))


class Reference:
    """The reference's own CPU code for the bake path, compiled from its sources (oracle/_ref)."""

    def __init__(self, path: str | None = None):
        path = path or _b.build_ref()
        if not path or not os.path.exists(path):
            raise FileNotFoundError("oracle/_ref/libitaly_ref.so is not built (the reference tree is absent)")
        L = C.CDLL(path)
        self.lib = L
        L.ref_grid_from_bounds.argtypes = [_f32p, _f32p, C.c_int32, _f32p, C.POINTER(C.c_float), _i32p]
        L.ref_grid_from_bounds.restype = None
        L.ref_occupancy_dense.argtypes = [_f32p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32, _u8p]
        L.ref_occupancy_dense.restype = None
        L.ref_voxelize.argtypes = [_f32p, C.c_int64, _f32p, _f32p, C.c_int32, _i32p, C.c_int64, _f32p,
                                   C.POINTER(C.c_float)]
        L.ref_voxelize.restype = C.c_int64
        L.ref_weld.argtypes = [_f32p, C.c_int64, _f32p, _f32p, _u32p]
        L.ref_weld.restype = C.c_int64
        L.ref_is_watertight.argtypes = [_f32p, C.c_int64, _f32p, _f32p, C.c_char_p, C.c_int32]
        L.ref_is_watertight.restype = C.c_int32
        L.ref_voxelize_colors.argtypes = [_f32p, C.c_int64, _f32p, _f32p, C.c_int32, *_REF_MAT_TYPES, _i32p, _f32p,
                                          C.c_int64]
        L.ref_voxelize_colors.restype = C.c_int64
        L.ref_materials_dense.argtypes = [_f32p, C.c_int64, _f32p, C.c_float, C.c_int32, C.c_int32, C.c_int32,
                                          *_REF_MAT_TYPES, _f32p, _f32p, _f32p]
        L.ref_materials_dense.restype = None

    def voxelize_colors(self, soup, bmin, bmax, res, materials):
        s = _f32(soup).reshape(-1, 3)
        f = flat_materials(materials)
        cap = 1 << 16
        while True:
            cells = np.empty((cap, 3), np.int32)
            cols = np.empty((cap, 3), np.float32)
            n = self.lib.ref_voxelize_colors(s, len(s) // 3, _f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res),
                                             *_ref_material_args(f), cells, cols.reshape(-1), cap)
            if n <= cap:
                return cells[:n].copy(), cols[:n].copy()
            cap = int(n)

    def materials_dense(self, soup, origin, voxel, n, materials):
        s = _f32(soup).reshape(-1, 3)
        f = flat_materials(materials)
        cells = int(n[0]) * int(n[1]) * int(n[2])
        col = np.empty((cells, 3), np.float32)
        met = np.empty(cells, np.float32)
        rou = np.empty(cells, np.float32)
        self.lib.ref_materials_dense(s, len(s) // 3, *_grid_args(origin, voxel, n), *_ref_material_args(f),
                                     col.reshape(-1), met, rou)
        return col, met, rou

    def grid_from_bounds(self, bmin, bmax, res):
        o = np.zeros(3, np.float32)
        v = C.c_float()
        n = np.zeros(3, np.int32)
        self.lib.ref_grid_from_bounds(_f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res), o, C.byref(v), n)
        return o, float(np.float32(v.value)), tuple(int(x) for x in n)

    def occupancy(self, soup, origin, voxel, n) -> np.ndarray:
        s = _f32(soup).reshape(-1, 3)
        occ = np.empty(int(n[0]) * int(n[1]) * int(n[2]), np.uint8)
        self.lib.ref_occupancy_dense(s, len(s) // 3, *_grid_args(origin, voxel, n), occ)
        return occ

    def voxelize(self, soup, bmin, bmax, res):
        s = _f32(soup).reshape(-1, 3)
        cap = 1 << 16
        while True:
            cells = np.empty((cap, 3), np.int32)
            o = np.zeros(3, np.float32)
            v = C.c_float()
            n = self.lib.ref_voxelize(s, len(s) // 3, _f32(bmin).reshape(3), _f32(bmax).reshape(3), int(res), cells,
                                      cap, o, C.byref(v))
            if n <= cap:
                return cells[:n].copy(), o, float(np.float32(v.value))
            cap = int(n)

    def weld(self, positions, bmin, bmax):
        p = _f32(positions).reshape(-1, 3)
        out = np.empty(len(p), np.uint32)
        n = self.lib.ref_weld(p, len(p), _f32(bmin).reshape(3), _f32(bmax).reshape(3), out)
        return out, int(n)

    def is_watertight(self, soup, bmin, bmax):
        s = _f32(soup).reshape(-1, 3)
        buf = C.create_string_buffer(512)
        ok = self.lib.ref_is_watertight(s, len(s) // 3, _f32(bmin).reshape(3), _f32(bmax).reshape(3), buf, 512)
        return bool(ok), buf.value.decode("utf-8", "replace")


def soup_of(verts, idx) -> np.ndarray:
    """The reference's MeshAsset layout: 3 positions per triangle."""
    v = _f32(verts).reshape(-1, 3)
    i = np.asarray(idx, dtype=np.int64).reshape(-1)
    return np.ascontiguousarray(v[i])
