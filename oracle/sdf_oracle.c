/*
 * CPU oracle for the mesh -> SDF bake. TEST INFRASTRUCTURE ONLY: it is loaded by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg, and is never linked into or called by
 * the product library (italy-rs_gb300/). Compile with -ffp-contract=off and without -ffast-math:
 * the FP32 parts must round exactly like the reference.
 *
 * What it restates, with the reference lines each part follows:
 *   orc_grid_from_bounds   grid sizing of bakeSdf, src/convert/sdf_baker.cpp:138-148
 *   orc_occupancy_dense    candidate-cell loop of bakePerCellMaterial, sdf_baker.cpp:89-118, with
 *                          occupancy = (count > 0) as at :115,121-122
 *   orc_voxelize_sparse    voxelizeMesh, src/convert/voxelize.cpp:52-107 (insertion-ordered cells)
 *   sat_overlap            triBoxOverlap, src/convert/tri_box_overlap.h:12-114 (FP32, same rounding)
 *   orc_materials_dense    per-cell material averages of bakePerCellMaterial,
 *                          sdf_baker.cpp:76-128, with triangleMaterial / sampleColorNearest /
 *                          srgbToLinear of sdf_baker.cpp:42-74
 *   orc_voxelize_colors    voxelizeMesh's per-cell colours, voxelize.cpp:12-37,52-107
 *   orc_sample_sdf,        the renderer's consumption of a baked grid: sampleSdf and
 *   orc_trace_sdf          __intersection__sdf with its slab test, src/render/kernels/
 *                          pathtracer.cu:587-613,684-702,740-787 (one IEEE operation per
 *                          operation, no contraction), and orc_ray_mesh, the exact FP64 first
 *                          ray/triangle hit (Moller & Trumbore, 1997) they are checked against
 *   orc_weld               weldPositions, src/io/mesh_weld.cpp:26-48
 *   orc_watertight         isWatertight, src/io/mesh_validate.cpp:21-59
 * and, because the reference's own distance/sign is an OptiX ray-cast estimate
 * (src/render/kernels/sdf_bake.cu:32-73) that cannot meet the accuracy target, the exact
 * quantities the bake is specified against:
 *   orc_distance           FP64 unsigned distance from the FP32 cell centre
 *                          (sdf_bake.cu:34-37 sample point) to the nearest triangle, by the
 *                          Voronoi-region closest-point method (Ericson, Real-Time Collision
 *                          Detection, 2005, sec. 5.1.5) through a median-split BVH.
 *   orc_sign_parity        exact ray parity along a chosen axis (the reference's first parity
 *                          ray is +z, sdf_bake.cu:56): orientation by an exact sum-of-products
 *                          expansion (Shewchuk, "Adaptive Precision Floating-Point Arithmetic",
 *                          1997: Two-Sum / Grow-Expansion) with simulation-of-simplicity
 *                          tie-breaking (Edelsbrunner & Muecke, 1990).
 *   orc_gwn                FP64 generalized winding number (Jacobson, Kavan & Sorkine-Hornung,
 *                          2013) as the sum of triangle solid angles (Van Oosterom & Strackee,
 *                          1983), summed directly.
 * The sign convention is the reference's: negative inside (sdf_bake.cu:69-72).
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------------------------ */
/* FP32 triangle / box separating-axis test (tri_box_overlap.h:12-114).                        */
/* Each C statement performs exactly the rounded operations of the reference, in its order.   */

typedef struct { float x, y, z; } f3;

static inline f3 f3_sub(f3 a, f3 b) { f3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline float fmin_ref(float a, float b) { return (b < a) ? b : a; } /* std::min */
static inline float fmax_ref(float a, float b) { return (a < b) ? b : a; } /* std::max */
static inline float f3_get(f3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

/* One of the nine edge-cross-axis tests: projections pa, pb of two vertices against radius
 * rad; the triangle and box are separated along the axis when min > rad or max < -rad. */
static inline int axis_overlaps(float pa, float pb, float rad) {
  const float mn = fmin_ref(pa, pb), mx = fmax_ref(pa, pb);
  return !(mn > rad || mx < -rad);
}

/* Projections onto e x X, e x Y, e x Z for edge components (a, b) as the reference pairs them. */
static inline float proj_x(float a, float b, f3 v) { return a * v.y - b * v.z; }
static inline float proj_y(float a, float b, f3 v) { return -a * v.x + b * v.z; }
static inline float proj_z(float a, float b, f3 v) { return a * v.x - b * v.y; }

static int plane_box_overlap(f3 n, f3 vert, f3 h) {
  float vmin[3], vmax[3];
  for (int q = 0; q < 3; ++q) {
    const float nq = f3_get(n, q), v = f3_get(vert, q), hq = f3_get(h, q);
    if (nq > 0.0f) {
      vmin[q] = -hq - v;
      vmax[q] = hq - v;
    } else {
      vmin[q] = hq - v;
      vmax[q] = -hq - v;
    }
  }
  /* glm::dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z */
  const float dmin = n.x * vmin[0] + n.y * vmin[1] + n.z * vmin[2];
  if (dmin > 0.0f) return 0;
  const float dmax = n.x * vmax[0] + n.y * vmax[1] + n.z * vmax[2];
  return dmax >= 0.0f;
}

static int sat_overlap(f3 c, f3 h, f3 t0, f3 t1, f3 t2) {
  const f3 v0 = f3_sub(t0, c), v1 = f3_sub(t1, c), v2 = f3_sub(t2, c);
  const f3 e0 = f3_sub(v1, v0), e1 = f3_sub(v2, v1), e2 = f3_sub(v0, v2);
  float fx = fabsf(e0.x), fy = fabsf(e0.y), fz = fabsf(e0.z);
  if (!axis_overlaps(proj_x(e0.z, e0.y, v0), proj_x(e0.z, e0.y, v2), fz * h.y + fy * h.z)) return 0;
  if (!axis_overlaps(proj_y(e0.z, e0.x, v0), proj_y(e0.z, e0.x, v2), fz * h.x + fx * h.z)) return 0;
  if (!axis_overlaps(proj_z(e0.y, e0.x, v1), proj_z(e0.y, e0.x, v2), fy * h.x + fx * h.y)) return 0;
  fx = fabsf(e1.x); fy = fabsf(e1.y); fz = fabsf(e1.z);
  if (!axis_overlaps(proj_x(e1.z, e1.y, v0), proj_x(e1.z, e1.y, v2), fz * h.y + fy * h.z)) return 0;
  if (!axis_overlaps(proj_y(e1.z, e1.x, v0), proj_y(e1.z, e1.x, v2), fz * h.x + fx * h.z)) return 0;
  if (!axis_overlaps(proj_z(e1.y, e1.x, v0), proj_z(e1.y, e1.x, v1), fy * h.x + fx * h.y)) return 0;
  fx = fabsf(e2.x); fy = fabsf(e2.y); fz = fabsf(e2.z);
  if (!axis_overlaps(proj_x(e2.z, e2.y, v0), proj_x(e2.z, e2.y, v1), fz * h.y + fy * h.z)) return 0;
  if (!axis_overlaps(proj_y(e2.z, e2.x, v0), proj_y(e2.z, e2.x, v1), fz * h.x + fx * h.z)) return 0;
  if (!axis_overlaps(proj_z(e2.y, e2.x, v1), proj_z(e2.y, e2.x, v2), fy * h.x + fx * h.y)) return 0;
  for (int a = 0; a < 3; ++a) {
    const float p = f3_get(v0, a), q = f3_get(v1, a), r = f3_get(v2, a), hh = f3_get(h, a);
    const float lo = fmin_ref(fmin_ref(p, q), r), hi = fmax_ref(fmax_ref(p, q), r);
    if (lo > hh || hi < -hh) return 0;
  }
  /* glm::cross(e0, e1) */
  const f3 n = {e0.y * e1.z - e1.y * e0.z, e0.z * e1.x - e1.z * e0.x, e0.x * e1.y - e1.x * e0.y};
  return plane_box_overlap(n, v0, h);
}

int32_t orc_tri_box_overlap(const float *center, const float *half, const float *t0, const float *t1,
                            const float *t2) {
  const f3 c = {center[0], center[1], center[2]}, h = {half[0], half[1], half[2]};
  const f3 a = {t0[0], t0[1], t0[2]}, b = {t1[0], t1[1], t1[2]}, d = {t2[0], t2[1], t2[2]};
  return sat_overlap(c, h, a, b, d);
}

/* ------------------------------------------------------------------------------------------ */
/* Grid conventions.                                                                           */

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* float -> int as static_cast after floor; saturating, NaN -> 0 (the conversion CUDA and Arm
 * perform; on x86 out-of-range values become INT_MIN, which the clamp then maps to 0). */
static inline int f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return 2147483647;
  if (f <= -2147483648.0f) return (int)(-2147483647 - 1);
  return (int)f;
}

/* Cell centre: origin + (float(i) + 0.5f) * voxel (sdf_baker.cpp:107, sdf_bake.cu:34-37). */
static inline float cell_center(float origin, int i, float voxel) { return origin + ((float)i + 0.5f) * voxel; }

void orc_grid_from_bounds(const float *bmin, const float *bmax, int32_t res, float *origin_out, float *voxel_out,
                          int32_t *n_out) {
  const float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  float longest = ex;
  if (longest < ey) longest = ey;
  if (longest < ez) longest = ez;
  if (longest < 1e-6f) longest = 1e-6f;
  const float voxel = longest / (float)(res > 1 ? res : 1);
  const float pad = voxel * 2.0f;        /* voxelSize * kPad, kPad = 2 */
  const float pad2 = voxel * 2.0f * 2.0f; /* voxelSize * kPad * 2.0f */
  const float e[3] = {ex, ey, ez};
  for (int a = 0; a < 3; ++a) {
    origin_out[a] = bmin[a] - pad;
    const float padded = e[a] + pad2;
    n_out[a] = (int)ceilf(padded / voxel) + 1;
  }
  *voxel_out = voxel;
}

static inline void tri_cell_range(f3 p0, f3 p1, f3 p2, const float *origin, float voxel, const int *nmax, int lo[3],
                                  int hi[3]) {
  const float mn[3] = {fmin_ref(fmin_ref(p0.x, p1.x), p2.x), fmin_ref(fmin_ref(p0.y, p1.y), p2.y),
                       fmin_ref(fmin_ref(p0.z, p1.z), p2.z)};
  const float mx[3] = {fmax_ref(fmax_ref(p0.x, p1.x), p2.x), fmax_ref(fmax_ref(p0.y, p1.y), p2.y),
                       fmax_ref(fmax_ref(p0.z, p1.z), p2.z)};
  for (int a = 0; a < 3; ++a) {
    lo[a] = clampi(f2i_sat(floorf((mn[a] - origin[a]) / voxel)), 0, nmax[a]);
    hi[a] = clampi(f2i_sat(floorf((mx[a] - origin[a]) / voxel)), 0, nmax[a]);
  }
}

static inline f3 vtx(const float *verts, const uint32_t *idx, int64_t t, int k) {
  const uint32_t i = idx ? idx[3 * t + k] : (uint32_t)(3 * t + k);
  f3 r = {verts[3 * (int64_t)i], verts[3 * (int64_t)i + 1], verts[3 * (int64_t)i + 2]};
  return r;
}

/* Dense occupancy (sdf_baker.cpp:89-118). idx may be NULL for a soup (3 vertices per triangle).
 * Returns 0, or -1 when an index is out of range. */
int32_t orc_occupancy_dense(const float *verts, int64_t nverts, const uint32_t *idx, int64_t ntris,
                            const float *origin, float voxel, int32_t nx, int32_t ny, int32_t nz, uint8_t *occ) {
  const int64_t cells = (int64_t)nx * ny * nz;
  memset(occ, 0, (size_t)cells);
  const int nmax[3] = {nx - 1, ny - 1, nz - 1};
  const float half = voxel * 0.5f;
  const f3 h = {half, half, half};
  for (int64_t t = 0; t < ntris; ++t) {
    if (idx)
      for (int k = 0; k < 3; ++k)
        if ((int64_t)idx[3 * t + k] >= nverts) return -1;
    const f3 p0 = vtx(verts, idx, t, 0), p1 = vtx(verts, idx, t, 1), p2 = vtx(verts, idx, t, 2);
    int lo[3], hi[3];
    tri_cell_range(p0, p1, p2, origin, voxel, nmax, lo, hi);
    for (int z = lo[2]; z <= hi[2]; ++z)
      for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) {
          const f3 c = {cell_center(origin[0], x, voxel), cell_center(origin[1], y, voxel),
                        cell_center(origin[2], z, voxel)};
          if (sat_overlap(c, h, p0, p1, p2)) occ[((int64_t)z * ny + y) * nx + x] = 1;
        }
  }
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Open-addressing hash map with int64 triple keys (weld) or uint64 keys (edges).             */

typedef struct {
  int64_t *keys; /* 3 per slot for triples, 1 per slot otherwise */
  int64_t *vals;
  uint8_t *used;
  int64_t cap, size;
  int width;
} hmap;

static uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
  return x;
}

static int hmap_init(hmap *m, int64_t expected, int width) {
  int64_t cap = 16;
  while (cap < expected * 2) cap <<= 1;
  m->cap = cap; m->size = 0; m->width = width;
  m->keys = (int64_t *)malloc((size_t)(cap * width) * sizeof(int64_t));
  m->vals = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  m->used = (uint8_t *)calloc((size_t)cap, 1);
  return (m->keys && m->vals && m->used) ? 0 : -1;
}
static void hmap_free(hmap *m) { free(m->keys); free(m->vals); free(m->used); }

/* Returns the slot of key; *inserted tells whether it was new (value set to new_val). */
static int64_t hmap_get_or_insert(hmap *m, const int64_t *key, int64_t new_val, int *inserted) {
  uint64_t h = 0x9e3779b97f4a7c15ULL;
  for (int i = 0; i < m->width; ++i) h = mix64(h ^ (uint64_t)key[i]);
  int64_t s = (int64_t)(h & (uint64_t)(m->cap - 1));
  for (;;) {
    if (!m->used[s]) {
      m->used[s] = 1;
      memcpy(m->keys + s * m->width, key, (size_t)m->width * sizeof(int64_t));
      m->vals[s] = new_val;
      m->size++;
      *inserted = 1;
      return s;
    }
    if (memcmp(m->keys + s * m->width, key, (size_t)m->width * sizeof(int64_t)) == 0) {
      *inserted = 0;
      return s;
    }
    s = (s + 1) & (m->cap - 1);
  }
}

/* weldPositions (mesh_weld.cpp:26-48): lattice cell max(|extent| * 1e-5, 1e-6) in FP32, keys
 * lround(p / cell), indices in first-occurrence order. Returns the unique count, -1 on OOM. */
int64_t orc_weld(const float *pos, int64_t n, const float *bmin, const float *bmax, uint32_t *welded) {
  const float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  const float diag = sqrtf(ex * ex + ey * ey + ez * ez);
  float cell = diag * 1e-5f;
  if (cell < 1e-6f) cell = 1e-6f;
  hmap m;
  if (hmap_init(&m, n, 3)) return -1;
  for (int64_t i = 0; i < n; ++i) {
    int64_t key[3];
    for (int a = 0; a < 3; ++a) key[a] = (int64_t)lroundf(pos[3 * i + a] / cell);
    int ins;
    const int64_t s = hmap_get_or_insert(&m, key, m.size, &ins);
    welded[i] = (uint32_t)m.vals[s];
  }
  const int64_t uniq = m.size;
  hmap_free(&m);
  return uniq;
}

/* isWatertight (mesh_validate.cpp:21-59) over a welded index buffer: degenerate triangles are
 * skipped, edges used once are boundary, more than twice non-manifold. Returns 1 watertight,
 * 0 not, -1 empty mesh, -2 OOM. */
int32_t orc_watertight(const uint32_t *welded, int64_t ntris, int64_t *boundary_out, int64_t *nonmanifold_out) {
  *boundary_out = 0;
  *nonmanifold_out = 0;
  if (ntris == 0) return -1;
  hmap m;
  if (hmap_init(&m, ntris * 3, 1)) return -2;
  for (int64_t t = 0; t < ntris; ++t) {
    const uint32_t a = welded[3 * t], b = welded[3 * t + 1], c = welded[3 * t + 2];
    if (a == b || b == c || c == a) continue;
    const uint32_t e[3][2] = {{a, b}, {b, c}, {c, a}};
    for (int k = 0; k < 3; ++k) {
      uint32_t u = e[k][0], v = e[k][1];
      if (u > v) { const uint32_t tmp = u; u = v; v = tmp; }
      const int64_t key = (int64_t)(((uint64_t)u << 32) | v);
      int ins;
      const int64_t s = hmap_get_or_insert(&m, &key, 0, &ins);
      m.vals[s] += 1;
    }
  }
  int64_t boundary = 0, nonman = 0;
  for (int64_t s = 0; s < m.cap; ++s) {
    if (!m.used[s]) continue;
    if (m.vals[s] == 1) boundary++;
    else if (m.vals[s] > 2) nonman++;
  }
  hmap_free(&m);
  *boundary_out = boundary;
  *nonmanifold_out = nonman;
  return (boundary == 0 && nonman == 0) ? 1 : 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Materials: per-triangle material (sdf_baker.cpp:42-74; the same sampling as voxelize.cpp:12-37) */
/* and per-cell averages (sdf_baker.cpp:76-128, voxelize.cpp:52-107).                             */

typedef struct {
  const float *mat_f;     /* 5 per material: base colour r, g, b, metallic, roughness */
  const int32_t *mat_tex; /* base colour texture per material, -1 = none */
  int64_t nmat;           /* >= 1 */
  const uint32_t *tri_mat;
  int64_t ntri_mat;       /* may be < ntris (missing entries use material 0) */
  const float *uvs;       /* 2 floats per soup vertex */
  int64_t nuv;            /* uv pairs */
  const uint8_t *pixels;  /* every texture's RGBA8 texels, concatenated */
  const int64_t *tex_off; /* byte offset of each texture in pixels */
  const int32_t *tex_w, *tex_h, *tex_srgb;
  int64_t ntex;
} orc_materials;

/* srgbToLinear (sdf_baker.cpp:42, voxelize.cpp:12). */
static float srgb_to_linear(float c) { return c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f); }

/* float -> int as static_cast (truncation) for the texel coordinate; NaN -> 0 as f2i_sat. */
static inline int f2i_trunc(float f) { return f2i_sat(f); }

/* triangleMaterial (sdf_baker.cpp:61-74): out = base colour r, g, b, metallic, roughness. */
void orc_triangle_material(const orc_materials *m, int64_t t, float *out) {
  const int64_t mi0 = t < m->ntri_mat ? (int64_t)m->tri_mat[t] : 0;
  const int64_t mi = mi0 < m->nmat ? mi0 : 0;
  const float *f = m->mat_f + 5 * mi;
  float r = f[0], g = f[1], b = f[2];
  const int32_t tex = m->mat_tex[mi];
  const int64_t base = t * 3;
  if (tex >= 0 && tex < m->ntex && base + 2 < m->nuv) {
    const int32_t w = m->tex_w[tex], h = m->tex_h[tex];
    if (w > 0 && h > 0) {
      const float *u = m->uvs + 2 * base;
      const float uu = ((u[0] + u[2]) + u[4]) / 3.0f, vv = ((u[1] + u[3]) + u[5]) / 3.0f;
      const float wu = uu - floorf(uu), wv = vv - floorf(vv);
      const int px = clampi(f2i_trunc(wu * (float)w), 0, w - 1);
      const int py = clampi(f2i_trunc(wv * (float)h), 0, h - 1);
      const uint8_t *p = m->pixels + m->tex_off[tex] + ((int64_t)py * w + px) * 4;
      float cr = (float)p[0] / 255.0f, cg = (float)p[1] / 255.0f, cb = (float)p[2] / 255.0f;
      if (m->tex_srgb[tex]) {
        cr = srgb_to_linear(cr);
        cg = srgb_to_linear(cg);
        cb = srgb_to_linear(cb);
      }
      r = cr * f[0];
      g = cg * f[1];
      b = cb * f[2];
    }
  }
  out[0] = r; out[1] = g; out[2] = b; out[3] = f[3]; out[4] = f[4];
}

/* bakePerCellMaterial (sdf_baker.cpp:76-128) over an explicit grid. Sums start at 0 and add in
 * triangle order; cells without a hit keep (1, 1, 1), metallic 0, roughness 1. color_out holds 3
 * floats per cell. Returns 0, -1 on OOM. */
int32_t orc_materials_dense(const float *soup, int64_t ntris, const float *origin, float voxel, int32_t nx,
                            int32_t ny, int32_t nz, const orc_materials *m, float *color_out, float *metal_out,
                            float *rough_out) {
  const int64_t cells = (int64_t)nx * ny * nz;
  float *sum = (float *)calloc((size_t)cells * 5, sizeof(float));
  int32_t *cnt = (int32_t *)calloc((size_t)cells, sizeof(int32_t));
  if (!sum || !cnt) { free(sum); free(cnt); return -1; }
  const int nmax[3] = {nx - 1, ny - 1, nz - 1};
  const float half = voxel * 0.5f;
  const f3 h = {half, half, half};
  for (int64_t t = 0; t < ntris; ++t) {
    const f3 p0 = vtx(soup, NULL, t, 0), p1 = vtx(soup, NULL, t, 1), p2 = vtx(soup, NULL, t, 2);
    int lo[3], hi[3];
    tri_cell_range(p0, p1, p2, origin, voxel, nmax, lo, hi);
    float mat[5];
    orc_triangle_material(m, t, mat);
    for (int z = lo[2]; z <= hi[2]; ++z)
      for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) {
          const f3 c = {cell_center(origin[0], x, voxel), cell_center(origin[1], y, voxel),
                        cell_center(origin[2], z, voxel)};
          if (!sat_overlap(c, h, p0, p1, p2)) continue;
          const int64_t i = ((int64_t)z * ny + y) * nx + x;
          for (int k = 0; k < 5; ++k) sum[5 * i + k] += mat[k];
          cnt[i] += 1;
        }
  }
  for (int64_t i = 0; i < cells; ++i) {
    if (cnt[i] == 0) {
      color_out[3 * i] = color_out[3 * i + 1] = color_out[3 * i + 2] = 1.0f;
      metal_out[i] = 0.0f;
      rough_out[i] = 1.0f;
      continue;
    }
    const float n = (float)cnt[i];
    for (int k = 0; k < 3; ++k) color_out[3 * i + k] = sum[5 * i + k] / n;
    metal_out[i] = sum[5 * i + 3] / n;
    rough_out[i] = sum[5 * i + 4] / n;
  }
  free(sum);
  free(cnt);
  return 0;
}

/* voxelizeMesh (voxelize.cpp:52-107): origin = boundsMin (no pad), voxel = longest / res, every
 * axis clamped to res - 1, cells listed in first-insertion order. Returns the cell count (cells
 * beyond cap are counted, not written), -1 on OOM. */
static int64_t voxelize_sparse(const float *soup, int64_t ntris, const float *bmin, const float *bmax, int32_t res,
                               const orc_materials *mats, int32_t *cells_out, float *colors_out, int64_t cap,
                               float *origin_out, float *voxel_out);

int64_t orc_voxelize_sparse(const float *soup, int64_t ntris, const float *bmin, const float *bmax, int32_t res,
                            int32_t *cells_out, int64_t cap, float *origin_out, float *voxel_out) {
  return voxelize_sparse(soup, ntris, bmin, bmax, res, NULL, cells_out, NULL, cap, origin_out, voxel_out);
}

/* voxelizeMesh with its colours (voxelize.cpp:78-104): a cell's sum starts at the colour of the
 * first triangle that inserts it and adds later ones in triangle order; colour = sum / count.
 * colors_out holds 3 floats per written cell. */
int64_t orc_voxelize_colors(const float *soup, int64_t ntris, const float *bmin, const float *bmax, int32_t res,
                            const orc_materials *mats, int32_t *cells_out, float *colors_out, int64_t cap,
                            float *origin_out, float *voxel_out) {
  return voxelize_sparse(soup, ntris, bmin, bmax, res, mats, cells_out, colors_out, cap, origin_out, voxel_out);
}

static int64_t voxelize_sparse(const float *soup, int64_t ntris, const float *bmin, const float *bmax, int32_t res,
                               const orc_materials *mats, int32_t *cells_out, float *colors_out, int64_t cap,
                               float *origin_out, float *voxel_out) {
  const float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  float longest = ex;
  if (longest < ey) longest = ey;
  if (longest < ez) longest = ez;
  if (longest < 1e-6f) longest = 1e-6f;
  const float voxel = longest / (float)(res > 1 ? res : 1);
  const float origin[3] = {bmin[0], bmin[1], bmin[2]};
  const int nmax[3] = {res - 1, res - 1, res - 1};
  const float half = voxel * 0.5f;
  const f3 h = {half, half, half};
  hmap m;
  if (hmap_init(&m, ntris * 4 + 16, 3)) return -1;
  const int with_colors = mats && colors_out;
  float *csum = NULL;
  int32_t *ccnt = NULL;
  if (with_colors && cap > 0) {
    csum = (float *)malloc((size_t)cap * 3 * sizeof(float));
    ccnt = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    if (!csum || !ccnt) { free(csum); free(ccnt); hmap_free(&m); return -1; }
  }
  int64_t count = 0;
  for (int64_t t = 0; t < ntris; ++t) {
    const f3 p0 = vtx(soup, NULL, t, 0), p1 = vtx(soup, NULL, t, 1), p2 = vtx(soup, NULL, t, 2);
    int lo[3], hi[3];
    tri_cell_range(p0, p1, p2, origin, voxel, nmax, lo, hi);
    float mat[5] = {0, 0, 0, 0, 0};
    if (with_colors) orc_triangle_material(mats, t, mat);
    for (int z = lo[2]; z <= hi[2]; ++z)
      for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) {
          const f3 c = {cell_center(origin[0], x, voxel), cell_center(origin[1], y, voxel),
                        cell_center(origin[2], z, voxel)};
          if (!sat_overlap(c, h, p0, p1, p2)) continue;
          if (m.size * 2 >= m.cap) { /* grow */
            hmap bigger;
            if (hmap_init(&bigger, m.cap, 3)) { hmap_free(&m); return -1; }
            for (int64_t s = 0; s < m.cap; ++s)
              if (m.used[s]) {
                int ins2;
                const int64_t s2 = hmap_get_or_insert(&bigger, m.keys + 3 * s, m.vals[s], &ins2);
                (void)s2;
              }
            hmap_free(&m);
            m = bigger;
          }
          const int64_t key[3] = {x, y, z};
          int ins;
          const int64_t slot = hmap_get_or_insert(&m, key, count, &ins);
          const int64_t ci = ins ? count : m.vals[slot];
          if (ins) {
            if (count < cap) {
              cells_out[3 * count] = x; cells_out[3 * count + 1] = y; cells_out[3 * count + 2] = z;
              if (csum) {
                csum[3 * count] = mat[0]; csum[3 * count + 1] = mat[1]; csum[3 * count + 2] = mat[2];
                ccnt[count] = 1;
              }
            }
            count++;
          } else if (csum && ci < cap) {
            csum[3 * ci] += mat[0]; csum[3 * ci + 1] += mat[1]; csum[3 * ci + 2] += mat[2];
            ccnt[ci] += 1;
          }
        }
  }
  hmap_free(&m);
  if (csum) {
    const int64_t n = count < cap ? count : cap;
    for (int64_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) colors_out[3 * i + k] = csum[3 * i + k] / (float)ccnt[i];
    free(csum);
    free(ccnt);
  }
  origin_out[0] = origin[0]; origin_out[1] = origin[1]; origin_out[2] = origin[2];
  *voxel_out = voxel;
  return count;
}

/* ------------------------------------------------------------------------------------------ */
/* Consumer check: the renderer's trilinear sample and SDF ray march (pathtracer.cu).          */

typedef struct {
  const float *dist;
  float o[3], v;
  int n[3];
} sdf_view;

static inline float sdf_at(const sdf_view *g, int x, int y, int z) {
  return g->dist[((int64_t)z * g->n[1] + y) * g->n[0] + x];
}

static inline float lerp_ref(float a, float b, float f) { return a * (1.0f - f) + b * f; }

static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* sampleSdf (pathtracer.cu:684-702) */
static float sample_sdf(const sdf_view *g, const float p[3]) {
  float l[3], f[3];
  int c0[3];
  for (int a = 0; a < 3; ++a) {
    l[a] = (p[a] - g->o[a]) / g->v - 0.5f;
    c0[a] = imax(0, imin(g->n[a] - 2, f2i_sat(floorf(l[a]))));
    f[a] = fminf(fmaxf(l[a] - (float)c0[a], 0.0f), 1.0f);
  }
  const int x0 = c0[0], y0 = c0[1], z0 = c0[2];
  const float c00 = lerp_ref(sdf_at(g, x0, y0, z0), sdf_at(g, x0 + 1, y0, z0), f[0]);
  const float c10 = lerp_ref(sdf_at(g, x0, y0 + 1, z0), sdf_at(g, x0 + 1, y0 + 1, z0), f[0]);
  const float c01 = lerp_ref(sdf_at(g, x0, y0, z0 + 1), sdf_at(g, x0 + 1, y0, z0 + 1), f[0]);
  const float c11 = lerp_ref(sdf_at(g, x0, y0 + 1, z0 + 1), sdf_at(g, x0 + 1, y0 + 1, z0 + 1), f[0]);
  const float cc0 = lerp_ref(c00, c10, f[1]);
  const float cc1 = lerp_ref(c01, c11, f[1]);
  return lerp_ref(cc0, cc1, f[2]);
}

static float sample_ray(const sdf_view *g, const float *o, const float *d, float t) {
  const float p[3] = {o[0] + t * d[0], o[1] + t * d[1], o[2] + t * d[2]};
  return sample_sdf(g, p);
}

/* slabTest (pathtracer.cu:587-613) */
static int slab_test(const float *o, const float *d, const float *lo, const float *hi, float *t0, float *t1) {
  for (int a = 0; a < 3; ++a) {
    const float inv = 1.0f / d[a];
    float tn = (lo[a] - o[a]) * inv, tf = (hi[a] - o[a]) * inv;
    if (tn > tf) { const float x = tn; tn = tf; tf = x; }
    if (tn > *t0) *t0 = tn;
    if (tf < *t1) *t1 = tf;
    if (*t0 > *t1) return 0;
  }
  return 1;
}

/* __intersection__sdf (pathtracer.cu:740-787): reported hit distance, or -1. */
static float trace_sdf(const sdf_view *g, const float *o, const float *d, float tmin, float tmax) {
  const float lo[3] = {g->o[0], g->o[1], g->o[2]};
  const float hi[3] = {g->o[0] + (float)g->n[0] * g->v, g->o[1] + (float)g->n[1] * g->v,
                       g->o[2] + (float)g->n[2] * g->v};
  float t0 = tmin, t1 = tmax;
  if (!slab_test(o, d, lo, hi, &t0, &t1)) return -1.0f;
  const float eps = g->v * 0.02f, min_step = g->v * 0.05f, min_adv = g->v * 0.3f;
  float t = t0, prev_t = t0;
  float prev = sample_ray(g, o, d, t0);
  t += fmaxf(fabsf(prev), min_step);
  for (int i = 1; i < 512 && t <= t1; ++i) {
    const float dist = sample_ray(g, o, d, t);
    const int crossed = (prev > 0.0f) != (dist > 0.0f);
    if ((crossed || fabsf(dist) < eps) && (t - t0) > min_adv) {
      float hit = t;
      if (crossed) {
        float a = prev_t, b = t, fa = prev, fb = dist;
        for (int k = 0; k < 8; ++k) {
          const float m = 0.5f * (a + b);
          const float fm = sample_ray(g, o, d, m);
          if ((fa > 0.0f) != (fm > 0.0f)) { b = m; fb = fm; } else { a = m; fa = fm; }
        }
        const float denom = fa - fb;
        hit = fabsf(denom) > 1e-9f ? a + (b - a) * (fa / denom) : 0.5f * (a + b);
      }
      return fmaxf(hit, t0);
    }
    prev_t = t;
    prev = dist;
    t += fmaxf(fabsf(dist) * 0.85f, min_step);
  }
  return -1.0f;
}

void orc_sample_sdf(const float *dist, const float *origin, float voxel, int32_t nx, int32_t ny, int32_t nz,
                    const float *pts, int64_t n, float *out) {
  const sdf_view g = {dist, {origin[0], origin[1], origin[2]}, voxel, {nx, ny, nz}};
  for (int64_t i = 0; i < n; ++i) out[i] = sample_sdf(&g, pts + 3 * i);
}

void orc_trace_sdf(const float *dist, const float *origin, float voxel, int32_t nx, int32_t ny, int32_t nz,
                   const float *rays, int64_t n, float tmin, float tmax, float *t_out) {
  const sdf_view g = {dist, {origin[0], origin[1], origin[2]}, voxel, {nx, ny, nz}};
  for (int64_t i = 0; i < n; ++i) t_out[i] = trace_sdf(&g, rays + 6 * i, rays + 6 * i + 3, tmin, tmax);
}

/* First hit t > 0 of each ray (origin, direction: 6 floats) with the mesh, in FP64 (Moller &
 * Trumbore, "Fast, minimum storage ray/triangle intersection", 1997), or -1. Brute force. */
void orc_ray_mesh(const float *verts, const uint32_t *idx, int64_t ntris, const float *rays, int64_t n,
                  double *t_out) {
  for (int64_t r = 0; r < n; ++r) {
    const double o[3] = {rays[6 * r], rays[6 * r + 1], rays[6 * r + 2]};
    const double d[3] = {rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]};
    double best = -1.0;
    for (int64_t t = 0; t < ntris; ++t) {
      const f3 A = vtx(verts, idx, t, 0), B = vtx(verts, idx, t, 1), Cc = vtx(verts, idx, t, 2);
      const double e1[3] = {(double)B.x - A.x, (double)B.y - A.y, (double)B.z - A.z};
      const double e2[3] = {(double)Cc.x - A.x, (double)Cc.y - A.y, (double)Cc.z - A.z};
      const double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
      const double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
      if (fabs(det) < 1e-300) continue;
      const double inv = 1.0 / det;
      const double s[3] = {o[0] - A.x, o[1] - A.y, o[2] - A.z};
      const double u = (s[0] * p[0] + s[1] * p[1] + s[2] * p[2]) * inv;
      if (u < 0.0 || u > 1.0) continue;
      const double q[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2], s[0] * e1[1] - s[1] * e1[0]};
      const double v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
      if (v < 0.0 || u + v > 1.0) continue;
      const double tt = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
      if (tt > 0.0 && (best < 0.0 || tt < best)) best = tt;
    }
    t_out[r] = best;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Thread pool helper: runs fn(ctx, i) for i in [0, n) over nthreads workers.                   */

typedef void (*work_fn)(void *ctx, int64_t begin, int64_t end);
typedef struct { work_fn fn; void *ctx; int64_t n, chunk; atomic_llong next; } pool_job;

static void *pool_worker(void *arg) {
  pool_job *j = (pool_job *)arg;
  for (;;) {
    const int64_t b = atomic_fetch_add(&j->next, j->chunk);
    if (b >= j->n) break;
    const int64_t e = b + j->chunk < j->n ? b + j->chunk : j->n;
    j->fn(j->ctx, b, e);
  }
  return NULL;
}

static void run_parallel(work_fn fn, void *ctx, int64_t n, int64_t chunk, int nthreads) {
  if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pool_job j;
  j.fn = fn; j.ctx = ctx; j.n = n; j.chunk = chunk < 1 ? 1 : chunk;
  atomic_init(&j.next, 0);
  if (nthreads == 1) { pool_worker(&j); return; }
  pthread_t th[256];
  int started = 0;
  for (int i = 0; i < nthreads; ++i)
    if (pthread_create(&th[i], NULL, pool_worker, &j) == 0) started++;
    else break;
  if (started == 0) pool_worker(&j);
  for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
}

int32_t orc_default_threads(void) { return (int32_t)sysconf(_SC_NPROCESSORS_ONLN); }

/* ------------------------------------------------------------------------------------------ */
/* FP64 nearest-triangle distance through a median-split BVH.                                  */

typedef struct { double a[3], b[3], c[3]; } dtri;
typedef struct { double lo[3], hi[3]; int32_t left, right, first, count; } bnode;
typedef struct { dtri *tris; int32_t *order; bnode *nodes; int64_t nnodes; double *cent; } dbvh;

static void tri_bounds(const dtri *t, double lo[3], double hi[3]) {
  for (int a = 0; a < 3; ++a) {
    lo[a] = fmin(fmin(t->a[a], t->b[a]), t->c[a]);
    hi[a] = fmax(fmax(t->a[a], t->b[a]), t->c[a]);
  }
}

/* Quickselect on order[lo..hi) by centroid coordinate along axis so position k is the median. */
static void select_kth(int32_t *ord, const double *cent, int axis, int64_t lo, int64_t hi, int64_t k) {
  while (hi - lo > 1) {
    const double pivot = cent[3 * (int64_t)ord[(lo + hi) / 2] + axis];
    int64_t i = lo, j = hi - 1;
    while (i <= j) {
      while (cent[3 * (int64_t)ord[i] + axis] < pivot) i++;
      while (cent[3 * (int64_t)ord[j] + axis] > pivot) j--;
      if (i <= j) { const int32_t t = ord[i]; ord[i] = ord[j]; ord[j] = t; i++; j--; }
    }
    if (k <= j) hi = j + 1;
    else if (k >= i) lo = i;
    else return;
  }
}

static int32_t build_node(dbvh *b, int64_t first, int64_t count) {
  const int32_t id = (int32_t)b->nnodes++;
  bnode *n = &b->nodes[id];
  for (int a = 0; a < 3; ++a) { n->lo[a] = INFINITY; n->hi[a] = -INFINITY; }
  double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = first; i < first + count; ++i) {
    double lo[3], hi[3];
    tri_bounds(&b->tris[b->order[i]], lo, hi);
    for (int a = 0; a < 3; ++a) {
      n->lo[a] = fmin(n->lo[a], lo[a]);
      n->hi[a] = fmax(n->hi[a], hi[a]);
      const double c = b->cent[3 * (int64_t)b->order[i] + a];
      clo[a] = fmin(clo[a], c);
      chi[a] = fmax(chi[a], c);
    }
  }
  if (count <= 4) {
    n->left = n->right = -1;
    n->first = (int32_t)first;
    n->count = (int32_t)count;
    return id;
  }
  int axis = 0;
  for (int a = 1; a < 3; ++a)
    if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
  const int64_t half = count / 2;
  select_kth(b->order, b->cent, axis, first, first + count, first + half);
  n->first = (int32_t)first;
  n->count = 0;
  const int32_t l = build_node(b, first, half);
  const int32_t r = build_node(b, first + half, count - half);
  b->nodes[id].left = l;
  b->nodes[id].right = r;
  return id;
}

static int dbvh_build(dbvh *b, const float *verts, const uint32_t *idx, int64_t ntris) {
  b->tris = (dtri *)malloc((size_t)(ntris > 0 ? ntris : 1) * sizeof(dtri));
  b->order = (int32_t *)malloc((size_t)(ntris > 0 ? ntris : 1) * sizeof(int32_t));
  b->cent = (double *)malloc((size_t)(ntris > 0 ? ntris : 1) * 3 * sizeof(double));
  b->nodes = (bnode *)malloc((size_t)(2 * ntris + 1) * sizeof(bnode));
  b->nnodes = 0;
  if (!b->tris || !b->order || !b->cent || !b->nodes) return -1;
  for (int64_t t = 0; t < ntris; ++t) {
    const f3 p[3] = {vtx(verts, idx, t, 0), vtx(verts, idx, t, 1), vtx(verts, idx, t, 2)};
    dtri *d = &b->tris[t];
    d->a[0] = p[0].x; d->a[1] = p[0].y; d->a[2] = p[0].z;
    d->b[0] = p[1].x; d->b[1] = p[1].y; d->b[2] = p[1].z;
    d->c[0] = p[2].x; d->c[1] = p[2].y; d->c[2] = p[2].z;
    for (int a = 0; a < 3; ++a) b->cent[3 * t + a] = (d->a[a] + d->b[a] + d->c[a]) / 3.0;
    b->order[t] = (int32_t)t;
  }
  if (ntris > 0) build_node(b, 0, ntris);
  return 0;
}

static void dbvh_free(dbvh *b) { free(b->tris); free(b->order); free(b->nodes); free(b->cent); }

static inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static double seg_dist2(const double *p, const double *a, const double *b) {
  double ab[3], ap[3];
  for (int i = 0; i < 3; ++i) { ab[i] = b[i] - a[i]; ap[i] = p[i] - a[i]; }
  const double l2 = dot3(ab, ab);
  double t = l2 > 0.0 ? dot3(ap, ab) / l2 : 0.0;
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = ap[i] - t * ab[i];
  return dot3(d, d);
}

/* Squared distance from p to triangle (a, b, c): Ericson's Voronoi-region walk; triangles with
 * no usable face region (zero area) fall back to their three edges. */
static double point_tri_dist2(const double *p, const dtri *t) {
  const double *a = t->a, *b = t->b, *c = t->c;
  double ab[3], ac[3], ap[3], bp[3], cp[3], q[3];
  for (int i = 0; i < 3; ++i) {
    ab[i] = b[i] - a[i]; ac[i] = c[i] - a[i];
    ap[i] = p[i] - a[i]; bp[i] = p[i] - b[i]; cp[i] = p[i] - c[i];
  }
  /* A zero-area triangle (collinear or coincident vertices) is the union of its edges; the region
   * walk below would divide by zero on a zero-length edge. */
  const double nx = ab[1] * ac[2] - ab[2] * ac[1], ny = ab[2] * ac[0] - ab[0] * ac[2], nz = ab[0] * ac[1] - ab[1] * ac[0];
  if (!(nx * nx + ny * ny + nz * nz > 1e-30 * dot3(ab, ab) * dot3(ac, ac))) {
    const double e0 = seg_dist2(p, a, b), e1 = seg_dist2(p, b, c), e2 = seg_dist2(p, c, a);
    return fmin(e0, fmin(e1, e2));
  }
  const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return dot3(ap, ap);
  const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return dot3(bp, bp);
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double s = d1 / (d1 - d3);
    for (int i = 0; i < 3; ++i) q[i] = a[i] + s * ab[i] - p[i];
    return dot3(q, q);
  }
  const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return dot3(cp, cp);
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double s = d2 / (d2 - d6);
    for (int i = 0; i < 3; ++i) q[i] = a[i] + s * ac[i] - p[i];
    return dot3(q, q);
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
    const double s = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    for (int i = 0; i < 3; ++i) q[i] = b[i] + s * (c[i] - b[i]) - p[i];
    return dot3(q, q);
  }
  const double den = va + vb + vc;
  if (!(den > 0.0) || !isfinite(den)) {
    const double e0 = seg_dist2(p, a, b), e1 = seg_dist2(p, b, c), e2 = seg_dist2(p, c, a);
    return fmin(e0, fmin(e1, e2));
  }
  const double v = vb / den, w = vc / den;
  for (int i = 0; i < 3; ++i) q[i] = a[i] + ab[i] * v + ac[i] * w - p[i];
  return dot3(q, q);
}

static inline double box_dist2(const double *p, const bnode *n) {
  double s = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double d = p[a] < n->lo[a] ? n->lo[a] - p[a] : (p[a] > n->hi[a] ? p[a] - n->hi[a] : 0.0);
    s += d * d;
  }
  return s;
}

static double dbvh_nearest(const dbvh *b, const double *p, int64_t *tri_out) {
  double best = INFINITY;
  int64_t best_t = -1;
  int32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const bnode *n = &b->nodes[stack[--sp]];
    if (box_dist2(p, n) >= best) continue;
    if (n->left < 0) {
      for (int32_t i = n->first; i < n->first + n->count; ++i) {
        const double d = point_tri_dist2(p, &b->tris[b->order[i]]);
        if (d < best) { best = d; best_t = b->order[i]; }
      }
      continue;
    }
    const bnode *l = &b->nodes[n->left], *r = &b->nodes[n->right];
    const double dl = box_dist2(p, l), dr = box_dist2(p, r);
    if (sp + 2 > 128) continue; /* cannot happen for a median-split tree of < 2^60 triangles */
    if (dl < dr) { stack[sp++] = n->right; stack[sp++] = n->left; }
    else { stack[sp++] = n->left; stack[sp++] = n->right; }
  }
  if (tri_out) *tri_out = best_t;
  return sqrt(best);
}

typedef struct {
  const dbvh *b;
  const float *origin;
  float voxel;
  int32_t nx, ny, nz;
  const int64_t *samples; /* NULL = every cell */
  double *out;
  int64_t *tri_out;
} dist_job;

static void dist_work(void *vctx, int64_t begin, int64_t end) {
  dist_job *j = (dist_job *)vctx;
  for (int64_t s = begin; s < end; ++s) {
    const int64_t cell = j->samples ? j->samples[s] : s;
    const int64_t x = cell % j->nx, y = (cell / j->nx) % j->ny, z = cell / ((int64_t)j->nx * j->ny);
    const double p[3] = {(double)cell_center(j->origin[0], (int)x, j->voxel),
                         (double)cell_center(j->origin[1], (int)y, j->voxel),
                         (double)cell_center(j->origin[2], (int)z, j->voxel)};
    int64_t t = -1;
    j->out[s] = j->b->nnodes ? dbvh_nearest(j->b, p, &t) : INFINITY;
    if (j->tri_out) j->tri_out[s] = t;
  }
}

/* Unsigned FP64 distance at FP32 cell centres; samples == NULL means every cell in x-fastest
 * order (n_samples ignored). tri_out (optional) receives the nearest triangle. */
int32_t orc_distance(const float *verts, const uint32_t *idx, int64_t ntris, const float *origin, float voxel,
                     int32_t nx, int32_t ny, int32_t nz, const int64_t *samples, int64_t n_samples, double *out,
                     int64_t *tri_out, int32_t nthreads) {
  dbvh b;
  if (dbvh_build(&b, verts, idx, ntris)) { dbvh_free(&b); return -1; }
  dist_job j = {&b, origin, voxel, nx, ny, nz, samples, out, tri_out};
  const int64_t n = samples ? n_samples : (int64_t)nx * ny * nz;
  run_parallel(dist_work, &j, n, 256, nthreads);
  dbvh_free(&b);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Exact 2-D orientation of float points with simulation of simplicity.                        */

static inline void two_sum(double a, double b, double *s, double *e) {
  const double x = a + b;
  const double bv = x - a;
  const double av = x - bv;
  *s = x;
  *e = (a - av) + (b - bv);
}

/* Exact sign of sum(t[0..n)), n <= 8, each t exactly representable. Grow-Expansion keeps a
 * non-overlapping expansion ordered by magnitude; its top non-zero component has the sum's sign. */
static int exact_sum_sign(const double *t, int n) {
  double e[9];
  int m = 1;
  e[0] = t[0];
  for (int k = 1; k < n; ++k) {
    double q = t[k];
    for (int i = 0; i < m; ++i) {
      double s, err;
      two_sum(q, e[i], &s, &err);
      e[i] = err;
      q = s;
    }
    e[m++] = q;
  }
  for (int i = m - 1; i >= 0; --i)
    if (e[i] != 0.0) return e[i] > 0.0 ? 1 : -1;
  return 0;
}

/* sign of (b - a) x (p - a) in the (u, v) plane, all inputs FP32 values. Expanded into six
 * products of inputs, each exact in FP64, whose sum's sign is found exactly. When the exact value
 * is zero the query point is taken as p + (eps, eps^2): the sign is then that of (a_v - b_v), or
 * failing that (b_u - a_u); both are zero only for a == b, a degenerate edge (returns 0). */
static int orient2_sos(float au, float av, float bu, float bv, float pu, float pv) {
  const double t[6] = {(double)bu * pv, -(double)bu * av, -(double)au * pv,
                       -(double)bv * pu, (double)bv * au, (double)av * pu};
  const int s = exact_sum_sign(t, 6);
  if (s) return s;
  if (av != bv) return av > bv ? 1 : -1;
  if (bu != au) return bu > au ? 1 : -1;
  return 0;
}

/* Approximate (b - a) x (p - a) for barycentric weights only. */
static inline double orient2_approx(double au, double av, double bu, double bv, double pu, double pv) {
  return (bu - au) * (pv - av) - (bv - av) * (pu - au);
}

/* Does the line through (pu, pv) along axis ax cross the triangle? If so *t receives the crossing
 * coordinate along ax. Degenerate projections never cross. */
static int column_crossing(const float *a, const float *b, const float *c, int ax, float pu, float pv,
                           double *t) {
  const int u = (ax + 1) % 3, v = (ax + 2) % 3;
  const int s0 = orient2_sos(a[u], a[v], b[u], b[v], pu, pv);
  if (s0 == 0) return 0;
  const int s1 = orient2_sos(b[u], b[v], c[u], c[v], pu, pv);
  if (s1 != s0) return 0;
  const int s2 = orient2_sos(c[u], c[v], a[u], a[v], pu, pv);
  if (s2 != s0) return 0;
  const double wa = fabs(orient2_approx(b[u], b[v], c[u], c[v], pu, pv));
  const double wb = fabs(orient2_approx(c[u], c[v], a[u], a[v], pu, pv));
  const double wc = fabs(orient2_approx(a[u], a[v], b[u], b[v], pu, pv));
  const double den = wa + wb + wc;
  if (den > 0.0) *t = (wa * a[ax] + wb * b[ax] + wc * c[ax]) / den;
  else *t = ((double)a[ax] + b[ax] + c[ax]) / 3.0;
  return 1;
}

int32_t orc_column_crossing(const float *a, const float *b, const float *c, int32_t ax, float pu, float pv,
                            double *t) {
  return column_crossing(a, b, c, ax, pu, pv, t);
}
int32_t orc_orient2_sos(float au, float av, float bu, float bv, float pu, float pv) {
  return orient2_sos(au, av, bu, bv, pu, pv);
}

/* Parity sign along axis ax for every cell: columns are binned by triangle projections; each
 * cell's sign is -1 when an odd number of crossings lie strictly beyond it along +ax. */
typedef struct {
  const float *verts;
  const uint32_t *idx;
  const float *origin;
  float voxel;
  int32_t n[3];
  int ax;
  int64_t *bin_start; /* CSR over columns */
  int32_t *bin_tris;
  int8_t *sign_out;
} parity_job;

static int cmp_double(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

static void parity_work(void *vctx, int64_t begin, int64_t end) {
  parity_job *j = (parity_job *)vctx;
  const int ax = j->ax, u = (ax + 1) % 3, v = (ax + 2) % 3;
  const int64_t nu = j->n[u];
  double *cross = NULL;
  int64_t cap = 0;
  for (int64_t col = begin; col < end; ++col) {
    const int iu = (int)(col % nu), iv = (int)(col / nu);
    const float pu = cell_center(j->origin[u], iu, j->voxel), pv = cell_center(j->origin[v], iv, j->voxel);
    const int64_t b0 = j->bin_start[col], b1 = j->bin_start[col + 1];
    if (b1 - b0 > cap) {
      cap = b1 - b0;
      free(cross);
      cross = (double *)malloc((size_t)cap * sizeof(double));
    }
    int64_t nc = 0;
    for (int64_t k = b0; k < b1; ++k) {
      const int64_t t = j->bin_tris[k];
      float P[3][3];
      for (int q = 0; q < 3; ++q) {
        const f3 w = vtx(j->verts, j->idx, t, q);
        P[q][0] = w.x; P[q][1] = w.y; P[q][2] = w.z;
      }
      double tc;
      if (column_crossing(P[0], P[1], P[2], ax, pu, pv, &tc)) cross[nc++] = tc;
    }
    if (nc > 1) qsort(cross, (size_t)nc, sizeof(double), cmp_double);
    /* Walk the column from the far end: parity of crossings beyond each cell. */
    int64_t k = nc;
    int parity = 0;
    for (int ia = j->n[ax] - 1; ia >= 0; --ia) {
      const double c = (double)cell_center(j->origin[ax], ia, j->voxel);
      while (k > 0 && cross[k - 1] > c) { k--; parity ^= 1; }
      int64_t cell3[3];
      cell3[ax] = ia; cell3[u] = iu; cell3[v] = iv;
      const int64_t lin = (cell3[2] * j->n[1] + cell3[1]) * j->n[0] + cell3[0];
      j->sign_out[lin] = parity ? -1 : 1;
    }
  }
  free(cross);
}

int32_t orc_sign_parity(const float *verts, const uint32_t *idx, int64_t ntris, const float *origin, float voxel,
                        int32_t nx, int32_t ny, int32_t nz, int32_t ax, int8_t *sign_out, int32_t nthreads) {
  const int u = (ax + 1) % 3, v = (ax + 2) % 3;
  const int32_t n[3] = {nx, ny, nz};
  const int64_t nu = n[u], nv = n[v], ncol = nu * nv;
  int64_t *count = (int64_t *)calloc((size_t)ncol + 1, sizeof(int64_t));
  if (!count) return -1;
  /* Candidate columns of a triangle: centres within its projected bounds, widened by one. */
  for (int pass = 0; pass < 2; ++pass) {
    int32_t *bins = NULL;
    int64_t *fill = NULL;
    if (pass == 1) {
      for (int64_t c = 0; c < ncol; ++c) count[c + 1] += count[c];
      bins = (int32_t *)malloc((size_t)(count[ncol] > 0 ? count[ncol] : 1) * sizeof(int32_t));
      fill = (int64_t *)malloc((size_t)(ncol > 0 ? ncol : 1) * sizeof(int64_t));
      if (!bins || !fill) { free(bins); free(fill); free(count); return -1; }
      memcpy(fill, count, (size_t)ncol * sizeof(int64_t));
    } else {
      memset(count, 0, (size_t)(ncol + 1) * sizeof(int64_t));
    }
    for (int64_t t = 0; t < ntris; ++t) {
      const f3 p[3] = {vtx(verts, idx, t, 0), vtx(verts, idx, t, 1), vtx(verts, idx, t, 2)};
      double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
      for (int q = 0; q < 3; ++q) {
        const double cu = f3_get(p[q], u), cv = f3_get(p[q], v);
        lo[0] = fmin(lo[0], cu); hi[0] = fmax(hi[0], cu);
        lo[1] = fmin(lo[1], cv); hi[1] = fmax(hi[1], cv);
      }
      const int axes[2] = {u, v};
      int64_t r0[2], r1[2];
      for (int q = 0; q < 2; ++q) {
        const double o = origin[axes[q]];
        r0[q] = (int64_t)floor((lo[q] - o) / voxel - 0.5) - 1;
        r1[q] = (int64_t)ceil((hi[q] - o) / voxel - 0.5) + 1;
        if (r0[q] < 0) r0[q] = 0;
        if (r1[q] > n[axes[q]] - 1) r1[q] = n[axes[q]] - 1;
      }
      for (int64_t iv = r0[1]; iv <= r1[1]; ++iv)
        for (int64_t iu = r0[0]; iu <= r1[0]; ++iu) {
          const int64_t col = iv * nu + iu;
          if (pass == 0) count[col + 1]++;
          else bins[fill[col]++] = (int32_t)t;
        }
    }
    if (pass == 1) {
      parity_job j = {verts, idx, origin, voxel, {nx, ny, nz}, ax, count, bins, sign_out};
      run_parallel(parity_work, &j, ncol, 64, nthreads);
      free(bins);
      free(fill);
    }
  }
  free(count);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* FP64 generalized winding number, summed directly over all triangles.                       */

static double solid_angle(const double *p, const float *A, const float *B, const float *C) {
  double a[3], b[3], c[3];
  for (int i = 0; i < 3; ++i) { a[i] = (double)A[i] - p[i]; b[i] = (double)B[i] - p[i]; c[i] = (double)C[i] - p[i]; }
  const double la = sqrt(dot3(a, a)), lb = sqrt(dot3(b, b)), lc = sqrt(dot3(c, c));
  const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                     a[2] * (b[0] * c[1] - b[1] * c[0]);
  const double den = la * lb * lc + dot3(a, b) * lc + dot3(b, c) * la + dot3(c, a) * lb;
  return 2.0 * atan2(det, den);
}

typedef struct {
  const float *verts;
  const uint32_t *idx;
  int64_t ntris;
  const float *origin;
  float voxel;
  int32_t nx, ny, nz;
  const int64_t *samples;
  double *out;
} gwn_job;

static void gwn_work(void *vctx, int64_t begin, int64_t end) {
  gwn_job *j = (gwn_job *)vctx;
  for (int64_t s = begin; s < end; ++s) {
    const int64_t cell = j->samples ? j->samples[s] : s;
    const int64_t x = cell % j->nx, y = (cell / j->nx) % j->ny, z = cell / ((int64_t)j->nx * j->ny);
    const double p[3] = {(double)cell_center(j->origin[0], (int)x, j->voxel),
                         (double)cell_center(j->origin[1], (int)y, j->voxel),
                         (double)cell_center(j->origin[2], (int)z, j->voxel)};
    double w = 0.0;
    for (int64_t t = 0; t < j->ntris; ++t) {
      const uint32_t i0 = j->idx ? j->idx[3 * t] : (uint32_t)(3 * t);
      const uint32_t i1 = j->idx ? j->idx[3 * t + 1] : (uint32_t)(3 * t + 1);
      const uint32_t i2 = j->idx ? j->idx[3 * t + 2] : (uint32_t)(3 * t + 2);
      w += solid_angle(p, j->verts + 3 * (int64_t)i0, j->verts + 3 * (int64_t)i1, j->verts + 3 * (int64_t)i2);
    }
    j->out[s] = w / (4.0 * 3.14159265358979323846);
  }
}

int32_t orc_gwn(const float *verts, const uint32_t *idx, int64_t ntris, const float *origin, float voxel, int32_t nx,
                int32_t ny, int32_t nz, const int64_t *samples, int64_t n_samples, double *out, int32_t nthreads) {
  gwn_job j = {verts, idx, ntris, origin, voxel, nx, ny, nz, samples, out};
  const int64_t n = samples ? n_samples : (int64_t)nx * ny * nz;
  run_parallel(gwn_work, &j, n, 16, nthreads);
  return 0;
}
