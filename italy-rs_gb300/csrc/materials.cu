// Per-cell materials: the material averaging of bakePerCellMaterial
// (src/convert/sdf_baker.cpp:76-128) and the colours of voxelizeMesh
// (src/convert/voxelize.cpp:78-104), on the device.
//
// 1. k_tri_material: one thread per triangle computes the triangle's material -- base colour
//    factor, modulated by the nearest texel at the wrapped mean of its uvs (sdf_baker.cpp:42-74,
//    voxelize.cpp:12-37) -- with one IEEE operation per reference operation. sRGB decoding reads a
//    256-entry table built on the host by the reference's own formula (the channel is an 8-bit
//    value divided by 255, so the table is exact).
// 2. occupancy_hits (occupancy.cu): every (cell, triangle) pair that passes the occupancy rule, as
//    one 64-bit key (cell << tri_bits | triangle).
// 3. A stable radix sort of the keys orders each cell's triangles by index -- the order in which
//    the reference's triangle loop adds them -- so the sums below round exactly as the reference's.
// 4. k_mat_dense: one thread per cell segment sums the segment in order and writes the means;
//    cells without a triangle keep (1, 1, 1), 0, 1. k_mat_sparse: one thread per sparse output
//    cell finds its segment by binary search; voxelizeMesh's sum starts at the first triangle's
//    colour rather than at 0.
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "host_mesh.h"
#include "kernels.h"

using namespace sdfb;

namespace {

constexpr int kThreads = 256;

struct TexRec {
  uint64_t offset;
  int32_t w, h, srgb, pad;
};

struct MatRec {
  float f[5];  // base colour r, g, b, metallic, roughness
  int32_t tex;
};

struct MatArgs {
  const MatRec *mats;
  uint32_t nmat;
  const uint32_t *tri_mat;
  uint64_t ntri_mat;
  const float *uvs;
  uint64_t nuv;
  const TexRec *tex;
  uint32_t ntex;
  const uint8_t *pixels;
  const float *srgb_lut;
};

// triangleMaterial (sdf_baker.cpp:61-74): cm = (r, g, b, metallic), rough = roughness.
__global__ __launch_bounds__(kThreads) void k_tri_material(MatArgs a, uint32_t T, float4 *__restrict__ cm,
                                                           float *__restrict__ rough) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= T) return;
  const uint64_t mi0 = t < a.ntri_mat ? uint64_t(__ldg(a.tri_mat + t)) : 0;
  const MatRec m = a.mats[mi0 < a.nmat ? mi0 : 0];
  float r = m.f[0], g = m.f[1], b = m.f[2];
  const uint64_t base = uint64_t(t) * 3;
  if (m.tex >= 0 && uint32_t(m.tex) < a.ntex && base + 2 < a.nuv) {
    const TexRec tx = a.tex[m.tex];
    if (tx.w > 0 && tx.h > 0) {
      const float *u = a.uvs + 2 * base;
      const float uu = __fdiv_rn(__fadd_rn(__fadd_rn(u[0], u[2]), u[4]), 3.0f);
      const float vv = __fdiv_rn(__fadd_rn(__fadd_rn(u[1], u[3]), u[5]), 3.0f);
      const float wu = __fsub_rn(uu, floorf(uu)), wv = __fsub_rn(vv, floorf(vv));
      const int px = clampi(f2i_sat(__fmul_rn(wu, static_cast<float>(tx.w))), 0, tx.w - 1);
      const int py = clampi(f2i_sat(__fmul_rn(wv, static_cast<float>(tx.h))), 0, tx.h - 1);
      const uint8_t *p = a.pixels + tx.offset + (uint64_t(py) * tx.w + px) * 4;
      float cr, cg, cb;
      if (tx.srgb) {
        cr = a.srgb_lut[p[0]];
        cg = a.srgb_lut[p[1]];
        cb = a.srgb_lut[p[2]];
      } else {
        cr = __fdiv_rn(static_cast<float>(p[0]), 255.0f);
        cg = __fdiv_rn(static_cast<float>(p[1]), 255.0f);
        cb = __fdiv_rn(static_cast<float>(p[2]), 255.0f);
      }
      r = __fmul_rn(cr, m.f[0]);
      g = __fmul_rn(cg, m.f[1]);
      b = __fmul_rn(cb, m.f[2]);
    }
  }
  cm[t] = make_float4(r, g, b, m.f[3]);
  rough[t] = m.f[4];
}

__global__ __launch_bounds__(kThreads) void k_mat_defaults(uint64_t cells, float *__restrict__ color,
                                                           float *__restrict__ metal, float *__restrict__ rough) {
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < cells; i += uint64_t(gridDim.x) * kThreads) {
    color[3 * i] = color[3 * i + 1] = color[3 * i + 2] = 1.0f;
    metal[i] = 0.0f;
    rough[i] = 1.0f;
  }
}

// One thread per segment of equal cells in the sorted keys: the triangles' materials added in
// triangle order starting from 0 (sdf_baker.cpp:110-114), then divided by the count (:121-127).
__global__ __launch_bounds__(kThreads) void k_mat_dense(const uint64_t *__restrict__ keys, uint64_t n, int tri_bits,
                                                        const float4 *__restrict__ cm,
                                                        const float *__restrict__ trough, float *__restrict__ color,
                                                        float *__restrict__ metal, float *__restrict__ rough) {
  const uint64_t mask = (uint64_t(1) << tri_bits) - 1;
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads) {
    const uint64_t cell = keys[i] >> tri_bits;
    if (i > 0 && (keys[i - 1] >> tri_bits) == cell) continue;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, sm = 0.0f, so = 0.0f;
    uint64_t j = i;
    for (; j < n && (keys[j] >> tri_bits) == cell; ++j) {
      const uint32_t t = static_cast<uint32_t>(keys[j] & mask);
      const float4 c = cm[t];
      sr = __fadd_rn(sr, c.x);
      sg = __fadd_rn(sg, c.y);
      sb = __fadd_rn(sb, c.z);
      sm = __fadd_rn(sm, c.w);
      so = __fadd_rn(so, trough[t]);
    }
    const float cnt = static_cast<float>(static_cast<int>(j - i));
    color[3 * cell] = __fdiv_rn(sr, cnt);
    color[3 * cell + 1] = __fdiv_rn(sg, cnt);
    color[3 * cell + 2] = __fdiv_rn(sb, cnt);
    metal[cell] = __fdiv_rn(sm, cnt);
    rough[cell] = __fdiv_rn(so, cnt);
  }
}

// One thread per sparse output cell: its segment found by binary search in the sorted keys; the
// first triangle's colour starts the sum (voxelize.cpp:87-95), the rest add in order (:96-99).
__global__ __launch_bounds__(kThreads) void k_mat_sparse(const uint32_t *__restrict__ cells_list, uint64_t n_out,
                                                         const uint64_t *__restrict__ keys, uint64_t n, int tri_bits,
                                                         const float4 *__restrict__ cm, float *__restrict__ colors) {
  const uint64_t mask = (uint64_t(1) << tri_bits) - 1;
  for (uint64_t o = uint64_t(blockIdx.x) * kThreads + threadIdx.x; o < n_out; o += uint64_t(gridDim.x) * kThreads) {
    const uint64_t cell = cells_list[o];
    const uint64_t want = cell << tri_bits;
    uint64_t lo = 0, hi = n;  // first key >= want
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < want) lo = mid + 1;
      else hi = mid;
    }
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    uint64_t j = lo;
    for (; j < n && (keys[j] >> tri_bits) == cell; ++j) {
      const float4 c = cm[static_cast<uint32_t>(keys[j] & mask)];
      if (j == lo) {
        sr = c.x;
        sg = c.y;
        sb = c.z;
      } else {
        sr = __fadd_rn(sr, c.x);
        sg = __fadd_rn(sg, c.y);
        sb = __fadd_rn(sb, c.z);
      }
    }
    const float cnt = static_cast<float>(static_cast<int>(j - lo));
    colors[3 * o] = __fdiv_rn(sr, cnt);
    colors[3 * o + 1] = __fdiv_rn(sg, cnt);
    colors[3 * o + 2] = __fdiv_rn(sb, cnt);
  }
}

#define CK(call)                                            \
  do {                                                      \
    const cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call); \
  } while (0)

#define ENSURE(buf, bytes)                                                                       \
  do {                                                                                           \
    if (!(buf).ensure(bytes))                                                                    \
      return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of device memory", \
                      static_cast<size_t>(bytes));                                               \
  } while (0)

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int bits_for(uint64_t n) {
  int b = 1;
  while (b < 63 && (uint64_t(1) << b) < n) ++b;
  return b;
}

sdfb_status check_materials(sdfb_ctx *ctx, const sdfb_materials *m) {
  if (!m || m->struct_size < sizeof(sdfb_materials))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: null or struct_size too small");
  if (m->num_materials == 0 || !m->materials)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: at least one material is required");
  if (m->num_triangle_material && !m->triangle_material)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: triangle_material is NULL");
  if (m->num_uvs && !m->uvs) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: uvs is NULL");
  if (m->num_textures && !m->textures) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: textures is NULL");
  for (uint32_t k = 0; k < m->num_textures; ++k) {
    const sdfb_texture &t = m->textures[k];
    if (t.width < 0 || t.height < 0 || (t.width > 0 && t.height > 0 && !t.rgba))
      return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "materials: texture %u has a bad size or no texels", k);
  }
  return SDFB_OK;
}

// Uploads the soup (with identity indices) and a one-mesh batch record whose occupancy output is
// ctx->out_occ, over grid g.
sdfb_status soup_batch(sdfb_ctx *ctx, const float *positions, uint32_t T, const sdfb_grid_desc &g, cudaStream_t st,
                       BatchDev &B) {
  const uint64_t V = uint64_t(3) * T;
  const uint64_t cells = uint64_t(g.nx) * g.ny * g.nz;
  std::vector<uint32_t> ident(V);
  for (uint64_t i = 0; i < V; ++i) ident[i] = static_cast<uint32_t>(i);
  ENSURE(ctx->in_verts, V * 12);
  ENSURE(ctx->in_idx, V * 4);
  ENSURE(ctx->out_occ, cells);
  CK(cudaMemcpyAsync(ctx->in_verts.p, positions, V * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, ident.data(), V * 4, cudaMemcpyHostToDevice, st));
  MeshRec r;
  std::memset(&r, 0, sizeof r);
  r.verts = static_cast<const float *>(ctx->in_verts.p);
  r.idx = static_cast<const uint32_t *>(ctx->in_idx.p);
  r.num_verts = static_cast<uint32_t>(V);
  r.num_tris = T;
  r.occ = static_cast<uint8_t *>(ctx->out_occ.p);
  r.g = to_dev(g);
  r.leaf_size = 1;
  const uint64_t tables[2][2] = {{0, T}, {0, cells}};
  const uint64_t zero[2] = {0, 0};
  static_assert(sizeof(MeshRec) <= 256, "the mesh record fits its slot");
  const size_t bytes = 256 * 4;
  ENSURE(ctx->mat_rec, bytes + 64);  // + the hit counter at byte 1024
  std::vector<char> hs(bytes, 0);
  std::memcpy(hs.data(), &r, sizeof r);
  std::memcpy(hs.data() + 256, tables[0], 16);
  std::memcpy(hs.data() + 512, tables[1], 16);
  std::memcpy(hs.data() + 768, zero, 16);
  CK(cudaMemcpyAsync(ctx->mat_rec.p, hs.data(), bytes, cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));  // hs and ident are host locals
  char *d = static_cast<char *>(ctx->mat_rec.p);
  B = BatchDev();
  B.num_meshes = 1;
  B.recs = reinterpret_cast<const MeshRec *>(d);
  B.tri_starts = reinterpret_cast<const uint64_t *>(d + 256);
  B.cell_starts = reinterpret_cast<const uint64_t *>(d + 512);
  B.ptri_starts = B.tile_starts = B.gwn_tile_starts = reinterpret_cast<const uint64_t *>(d + 768);
  B.total_tris = T;
  B.total_cells = cells;
  return SDFB_OK;
}

// Per-triangle materials into ctx->mat_tri: T float4 (r, g, b, metallic) then T roughness floats.
sdfb_status triangle_materials(sdfb_ctx *ctx, const sdfb_materials &m, uint32_t T, cudaStream_t st) {
  // One device block: materials | textures | sRGB table | per-triangle indices | uvs | texels.
  std::vector<MatRec> mats(m.num_materials);
  for (uint32_t i = 0; i < m.num_materials; ++i) {
    const sdfb_material &s = m.materials[i];
    mats[i] = MatRec{{s.base_color[0], s.base_color[1], s.base_color[2], s.metallic, s.roughness},
                     s.base_color_texture};
  }
  std::vector<TexRec> tex(m.num_textures);
  uint64_t pix = 0;
  for (uint32_t k = 0; k < m.num_textures; ++k) {
    const sdfb_texture &t = m.textures[k];
    tex[k] = TexRec{pix, t.width, t.height, t.srgb ? 1 : 0, 0};
    if (t.width > 0 && t.height > 0) pix += uint64_t(t.width) * uint64_t(t.height) * 4;
  }
  float lut[256];
  srgb_to_linear_table(lut);
  const size_t o_mat = 0, o_tex = align256(mats.size() * sizeof(MatRec));
  const size_t o_lut = o_tex + align256(std::max<size_t>(tex.size(), 1) * sizeof(TexRec));
  const size_t o_tri = o_lut + align256(sizeof lut);
  const size_t o_uv = o_tri + align256(m.num_triangle_material * 4 + 4);
  const size_t o_pix = o_uv + align256(m.num_uvs * 8 + 8);
  const size_t total = o_pix + align256(pix + 4);
  ENSURE(ctx->mat_in, total);
  char *d = static_cast<char *>(ctx->mat_in.p);
  CK(cudaMemcpyAsync(d + o_mat, mats.data(), mats.size() * sizeof(MatRec), cudaMemcpyHostToDevice, st));
  if (!tex.empty()) CK(cudaMemcpyAsync(d + o_tex, tex.data(), tex.size() * sizeof(TexRec), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(d + o_lut, lut, sizeof lut, cudaMemcpyHostToDevice, st));
  if (m.num_triangle_material)
    CK(cudaMemcpyAsync(d + o_tri, m.triangle_material, m.num_triangle_material * 4, cudaMemcpyHostToDevice, st));
  if (m.num_uvs) CK(cudaMemcpyAsync(d + o_uv, m.uvs, m.num_uvs * 8, cudaMemcpyHostToDevice, st));
  for (uint32_t k = 0; k < m.num_textures; ++k) {
    const sdfb_texture &t = m.textures[k];
    if (t.width > 0 && t.height > 0)
      CK(cudaMemcpyAsync(d + o_pix + tex[k].offset, t.rgba, uint64_t(t.width) * uint64_t(t.height) * 4,
                         cudaMemcpyHostToDevice, st));
  }
  MatArgs a;
  a.mats = reinterpret_cast<const MatRec *>(d + o_mat);
  a.nmat = m.num_materials;
  a.tri_mat = reinterpret_cast<const uint32_t *>(d + o_tri);
  a.ntri_mat = m.num_triangle_material;
  a.uvs = reinterpret_cast<const float *>(d + o_uv);
  a.nuv = m.num_uvs;
  a.tex = reinterpret_cast<const TexRec *>(d + o_tex);
  a.ntex = m.num_textures;
  a.pixels = reinterpret_cast<const uint8_t *>(d + o_pix);
  a.srgb_lut = reinterpret_cast<const float *>(d + o_lut);
  ENSURE(ctx->mat_tri, align256(size_t(T) * 16) + size_t(T) * 4);
  float4 *cm = static_cast<float4 *>(ctx->mat_tri.p);
  float *rough = reinterpret_cast<float *>(static_cast<char *>(ctx->mat_tri.p) + align256(size_t(T) * 16));
  k_tri_material<<<(T + kThreads - 1) / kThreads, kThreads, 0, st>>>(a, T, cm, rough);
  note_launch();
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));  // the host tables above are locals
  return SDFB_OK;
}

// Occupancy hits of the one-mesh batch B, sorted by (cell, triangle): keys in ctx->hit_keys.
sdfb_status sorted_hits(sdfb_ctx *ctx, const BatchDev &B, uint32_t T, cudaStream_t st, uint64_t &n_hits,
                        int &tri_bits) {
  tri_bits = bits_for(uint64_t(T));
  const int cell_bits = bits_for(B.total_cells);
  if (tri_bits + cell_bits > 64) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "grid and mesh too large for hit keys");
  ENSURE(ctx->sparse_tmp, occupancy_temp_bytes(T));
  uint64_t cap = std::max<uint64_t>(uint64_t(1) << 20, uint64_t(8) * T);
  if (ctx->hit_keys.cap / 8 > cap) cap = ctx->hit_keys.cap / 8;
  unsigned long long *d_count =
      reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->mat_rec.p) + 1024);  // past the records
  for (int attempt = 0; attempt < 3; ++attempt) {
    ENSURE(ctx->hit_keys, cap * 8);
    CK(occupancy_hits(B, ctx->sparse_tmp.p, ctx->sparse_tmp.cap, static_cast<uint64_t *>(ctx->hit_keys.p), cap,
                      d_count, tri_bits, ctx->num_sms, st));
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, d_count, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    n_hits = h;
    if (n_hits <= cap) break;
    cap = n_hits + n_hits / 8;
  }
  if (n_hits > ctx->hit_keys.cap / 8) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "hit list did not settle");
  ENSURE(ctx->hit_vals, n_hits * 4 + 4);
  ENSURE(ctx->hit_alt, n_hits * 12 + 512);
  ENSURE(ctx->sparse_tmp, sort_scratch_bytes(n_hits));
  uint64_t *keys_alt = static_cast<uint64_t *>(ctx->hit_alt.p);
  uint32_t *vals_alt = reinterpret_cast<uint32_t *>(static_cast<char *>(ctx->hit_alt.p) + align256(n_hits * 8));
  CK(radix_sort_pairs(static_cast<uint64_t *>(ctx->hit_keys.p), static_cast<uint32_t *>(ctx->hit_vals.p), keys_alt,
                      vals_alt, n_hits, tri_bits + cell_bits, Scratch{ctx->sparse_tmp.p, ctx->sparse_tmp.cap}, st));
  return SDFB_OK;
}

}  // namespace

extern "C" sdfb_status sdfb_bake_materials(sdfb_ctx *ctx, const float *positions, uint32_t num_tris,
                                           const sdfb_grid_desc *grid, const sdfb_materials *materials,
                                           float *base_color_out, float *metallic_out, float *roughness_out) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!grid_ok(grid)) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "bad grid");
  if (num_tris && !positions) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "positions is NULL");
  const sdfb_status ms = check_materials(ctx, materials);
  if (ms != SDFB_OK) return ms;
  cudaSetDevice(ctx->device);
  const cudaStream_t st = ctx->stream;
  const uint64_t cells = uint64_t(grid->nx) * grid->ny * grid->nz;
  ENSURE(ctx->mat_cells, align256(cells * 12) + 2 * align256(cells * 4));
  float *color = static_cast<float *>(ctx->mat_cells.p);
  float *metal = reinterpret_cast<float *>(static_cast<char *>(ctx->mat_cells.p) + align256(cells * 12));
  float *rough = reinterpret_cast<float *>(reinterpret_cast<char *>(metal) + align256(cells * 4));
  const unsigned fill_blocks = static_cast<unsigned>(std::min<uint64_t>((cells + kThreads - 1) / kThreads,
                                                                        uint64_t(ctx->num_sms) * 16));
  k_mat_defaults<<<std::max(fill_blocks, 1u), kThreads, 0, st>>>(cells, color, metal, rough);
  note_launch();
  CK(cudaGetLastError());
  if (num_tris > 0) {
    BatchDev B;
    sdfb_status s = soup_batch(ctx, positions, num_tris, *grid, st, B);
    if (s != SDFB_OK) return s;
    if ((s = triangle_materials(ctx, *materials, num_tris, st)) != SDFB_OK) return s;
    uint64_t n_hits = 0;
    int tri_bits = 0;
    if ((s = sorted_hits(ctx, B, num_tris, st, n_hits, tri_bits)) != SDFB_OK) return s;
    if (n_hits) {
      const float4 *cm = static_cast<const float4 *>(ctx->mat_tri.p);
      const float *tr = reinterpret_cast<const float *>(static_cast<char *>(ctx->mat_tri.p) +
                                                        align256(size_t(num_tris) * 16));
      const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n_hits + kThreads - 1) / kThreads,
                                                                       uint64_t(ctx->num_sms) * 16));
      k_mat_dense<<<blocks, kThreads, 0, st>>>(static_cast<const uint64_t *>(ctx->hit_keys.p), n_hits, tri_bits, cm,
                                               tr, color, metal, rough);
      note_launch();
      CK(cudaGetLastError());
    }
  }
  if (base_color_out) CK(cudaMemcpyAsync(base_color_out, color, cells * 12, cudaMemcpyDeviceToHost, st));
  if (metallic_out) CK(cudaMemcpyAsync(metallic_out, metal, cells * 4, cudaMemcpyDeviceToHost, st));
  if (roughness_out) CK(cudaMemcpyAsync(roughness_out, rough, cells * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

extern "C" sdfb_status sdfb_voxelize_sparse_colors(sdfb_ctx *ctx, const float *positions, uint32_t num_tris,
                                                   const float bounds_min[3], const float bounds_max[3],
                                                   int32_t resolution, const sdfb_materials *materials,
                                                   int32_t *cells_out, float *colors_out, uint64_t cap,
                                                   uint64_t *count, float origin_out[3], float *voxel_out) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (cap && !colors_out) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "colors_out is NULL");
  const sdfb_status ms = check_materials(ctx, materials);
  if (ms != SDFB_OK) return ms;
  const uint32_t *d_list = nullptr;
  sdfb_grid_desc g;
  sdfb_status s = voxelize_sparse_run(ctx, positions, num_tris, bounds_min, bounds_max, resolution, cells_out, cap,
                                      count, origin_out, voxel_out, &d_list, &g);
  if (s != SDFB_OK) return s;
  const uint64_t n_out = std::min<uint64_t>(*count, cap);
  if (n_out == 0) return SDFB_OK;
  const cudaStream_t st = ctx->stream;
  BatchDev B;
  if ((s = soup_batch(ctx, positions, num_tris, g, st, B)) != SDFB_OK) return s;
  if ((s = triangle_materials(ctx, *materials, num_tris, st)) != SDFB_OK) return s;
  uint64_t n_hits = 0;
  int tri_bits = 0;
  if ((s = sorted_hits(ctx, B, num_tris, st, n_hits, tri_bits)) != SDFB_OK) return s;
  ENSURE(ctx->mat_cells, n_out * 12);
  const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n_out + kThreads - 1) / kThreads,
                                                                   uint64_t(ctx->num_sms) * 16));
  k_mat_sparse<<<blocks, kThreads, 0, st>>>(d_list, n_out, static_cast<const uint64_t *>(ctx->hit_keys.p), n_hits,
                                            tri_bits, static_cast<const float4 *>(ctx->mat_tri.p),
                                            static_cast<float *>(ctx->mat_cells.p));
  note_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(colors_out, ctx->mat_cells.p, n_out * 12, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}
