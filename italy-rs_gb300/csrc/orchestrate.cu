// The batch orchestrator behind every bake entry point.
//
//   upload mesh records + prefix tables -> BVH over all meshes (lbvh.cu) -> occupancy
//   (occupancy.cu) -> +z crossing lists of the parity and winding-number meshes (parity.cu) ->
//   caps hierarchy for the winding number -> distance with fused parity sign, one persistent
//   launch over every mesh's tiles (distance.cu) -> winding-number signs (gwn.cu)
//
// CUDA events bracket each stage for the per-stage times in sdfb_stats. After the stream drains,
// the device error word is read: bad indices and non-finite vertices become SDFB_ERR_BAD_MESH; a
// crossing list that outgrew its buffer is rebuilt at its exact size. For batches whose stages
// need no host round trip (no winding-number meshes), the launch sequence is captured into a CUDA
// graph and replayed while the same batch (same tables, sizes and buffers) comes again.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "host_mesh.h"
#include "kernels.h"

using namespace sdfb;

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

// ---------------------------------------------------------------------------------------------
// Tuned defaults: leaf size, tile shape and stack depth per (log2 triangles, log2 grid edge - 4).
// The table is written by the autotuner (italy-rs_gb300/sdfb/autotune.py) as lines
// "tri_bucket grid_bucket leaf tile stack" in italy-rs_gb300/tuning/gb300.tsv next to lib/;
// SDFB_TUNING names another file.

int bucket_tris(uint64_t T) {
  int b = 0;
  while (b < 31 && (uint64_t(2) << b) <= T) ++b;
  return b;
}

int bucket_grid(const sdfb_grid_desc &g) {
  const int n = std::max(g.nx, std::max(g.ny, g.nz));
  int b = 0;
  while (b < 20 && (2 << b) <= n) ++b;
  return std::max(0, std::min(7, b - 4));
}

void load_tuning(sdfb_ctx *ctx) {
  for (int i = 0; i < 32; ++i)
    for (int j = 0; j < 8; ++j) {
      ctx->tuned_leaf[i][j] = 4;
      ctx->tuned_tile[i][j] = 2;
      ctx->tuned_stack[i][j] = 64;
    }
  std::string path;
  if (const char *env = std::getenv("SDFB_TUNING")) {
    path = env;
  } else {
    Dl_info info;
    if (dladdr(reinterpret_cast<void *>(&load_tuning), &info) && info.dli_fname) {
      path = info.dli_fname;
      const size_t cut = path.rfind('/');
      path = (cut == std::string::npos ? std::string(".") : path.substr(0, cut)) + "/../tuning/gb300.tsv";
    }
  }
  FILE *f = path.empty() ? nullptr : std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[256];
  while (std::fgets(line, sizeof line, f)) {
    int tb, nb, leaf, tile, stack;
    if (line[0] == '#' || std::sscanf(line, "%d %d %d %d %d", &tb, &nb, &leaf, &tile, &stack) != 5) continue;
    if (tb < 0 || tb >= 32 || nb < 0 || nb >= 8) continue;
    if (leaf >= 1 && leaf <= 16) ctx->tuned_leaf[tb][nb] = leaf;
    if (tile >= 0 && tile < tile_shape_count()) ctx->tuned_tile[tb][nb] = tile;
    if (stack == 32 || stack == 64) ctx->tuned_stack[tb][nb] = stack;
  }
  std::fclose(f);
}

// ---------------------------------------------------------------------------------------------
// Winding-number caps.

void build_caps(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, CapBuild &out) {
  std::vector<float> centres;
  out.loops = boundary_caps(verts, V, idx, T, centres, out.cidx);
  out.verts.assign(verts, verts + 3 * size_t(V));
  out.verts.insert(out.verts.end(), centres.begin(), centres.end());
  out.pidx.assign(idx, idx + 3 * size_t(T));
  out.pidx.insert(out.pidx.end(), out.cidx.begin(), out.cidx.end());
}

// ---------------------------------------------------------------------------------------------
// Batch layout: per-mesh records and prefix tables, uploaded in one copy.

namespace {

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  std::vector<MeshRec> recs, cap_recs;
  std::vector<uint64_t> tri, ptri, tile, gtile, cell, cap_tri, cap_zero;
  uint64_t total_cols = 0, gwn_cells = 0, cap_total = 0;
  int tile_id = 2, stack = 64;
  size_t o_recs = 0, o_tri = 0, o_ptri = 0, o_tile = 0, o_gtile = 0, o_cell = 0, o_caprecs = 0, o_captri = 0,
         o_capzero = 0, bytes = 0;
};

void make_layout(sdfb_ctx *ctx, const std::vector<PlanMesh> &ms, const sdfb_opts &o, Layout &L) {
  const int M = static_cast<int>(ms.size());
  // Batch-wide tile shape and stack depth: tuned for the mesh with the most cells, unless forced.
  size_t big = 0;
  for (int m = 1; m < M; ++m)
    if (uint64_t(ms[m].grid.nx) * ms[m].grid.ny * ms[m].grid.nz >
        uint64_t(ms[big].grid.nx) * ms[big].grid.ny * ms[big].grid.nz)
      big = m;
  const int tb = bucket_tris(ms[big].T), nb = bucket_grid(ms[big].grid);
  L.tile_id = (o.tile >= 1 && o.tile <= tile_shape_count()) ? o.tile - 1 : ctx->tuned_tile[tb][nb];
  L.stack = (o.stack_depth == 32 || o.stack_depth == 64) ? o.stack_depth : ctx->tuned_stack[tb][nb];
  uint64_t T_total = 0;
  for (const auto &p : ms) T_total += p.T;
  const int num_inner = T_total >= 2 ? static_cast<int>(T_total - 1) : 0;
  L.recs.resize(M);
  L.tri.assign(M + 1, 0);
  L.ptri.assign(M + 1, 0);
  L.tile.assign(M + 1, 0);
  L.gtile.assign(M + 1, 0);
  L.cell.assign(M + 1, 0);
  L.cap_tri.assign(1, 0);
  uint64_t cols = 0;
  for (int m = 0; m < M; ++m) {
    const PlanMesh &p = ms[m];
    MeshRec &r = L.recs[m];
    std::memset(&r, 0, sizeof r);
    r.verts = p.verts;
    r.idx = p.idx;
    r.pverts = p.pverts ? p.pverts : p.verts;
    r.pidx = p.pidx ? p.pidx : p.idx;
    r.num_verts = p.V;
    r.num_tris = p.T;
    r.pnum_verts = p.pverts ? p.pV : p.V;
    r.pnum_tris = p.pverts ? p.pT : p.T;
    r.dist = p.dist;
    r.occ = p.occ;
    r.g = to_dev(p.grid);
    r.sign = p.dist ? p.sign : kSignNone;
    const int leaf = p.leaf > 0 ? p.leaf
                                : (o.leaf_size > 0 ? o.leaf_size
                                                   : ctx->tuned_leaf[bucket_tris(p.T)][bucket_grid(p.grid)]);
    r.leaf_size = std::max(1, std::min(leaf, 16));
    r.root = num_inner + m;
    r.cap_root = -1;
    const uint64_t cells = uint64_t(p.grid.nx) * p.grid.ny * p.grid.nz;
    r.tri_base = L.tri[m];
    r.cell_base = L.cell[m];
    L.tri[m + 1] = L.tri[m] + p.T;
    L.cell[m + 1] = L.cell[m] + cells;
    const bool crossings = r.sign == kSignParity || r.sign == kSignGwn;
    L.ptri[m + 1] = L.ptri[m] + (crossings ? r.pnum_tris : 0);
    r.col_base = cols;
    if (crossings) cols += uint64_t(p.grid.nx) * p.grid.ny;
    L.tile[m + 1] = L.tile[m] + (p.dist ? tiles_for(r.g, L.tile_id) : 0);
    const bool gwn = p.dist && r.sign == kSignGwn;
    L.gtile[m + 1] = L.gtile[m] + (gwn ? uint64_t((p.grid.nx + 3) / 4) * uint64_t((p.grid.ny + 3) / 4) *
                                             uint64_t((p.grid.nz + 1) / 2)
                                       : 0);
    if (gwn) {
      L.gwn_cells += cells;
      r.cverts = p.cverts;
      r.cidx = p.cidx;
      r.cap_tris = p.cT;
      if (p.cT > 0) {
        MeshRec c;
        std::memset(&c, 0, sizeof c);
        c.verts = p.cverts;
        c.idx = p.cidx;
        c.num_verts = p.pV;
        c.num_tris = p.cT;
        c.leaf_size = 4;
        c.tri_base = L.cap_tri.back();
        L.cap_recs.push_back(c);
        L.cap_tri.push_back(L.cap_tri.back() + p.cT);
        r.cap_root = static_cast<int>(L.cap_recs.size()) - 1;  // offset by the caps' inner nodes below
      }
    }
  }
  L.total_cols = cols;
  L.cap_total = L.cap_tri.back();
  const int K = static_cast<int>(L.cap_recs.size());
  const int cap_inner = L.cap_total >= 2 ? static_cast<int>(L.cap_total - 1) : 0;
  for (int m = 0; m < M; ++m)
    if (L.recs[m].cap_root >= 0) L.recs[m].cap_root += cap_inner;
  for (int k = 0; k < K; ++k) L.cap_recs[k].root = cap_inner + k;
  L.cap_zero.assign(K + 1, 0);
  size_t off = 0;
  auto put = [&](size_t bytes) {
    const size_t at = off;
    off += align256(bytes);
    return at;
  };
  L.o_recs = put(M * sizeof(MeshRec));
  L.o_tri = put((M + 1) * 8);
  L.o_ptri = put((M + 1) * 8);
  L.o_tile = put((M + 1) * 8);
  L.o_gtile = put((M + 1) * 8);
  L.o_cell = put((M + 1) * 8);
  L.o_caprecs = put(std::max(K, 1) * sizeof(MeshRec));
  L.o_captri = put((K + 1) * 8);
  L.o_capzero = put((K + 1) * 8);
  L.bytes = off;
}

void fill_staging(const Layout &L, char *s) {
  std::memset(s, 0, L.bytes);
  std::memcpy(s + L.o_recs, L.recs.data(), L.recs.size() * sizeof(MeshRec));
  std::memcpy(s + L.o_tri, L.tri.data(), L.tri.size() * 8);
  std::memcpy(s + L.o_ptri, L.ptri.data(), L.ptri.size() * 8);
  std::memcpy(s + L.o_tile, L.tile.data(), L.tile.size() * 8);
  std::memcpy(s + L.o_gtile, L.gtile.data(), L.gtile.size() * 8);
  std::memcpy(s + L.o_cell, L.cell.data(), L.cell.size() * 8);
  if (!L.cap_recs.empty()) std::memcpy(s + L.o_caprecs, L.cap_recs.data(), L.cap_recs.size() * sizeof(MeshRec));
  std::memcpy(s + L.o_captri, L.cap_tri.data(), L.cap_tri.size() * 8);
  std::memcpy(s + L.o_capzero, L.cap_zero.data(), L.cap_zero.size() * 8);
}

BatchDev batch_dev(const Layout &L, char *d) {
  BatchDev B;
  B.num_meshes = static_cast<int>(L.recs.size());
  B.recs = reinterpret_cast<const MeshRec *>(d + L.o_recs);
  B.tri_starts = reinterpret_cast<const uint64_t *>(d + L.o_tri);
  B.ptri_starts = reinterpret_cast<const uint64_t *>(d + L.o_ptri);
  B.tile_starts = reinterpret_cast<const uint64_t *>(d + L.o_tile);
  B.gwn_tile_starts = reinterpret_cast<const uint64_t *>(d + L.o_gtile);
  B.cell_starts = reinterpret_cast<const uint64_t *>(d + L.o_cell);
  B.total_tris = L.tri.back();
  B.total_ptris = L.ptri.back();
  B.total_cells = L.cell.back();
  B.total_cols = L.total_cols;
  B.total_tiles = L.tile.back();
  B.total_gwn_tiles = L.gtile.back();
  return B;
}

BatchDev caps_dev(const Layout &L, char *d) {
  BatchDev B;
  B.num_meshes = static_cast<int>(L.cap_recs.size());
  B.recs = reinterpret_cast<const MeshRec *>(d + L.o_caprecs);
  B.tri_starts = reinterpret_cast<const uint64_t *>(d + L.o_captri);
  B.ptri_starts = B.tile_starts = B.gwn_tile_starts = B.cell_starts =
      reinterpret_cast<const uint64_t *>(d + L.o_capzero);
  B.total_tris = L.cap_total;
  return B;
}

}  // namespace

sdfb_status run_batch(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &ms, const sdfb_opts &o, bool use_graph,
                      sdfb_stats *stats) {
  if (ms.empty()) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "empty batch");
  Layout L;
  make_layout(ctx, ms, o, L);
  const int M = static_cast<int>(ms.size());
  const int K = static_cast<int>(L.cap_recs.size());
  const uint64_t T = L.tri.back();
  if (T == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh has no triangles");
  if (T >= (1ull << 31) || L.ptri.back() >= (1ull << 31) || M >= (1 << 25))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "batch too large");
  const bool any_gwn = L.gtile.back() > 0;
  const bool any_cross = L.ptri.back() > 0;
  const bool any_occ = std::any_of(ms.begin(), ms.end(), [](const PlanMesh &p) { return p.occ != nullptr; });

  // Workspace.
  ENSURE(ctx->batch_buf, L.bytes);
  if (!ctx->staging.ensure(L.bytes)) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "pinned staging");
  ENSURE(ctx->bvh, lbvh_bytes(T, M, false));
  ENSURE(ctx->build_tmp, std::max(lbvh_temp_bytes(T, M), occupancy_temp_bytes(T)));
  ENSURE(ctx->misc, 256);
  uint64_t capacity = 0;
  if (any_cross) {
    ENSURE(ctx->par_tmp, parity_temp_bytes(L.ptri.back(), L.total_cols));
    ENSURE(ctx->col_start, (L.total_cols + 1) * 8);
    capacity = std::max<uint64_t>(ctx->col_capacity_hint, 4 * L.total_cols + 2 * L.ptri.back());
    ENSURE(ctx->col_z, capacity * 4);
    ENSURE(ctx->col_s, capacity);
    capacity = std::min<uint64_t>(ctx->col_z.cap / 4, ctx->col_s.cap);
  }
  if (K > 0) {
    ENSURE(ctx->caps_bvh, lbvh_bytes(L.cap_total, K, true));
    ENSURE(ctx->caps_tmp, lbvh_temp_bytes(L.cap_total, K));
  }
  fill_staging(L, static_cast<char *>(ctx->staging.p));
  const BatchDev B = batch_dev(L, static_cast<char *>(ctx->batch_buf.p));
  BvhDev bvh;
  lbvh_bind(bvh, ctx->bvh.p, T, M, false);
  BvhDev caps;
  BatchDev CB;
  if (K > 0) {
    lbvh_bind(caps, ctx->caps_bvh.p, L.cap_total, K, true);
    CB = caps_dev(L, static_cast<char *>(ctx->batch_buf.p));
  }
  uint32_t *d_err = static_cast<uint32_t *>(ctx->misc.p);
  unsigned long long *d_tile = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->misc.p) + 64);
  unsigned long long *d_work = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->misc.p) + 128);
  unsigned long long *d_sat = d_work + 2;
  DistanceArgs da{};
  da.batch = B;
  da.nodes = bvh.nodes;
  da.tris = bvh.tris;
  da.num_nodes = bvh.num_nodes;
  da.col_start = static_cast<const uint64_t *>(ctx->col_start.p);
  da.col_z = static_cast<const float *>(ctx->col_z.p);
  da.err = d_err;
  da.tile_counter = d_tile;
  da.work_counters = o.count_work ? d_work : nullptr;

  auto enqueue = [&]() -> sdfb_status {
    CK(cudaMemcpyAsync(ctx->batch_buf.p, ctx->staging.p, L.bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(ctx->misc.p, 0, 256, st));
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(lbvh_build(B, bvh, ctx->build_tmp.p, ctx->build_tmp.cap, d_err, st));
    CK(cudaEventRecord(ctx->ev[1], st));
    if (any_occ) CK(occupancy_batch(B, nullptr, ctx->build_tmp.p, ctx->build_tmp.cap, d_sat, ctx->num_sms, st));
    CK(cudaEventRecord(ctx->ev[2], st));
    if (any_cross)
      CK(parity_columns(B, static_cast<uint64_t *>(ctx->col_start.p), static_cast<float *>(ctx->col_z.p),
                        static_cast<int8_t *>(ctx->col_s.p), capacity, ctx->par_tmp.p, ctx->par_tmp.cap, d_err,
                        ctx->num_sms, st));
    if (K > 0) CK(lbvh_build(CB, caps, ctx->caps_tmp.p, ctx->caps_tmp.cap, d_err, st));
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(distance_launch(da, L.tile_id, L.stack, ctx->num_sms, st));
    CK(cudaEventRecord(ctx->ev[4], st));
    return SDFB_OK;
  };

  const uint64_t launches0 = launch_count();
  uint64_t launched = 0;
  sdfb_status s;
  bool graphed = false;
  if (use_graph && !any_gwn && !o.count_work) {
    // Key: the uploaded tables plus every buffer and option the launch sequence bakes in.
    std::vector<uint8_t> key(static_cast<const uint8_t *>(ctx->staging.p),
                             static_cast<const uint8_t *>(ctx->staging.p) + L.bytes);
    const void *ptrs[] = {ctx->batch_buf.p, ctx->bvh.p, ctx->build_tmp.p, ctx->par_tmp.p, ctx->col_start.p,
                          ctx->col_z.p,     ctx->col_s.p, ctx->misc.p,    ctx->staging.p, static_cast<void *>(st)};
    const uint64_t extra[] = {uint64_t(L.tile_id), uint64_t(L.stack), capacity, L.bytes, ctx->build_tmp.cap,
                              ctx->par_tmp.cap};
    key.insert(key.end(), reinterpret_cast<const uint8_t *>(ptrs), reinterpret_cast<const uint8_t *>(ptrs) + sizeof ptrs);
    key.insert(key.end(), reinterpret_cast<const uint8_t *>(extra),
               reinterpret_cast<const uint8_t *>(extra) + sizeof extra);
    if (!ctx->graph || key != ctx->graph_key) {
      if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
        ctx->graph_key.clear();
      }
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      s = enqueue();
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(st, &g);
      if (s != SDFB_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
      }
      if (ce != cudaSuccess) return ctx_cuda(ctx, ce, "cudaStreamEndCapture");
      const cudaError_t ie = cudaGraphInstantiate(&ctx->graph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) {
        ctx->graph = nullptr;
        return ctx_cuda(ctx, ie, "cudaGraphInstantiate");
      }
      ctx->graph_key.swap(key);
      ctx->graph_launches = launch_count() - launches0;
    }
    CK(cudaGraphLaunch(ctx->graph, st));
    launched = ctx->graph_launches;
    graphed = true;
  } else {
    if ((s = enqueue()) != SDFB_OK) return s;
  }
  ctx->gwn_refined = 0;
  if (any_gwn) {
    // the winding-number pass reads the crossing lists: make sure they fit first
    uint32_t h_err0 = 0;
    CK(cudaMemcpyAsync(&h_err0, d_err, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (!(h_err0 & (kErrCrossingOverflow | kErrBadIndex | kErrNonFinite))) {
      GwnInput gi;
      gi.batch = B;
      gi.col_start = static_cast<const uint64_t *>(ctx->col_start.p);
      gi.col_z = static_cast<const float *>(ctx->col_z.p);
      gi.col_s = static_cast<const int8_t *>(ctx->col_s.p);
      gi.caps = caps;
      gi.cap_total_tris = L.cap_total;
      gi.band_voxels = o.band_voxels;
      gi.err = d_err;
      gi.gwn_cells = L.gwn_cells;
      if ((s = gwn_apply(ctx, st, gi)) != SDFB_OK) return s;
    }
  }
  CK(cudaEventRecord(ctx->ev[5], st));
  if (!graphed) launched = launch_count() - launches0;

  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err & (kErrBadIndex | kErrNonFinite))
    return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "%s",
                    (h_err & kErrBadIndex) ? "triangle index out of range" : "mesh has a non-finite vertex");
  if (h_err & kErrStackOverflow) {
    if (L.stack < 64) {  // the tuned shallow stack was too small for this tree: rerun with 64
      sdfb_opts o2 = o;
      o2.stack_depth = 64;
      return run_batch(ctx, st, ms, o2, use_graph, stats);
    }
    return ctx_fail(ctx, SDFB_ERR_OVERFLOW, "BVH traversal stack overflow (depth > 64)");
  }
  if (h_err & kErrCorruptTree) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "BVH walk met an invalid reference");
  if (h_err & kErrCrossingOverflow) {
    uint64_t need = 0;
    CK(cudaMemcpy(&need, static_cast<uint64_t *>(ctx->col_start.p) + L.total_cols, 8, cudaMemcpyDeviceToHost));
    if (need <= capacity) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "crossing list overflow after resize");
    ctx->col_capacity_hint = need + need / 4 + 1024;
    return run_batch(ctx, st, ms, o, use_graph, stats);
  }

  if (stats) {
    sdfb_stats sv;
    std::memset(&sv, 0, sizeof sv);
    sv.struct_size = sizeof sv;
    sv.sign_mode_used = ms[0].sign == kSignParity ? SDFB_SIGN_PARITY
                                                  : (ms[0].sign == kSignGwn ? SDFB_SIGN_GWN : SDFB_SIGN_NONE);
    sv.watertight = ms[0].watertight;
    sv.leaf_size_used = L.recs[0].leaf_size;
    sv.tile_used = L.tile_id + 1;
    sv.stack_used = L.stack;
    float ms_b = 0, ms_o = 0, ms_s = 0, ms_d = 0, ms_g = 0, tot = 0;
    cudaEventElapsedTime(&ms_b, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&ms_o, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&ms_s, ctx->ev[2], ctx->ev[3]);
    cudaEventElapsedTime(&ms_d, ctx->ev[3], ctx->ev[4]);
    cudaEventElapsedTime(&ms_g, ctx->ev[4], ctx->ev[5]);
    cudaEventElapsedTime(&tot, ctx->ev[0], ctx->ev[5]);
    sv.ms_total = tot;
    sv.ms_build = ms_b;
    sv.ms_occupancy = ms_o;
    sv.ms_sign = ms_s + ms_g;
    sv.ms_distance = ms_d;
    sv.voxels = L.cell.back();
    sv.triangles = T;
    unsigned long long w[3] = {0, 0, 0};
    cudaMemcpy(w, d_work, sizeof w, cudaMemcpyDeviceToHost);
    sv.box_tests = w[0];
    sv.tri_tests = w[1];
    sv.sat_tests = w[2];
    sv.flops_distance = double(w[0]) * kFlopsPointBox + double(w[1]) * kFlopsPointTri;
    if (any_cross)
      cudaMemcpy(&sv.crossings, static_cast<uint64_t *>(ctx->col_start.p) + L.total_cols, 8, cudaMemcpyDeviceToHost);
    sv.kernel_launches = launched;
    sv.gwn_fp64_cells = ctx->gwn_refined;
    sv.graph_replayed = graphed ? 1 : 0;
    const size_t n = std::min<size_t>(stats->struct_size ? stats->struct_size : sizeof sv, sizeof sv);
    std::memcpy(stats, &sv, n);
  }
  return SDFB_OK;
}
