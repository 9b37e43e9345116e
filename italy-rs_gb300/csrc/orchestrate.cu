// The batch orchestrator behind every bake entry point.
//
//   upload mesh records + prefix tables -> BVH over all meshes (lbvh.cu) -> occupancy
//   (occupancy.cu) -> +z crossing lists of the parity and winding-number meshes (parity.cu) ->
//   caps hierarchy for the winding number -> distance with fused parity sign, one persistent
//   launch over every mesh's tiles (distance.cu) -> winding-number signs (gwn.cu)
//
// CUDA events bracket each stage for the per-stage times in sdfb_stats. After the stream drains,
// the device error word is read: bad indices and non-finite vertices become SDFB_ERR_BAD_MESH; a
// crossing list that outgrew its buffer is rebuilt at its exact size. For the batch entry points
// the launch sequence is captured into a CUDA graph and replayed while the same batch (same
// tables, sizes and buffers) comes again; no stage inside it needs a host round trip (the
// winding-number passes read their list lengths on the device, and the caps of winding-number
// meshes are built before it, by api.cu's device_caps).
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

// A test-only cap on single workspace allocations (sdfb_opts.alloc_cap_kib), set per bake on the
// calling thread: an allocation above it fails as cudaMalloc would when the device is full.
thread_local uint64_t t_alloc_cap = 0;

#define ENSURE(buf, bytes)                                                                       \
  do {                                                                                           \
    if ((t_alloc_cap && static_cast<uint64_t>(bytes) > t_alloc_cap) || !(buf).ensure(bytes))     \
      return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of device memory", \
                      static_cast<size_t>(bytes));                                               \
  } while (0)

// ---------------------------------------------------------------------------------------------
// Tuned defaults: leaf size, tile shape, stack depth and the distance pass's deferral budget per
// (log2 triangles, log2 grid edge - 4). The table is written by the autotuner
// (italy-rs_gb300/sdfb/autotune.py) as lines "tri_bucket grid_bucket leaf tile stack [budget]" in
// italy-rs_gb300/tuning/gb300.tsv next to lib/; SDFB_TUNING names another file. An optional line
// "batch tile stack budget" (written by the tuner's batch mode) sets the tile shape, stack depth
// and budget of every bake of more than one mesh.

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
      ctx->tuned_budget[i][j] = kDefaultStepBudget;
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
    int tb, nb, leaf, tile, stack, budget = -1;
    if (std::sscanf(line, "batch %d %d %d", &tile, &stack, &budget) == 3) {
      if (tile >= 0 && tile < tile_shape_count() && (stack == 32 || stack == 64) && budget >= 0) {
        ctx->batch_tile = tile;
        ctx->batch_stack = stack;
        ctx->batch_budget = budget;
      }
      continue;
    }
    if (line[0] == '#' || std::sscanf(line, "%d %d %d %d %d %d", &tb, &nb, &leaf, &tile, &stack, &budget) < 5)
      continue;
    if (tb < 0 || tb >= 32 || nb < 0 || nb >= 8) continue;
    if (leaf >= 1 && leaf <= 16) ctx->tuned_leaf[tb][nb] = leaf;
    if (tile >= 0 && tile < tile_shape_count()) ctx->tuned_tile[tb][nb] = tile;
    if (stack == 32 || stack == 64) ctx->tuned_stack[tb][nb] = stack;
    if (budget >= 0) ctx->tuned_budget[tb][nb] = budget;  // 0 turns deferral off
  }
  std::fclose(f);
}

// ---------------------------------------------------------------------------------------------
// Workspace.

bool Workspace::init() {
  for (auto &e : ev)
    if (!e && cudaEventCreate(&e) != cudaSuccess) return false;
  return true;
}

Workspace::~Workspace() {
  if (graph) cudaGraphExecDestroy(graph);
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
}

void Workspace::release() {
  if (graph) {
    cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_key.clear();
  }
  DevBuf *b[] = {&batch_buf, &bvh, &build_tmp, &par_tmp, &col_start, &col_z, &col_s, &caps_bvh, &caps_tmp, &misc,
                 &gwn_tmp, &defer};
  for (DevBuf *x : b) x->release();
  staging.release();
}

uint64_t Workspace::bytes() const {
  const DevBuf *b[] = {&batch_buf, &bvh, &build_tmp, &par_tmp, &col_start, &col_z, &col_s, &caps_bvh, &caps_tmp,
                       &misc, &gwn_tmp, &defer};
  uint64_t s = 0;
  for (const DevBuf *x : b) s += x->cap;
  return s;
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
  long long step_budget = 0;
  bool resident = false;
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
  const bool batch = M > 1 && ctx->batch_tile >= 0;  // the table's batch-wide line, when it has one
  L.tile_id = (o.tile >= 1 && o.tile <= tile_shape_count()) ? o.tile - 1
                                                           : (batch ? ctx->batch_tile : ctx->tuned_tile[tb][nb]);
  L.stack = (o.stack_depth == 32 || o.stack_depth == 64) ? o.stack_depth
                                                         : (batch ? ctx->batch_stack : ctx->tuned_stack[tb][nb]);
  L.step_budget = o.step_budget > 0 ? o.step_budget
                                    : (o.step_budget < 0 ? 0 : (batch ? ctx->batch_budget : ctx->tuned_budget[tb][nb]));
  L.resident = ms[0].bvh != nullptr;
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
    if (p.bvh) {
      r.nodes = p.bvh->nodes;
      r.tris = p.bvh->dtris;
      r.bvh_nodes = p.bvh->num_nodes;
      r.bvh_tris = p.bvh->num_tris;
      r.root = p.bvh->root;
    }
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
                                             uint64_t((p.grid.nz + kGwnTileZ - 1) / kGwnTileZ)
                                       : 0);
    if (gwn) {
      L.gwn_cells += cells;
      r.cverts = p.cverts;
      r.cidx = p.cidx;
      r.cap_tris = p.cT;
      if (p.caps) {
        r.cap_root = p.caps->root;
        r.cap_nodes = p.caps->nodes;
        r.cap_trec = p.caps->tris;
        r.cap_moment = p.caps->node_moment;
        r.cap_order = p.caps->leaf_order;
        r.cap_nodes_n = p.caps->num_nodes;
        r.cap_inner_n = p.caps->num_inner;
        r.cap_recs_n = p.caps->num_tris;
      } else if (p.cT > 0) {
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
    if (L.recs[m].cap_root >= 0 && !ms[m].caps) L.recs[m].cap_root += cap_inner;
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

// Points the records at the combined hierarchies built for this batch.
void bind_built(Layout &L, const BvhDev &bvh, const BvhDev *caps) {
  for (auto &r : L.recs) {
    if (bvh.nodes) {
      r.nodes = bvh.nodes;
      r.tris = bvh.dtris;
      r.bvh_nodes = bvh.num_nodes;
      r.bvh_tris = static_cast<int>(L.tri.back());
    }
    if (caps && r.cap_root >= 0 && !r.cap_nodes) {
      r.cap_nodes = caps->nodes;
      r.cap_trec = caps->tris;
      r.cap_moment = caps->node_moment;
      r.cap_order = caps->leaf_order;
      r.cap_nodes_n = caps->num_nodes;
      r.cap_inner_n = caps->num_inner;
      r.cap_recs_n = static_cast<int>(L.cap_total);
    }
  }
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

sdfb_status enqueue_batch(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, std::vector<PlanMesh> &ms,
                          const sdfb_opts &o, bool use_graph, BatchState &S) {
  if (ms.empty()) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "empty batch");
  cudaGetLastError();  // start from a clean error state
  if (!ws.init()) return ctx_fail(ctx, SDFB_ERR_CUDA, "cannot create events");
  for (const auto &p : ms)
    if ((p.bvh != nullptr) != (ms[0].bvh != nullptr))
      return ctx_fail(ctx, SDFB_ERR_INTERNAL, "a batch mixes resident and unbuilt meshes");
  t_alloc_cap = o.alloc_cap_kib > 0 ? uint64_t(o.alloc_cap_kib) << 10 : 0;
  Layout L;
  make_layout(ctx, ms, o, L);
  const int M = static_cast<int>(ms.size());
  const int K = static_cast<int>(L.cap_recs.size());
  const uint64_t T = L.tri.back();
  if (T == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh has no triangles");
  if (T >= (1ull << 31) || L.ptri.back() >= (1ull << 31) || M >= (1 << 25))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "batch too large");
  S = BatchState();
  S.any_gwn = L.gtile.back() > 0;
  S.any_cross = L.ptri.back() > 0;
  S.total_cols = L.total_cols;
  S.total_cells = L.cell.back();
  S.total_tris = T;
  S.tile_id = L.tile_id;
  S.stack = L.stack;
  S.leaf0 = L.recs[0].leaf_size;
  const bool any_occ = std::any_of(ms.begin(), ms.end(), [](const PlanMesh &p) { return p.occ != nullptr; });
  const bool build = !L.resident;

  // Workspace.
  ENSURE(ws.batch_buf, L.bytes);
  if (!ws.staging.ensure(L.bytes)) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "pinned staging");
  if (build) ENSURE(ws.bvh, lbvh_bytes(T, M, false));
  ENSURE(ws.build_tmp, std::max(build ? lbvh_temp_bytes(T, M) : size_t(0), occupancy_temp_bytes(T)));
  ENSURE(ws.misc, 256);
  if (S.any_cross) {
    ENSURE(ws.par_tmp, parity_temp_bytes(L.ptri.back(), L.total_cols));
    ENSURE(ws.col_start, (L.total_cols + 1) * 8);
    const uint64_t want = std::max<uint64_t>(ws.col_capacity_hint, 4 * L.total_cols + 2 * L.ptri.back());
    ENSURE(ws.col_z, want * 4);
    ENSURE(ws.col_s, want);
    S.capacity = std::min<uint64_t>(ws.col_z.cap / 4, ws.col_s.cap);
  }
  if (K > 0) {
    ENSURE(ws.caps_bvh, lbvh_bytes(L.cap_total, K, true));
    ENSURE(ws.caps_tmp, lbvh_temp_bytes(L.cap_total, K));
  }
  if (S.any_gwn) ENSURE(ws.gwn_tmp, gwn_temp_bytes(L.gwn_cells));
  const uint64_t defer_cap = L.step_budget > 0 ? defer_capacity_for(L.tile.back()) : 0;
  if (defer_cap > 0) ENSURE(ws.defer, defer_cap * 8);
  BvhDev bvh, caps;
  if (build) lbvh_bind(bvh, ws.bvh.p, T, M, false);
  if (K > 0) lbvh_bind(caps, ws.caps_bvh.p, L.cap_total, K, true);
  bind_built(L, build ? bvh : BvhDev(), K > 0 ? &caps : nullptr);
  fill_staging(L, static_cast<char *>(ws.staging.p));
  const BatchDev B = batch_dev(L, static_cast<char *>(ws.batch_buf.p));
  const BatchDev CB = K > 0 ? caps_dev(L, static_cast<char *>(ws.batch_buf.p)) : BatchDev();
  uint32_t *d_err = static_cast<uint32_t *>(ws.misc.p);
  unsigned long long *d_tile = reinterpret_cast<unsigned long long *>(static_cast<char *>(ws.misc.p) + 64);
  unsigned long long *d_work = reinterpret_cast<unsigned long long *>(static_cast<char *>(ws.misc.p) + 128);
  unsigned long long *d_sat = d_work + 2;
  DistanceArgs da{};
  da.batch = B;
  da.col_start = static_cast<const uint64_t *>(ws.col_start.p);
  da.col_z = static_cast<const float *>(ws.col_z.p);
  da.err = d_err;
  da.tile_counter = d_tile;
  da.work_counters = o.count_work ? d_work : nullptr;
  da.defer_list = defer_cap > 0 ? static_cast<unsigned long long *>(ws.defer.p) : nullptr;
  da.defer_capacity = defer_cap;
  da.defer_counters = reinterpret_cast<unsigned long long *>(static_cast<char *>(ws.misc.p) + kMiscDeferOffset);
  da.step_budget = L.step_budget;
  da.fault = o.fault_inject;
  GwnInput gi;
  gi.batch = B;
  gi.col_start = static_cast<const uint64_t *>(ws.col_start.p);
  gi.col_z = static_cast<const float *>(ws.col_z.p);
  gi.col_s = static_cast<const int8_t *>(ws.col_s.p);
  gi.band_voxels = o.band_voxels;
  gi.err = d_err;
  gi.gwn_cells = L.gwn_cells;

  bool capturing = false;
  // Inside a capture, an event record must be an external node to time the replay.
  auto rec = [&](cudaEvent_t e) {
    return cudaEventRecordWithFlags(e, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
  };
  auto enqueue = [&]() -> sdfb_status {
    CK(rec(ws.ev[6]));
    {
      NvtxRange r("sdfb prepare");
      CK(cudaMemcpyAsync(ws.batch_buf.p, ws.staging.p, L.bytes, cudaMemcpyHostToDevice, st));
      CK(cudaMemsetAsync(ws.misc.p, 0, 256, st));
    }
    CK(rec(ws.ev[0]));
    if (build) {
      NvtxRange r("sdfb build");
      CK(lbvh_build(B, bvh, ws.build_tmp.p, ws.build_tmp.cap, d_err, st));
    }
    CK(rec(ws.ev[1]));
    if (any_occ) {
      NvtxRange r("sdfb occupancy");
      CK(occupancy_batch(B, nullptr, ws.build_tmp.p, ws.build_tmp.cap, d_sat, ctx->num_sms, st));
    }
    CK(rec(ws.ev[2]));
    if (S.any_cross) {
      NvtxRange r("sdfb crossings");
      CK(parity_columns(B, static_cast<uint64_t *>(ws.col_start.p), static_cast<float *>(ws.col_z.p),
                        static_cast<int8_t *>(ws.col_s.p), S.capacity, ws.par_tmp.p, ws.par_tmp.cap, d_err,
                        ctx->num_sms, st));
    }
    if (K > 0) {
      NvtxRange r("sdfb caps build");
      CK(lbvh_build(CB, caps, ws.caps_tmp.p, ws.caps_tmp.cap, d_err, st));
    }
    CK(rec(ws.ev[3]));
    {
      NvtxRange r("sdfb distance");
      CK(distance_launch(da, L.tile_id, L.stack, ctx->num_sms, st));
    }
    CK(rec(ws.ev[4]));
    if (S.any_gwn) {
      NvtxRange r("sdfb winding number");
      CK(gwn_enqueue(gi, ws.gwn_tmp.p, ctx->num_sms, st));
    }
    CK(rec(ws.ev[5]));
    return SDFB_OK;
  };

  const uint64_t launches0 = launch_count();
  if (use_graph && !o.count_work) {
    // Key: the uploaded tables plus every buffer and option the launch sequence bakes in.
    std::vector<uint8_t> key(static_cast<const uint8_t *>(ws.staging.p),
                             static_cast<const uint8_t *>(ws.staging.p) + L.bytes);
    const void *ptrs[] = {ws.batch_buf.p, ws.bvh.p,  ws.build_tmp.p, ws.par_tmp.p,  ws.col_start.p,
                          ws.col_z.p,     ws.col_s.p, ws.misc.p,      ws.staging.p,  ws.caps_bvh.p,
                          ws.caps_tmp.p,  ws.gwn_tmp.p, ws.defer.p, static_cast<void *>(st)};
    const uint64_t extra[] = {uint64_t(L.tile_id), uint64_t(L.stack), S.capacity, L.bytes, ws.build_tmp.cap,
                              ws.par_tmp.cap, ws.caps_tmp.cap, uint64_t(o.band_voxels * 1e6f),
                              uint64_t(L.step_budget), defer_cap, uint64_t(uint32_t(o.fault_inject))};
    key.insert(key.end(), reinterpret_cast<const uint8_t *>(ptrs), reinterpret_cast<const uint8_t *>(ptrs) + sizeof ptrs);
    key.insert(key.end(), reinterpret_cast<const uint8_t *>(extra),
               reinterpret_cast<const uint8_t *>(extra) + sizeof extra);
    if (!ws.graph || key != ws.graph_key) {
      if (ws.graph) {
        cudaGraphExecDestroy(ws.graph);
        ws.graph = nullptr;
        ws.graph_key.clear();
      }
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      const sdfb_status s = enqueue();
      capturing = false;
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(st, &g);
      if (s != SDFB_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
      }
      if (ce != cudaSuccess) return ctx_cuda(ctx, ce, "cudaStreamEndCapture");
      const cudaError_t ie = cudaGraphInstantiate(&ws.graph, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) {
        ws.graph = nullptr;
        return ctx_cuda(ctx, ie, "cudaGraphInstantiate");
      }
      ws.graph_key.swap(key);
      ws.graph_launches = launch_count() - launches0;
    }
    CK(cudaGraphLaunch(ws.graph, st));
    S.launched = ws.graph_launches;
    S.graphed = true;
  } else {
    const sdfb_status s = enqueue();
    if (s != SDFB_OK) return s;
    S.launched = launch_count() - launches0;
  }
  return SDFB_OK;
}

sdfb_status finish_batch(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, const BatchState &S,
                         const std::vector<PlanMesh> &ms, sdfb_stats *stats) {
  uint32_t *d_err = static_cast<uint32_t *>(ws.misc.p);
  unsigned long long *d_work = reinterpret_cast<unsigned long long *>(static_cast<char *>(ws.misc.p) + 128);
  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err & (kErrBadIndex | kErrNonFinite))
    return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "%s",
                    (h_err & kErrBadIndex) ? "triangle index out of range" : "mesh has a non-finite vertex");
  if (h_err & kErrCrossingOverflow) {
    uint64_t need = 0;
    CK(cudaMemcpy(&need, static_cast<uint64_t *>(ws.col_start.p) + S.total_cols, 8, cudaMemcpyDeviceToHost));
    if (need <= S.capacity) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "crossing list overflow after resize");
    ws.col_capacity_hint = need + need / 4 + 1024;
    return ctx_fail(ctx, SDFB_ERR_BUSY, "crossing list resized; enqueue again");
  }
  if (h_err & kErrStackOverflow)
    return ctx_fail(ctx, SDFB_ERR_OVERFLOW, "BVH traversal stack overflow (depth > %d)", S.stack);
  if (h_err & kErrCorruptTree)
    return ctx_fail(ctx, SDFB_ERR_INTERNAL, "BVH walk met an invalid reference or ran past its step limit");
  if (h_err & kErrDispatch) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "distance tile dispatch timed out");
  if (stats) {
    sdfb_stats sv;
    std::memset(&sv, 0, sizeof sv);
    sv.struct_size = sizeof sv;
    sv.sign_mode_used = ms[0].sign == kSignParity ? SDFB_SIGN_PARITY
                                                  : (ms[0].sign == kSignGwn ? SDFB_SIGN_GWN : SDFB_SIGN_NONE);
    sv.watertight = ms[0].watertight;
    sv.leaf_size_used = S.leaf0;
    sv.tile_used = S.tile_id + 1;
    sv.stack_used = S.stack;
    float ms_p = 0, ms_b = 0, ms_o = 0, ms_s = 0, ms_d = 0, ms_g = 0, tot = 0;
    cudaEventElapsedTime(&ms_p, ws.ev[6], ws.ev[0]);
    cudaEventElapsedTime(&ms_b, ws.ev[0], ws.ev[1]);
    cudaEventElapsedTime(&ms_o, ws.ev[1], ws.ev[2]);
    cudaEventElapsedTime(&ms_s, ws.ev[2], ws.ev[3]);
    cudaEventElapsedTime(&ms_d, ws.ev[3], ws.ev[4]);
    cudaEventElapsedTime(&ms_g, ws.ev[4], ws.ev[5]);
    cudaEventElapsedTime(&tot, ws.ev[6], ws.ev[5]);
    sv.ms_total = tot;
    sv.ms_prepare = ms_p;
    sv.ms_build = ms_b;
    sv.ms_occupancy = ms_o;
    sv.ms_sign = ms_s + ms_g;
    sv.ms_distance = ms_d;
    sv.voxels = S.total_cells;
    sv.triangles = S.total_tris;
    unsigned long long w[5] = {0, 0, 0, 0, 0};
    cudaMemcpy(w, d_work, sizeof w, cudaMemcpyDeviceToHost);
    sv.box_tests = w[0];
    sv.tri_tests = w[1];
    sv.sat_tests = w[2];
    sv.plane_tests = w[3];
    sv.rect_tests = w[4];
    sv.flops_distance = distance_work_flops(S.tile_id, w);
    if (S.any_cross)
      cudaMemcpy(&sv.crossings, static_cast<uint64_t *>(ws.col_start.p) + S.total_cols, 8, cudaMemcpyDeviceToHost);
    if (S.any_gwn) {
      cudaMemcpy(&sv.gwn_fp64_cells, gwn_refine_counter(ws.gwn_tmp.p), 8, cudaMemcpyDeviceToHost);
      cudaMemcpy(&sv.gwn_direct_cells, gwn_direct_counter(ws.gwn_tmp.p), 8, cudaMemcpyDeviceToHost);
    }
    sv.kernel_launches = S.launched;
    sv.graph_replayed = S.graphed ? 1 : 0;
    cudaMemcpy(&sv.tiles_deferred, static_cast<char *>(ws.misc.p) + kMiscDeferOffset, 8, cudaMemcpyDeviceToHost);
    cudaGetLastError();  // a failed statistics read does not fail the bake
    const size_t n = std::min<size_t>(stats->struct_size ? stats->struct_size : sizeof sv, sizeof sv);
    std::memcpy(stats, &sv, n);
  }
  return SDFB_OK;
}

sdfb_status run_batch(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &ms, const sdfb_opts &o, bool use_graph,
                      sdfb_stats *stats) {
  sdfb_opts oo = o;
  for (int attempt = 0; attempt < 4; ++attempt) {
    BatchState S;
    sdfb_status s = enqueue_batch(ctx, ctx->ws, st, ms, oo, use_graph, S);
    if (s != SDFB_OK) return s;
    s = finish_batch(ctx, ctx->ws, st, S, ms, stats);
    if (s == SDFB_ERR_BUSY) continue;  // crossing list resized
    if (s == SDFB_ERR_OVERFLOW && S.stack < 64) {
      oo.stack_depth = 64;  // the tuned shallow stack was too small for this tree
      continue;
    }
    return s;
  }
  return ctx_fail(ctx, SDFB_ERR_INTERNAL, "bake did not settle after retries");
}

// ---------------------------------------------------------------------------------------------
// Resident hierarchies (serving).

size_t resident_bytes(uint64_t tris, bool winding) { return lbvh_bytes(tris, 1, winding); }

sdfb_status build_resident(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, const PlanMesh &p, void *mem,
                           ResidentBvh &out, void *cap_mem, ResidentBvh &cap_out) {
  if (!ws.init()) return ctx_fail(ctx, SDFB_ERR_CUDA, "cannot create events");
  const bool with_caps = p.cT > 0 && cap_mem;
  MeshRec r[2];
  std::memset(r, 0, sizeof r);
  r[0].verts = p.verts;
  r[0].idx = p.idx;
  r[0].num_verts = p.V;
  r[0].num_tris = p.T;
  r[0].leaf_size = std::max(1, std::min(p.leaf > 0 ? p.leaf : ctx->tuned_leaf[bucket_tris(p.T)][bucket_grid(p.grid)], 16));
  r[1].verts = p.cverts;
  r[1].idx = p.cidx;
  r[1].num_verts = p.pV;
  r[1].num_tris = p.cT;
  r[1].leaf_size = 4;
  const uint64_t tables[2][2] = {{0, p.T}, {0, p.cT}};
  const uint64_t zero[2] = {0, 0};
  const size_t bytes = 256 * 6;
  ENSURE(ws.batch_buf, bytes);
  if (!ws.staging.ensure(bytes)) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "pinned staging");
  ENSURE(ws.build_tmp, std::max(lbvh_temp_bytes(p.T, 1), with_caps ? lbvh_temp_bytes(p.cT, 1) : size_t(0)));
  ENSURE(ws.misc, 256);
  char *hs = static_cast<char *>(ws.staging.p);
  std::memset(hs, 0, bytes);
  std::memcpy(hs, &r[0], sizeof(MeshRec));
  std::memcpy(hs + 256, tables[0], 16);
  std::memcpy(hs + 512, zero, 16);
  std::memcpy(hs + 768, &r[1], sizeof(MeshRec));
  std::memcpy(hs + 1024, tables[1], 16);
  CK(cudaMemcpyAsync(ws.batch_buf.p, hs, bytes, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(ws.misc.p, 0, 256, st));
  char *d = static_cast<char *>(ws.batch_buf.p);
  auto one = [&](int off_rec, int off_tab, uint64_t T, void *m, bool areas, ResidentBvh &o) -> sdfb_status {
    BatchDev B;
    B.num_meshes = 1;
    B.recs = reinterpret_cast<const MeshRec *>(d + off_rec);
    B.tri_starts = reinterpret_cast<const uint64_t *>(d + off_tab);
    B.ptri_starts = B.tile_starts = B.gwn_tile_starts = B.cell_starts = reinterpret_cast<const uint64_t *>(d + 512);
    B.total_tris = T;
    BvhDev b;
    lbvh_bind(b, m, T, 1, areas);
    CK(lbvh_build(B, b, ws.build_tmp.p, ws.build_tmp.cap, static_cast<uint32_t *>(ws.misc.p), st));
    o.nodes = b.nodes;
    o.dtris = b.dtris;
    o.tris = b.tris;
    o.leaf_order = b.leaf_order;
    o.node_moment = b.node_moment;
    o.num_nodes = b.num_nodes;
    o.num_inner = b.num_inner;
    o.num_tris = static_cast<int>(T);
    o.root = b.num_inner;  // the single virtual root
    return SDFB_OK;
  };
  sdfb_status s = one(0, 256, p.T, mem, false, out);
  if (s != SDFB_OK) return s;
  if (with_caps && (s = one(768, 1024, p.cT, cap_mem, true, cap_out)) != SDFB_OK) return s;
  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(&h_err, ws.misc.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err & (kErrBadIndex | kErrNonFinite))
    return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "%s",
                    (h_err & kErrBadIndex) ? "triangle index out of range" : "mesh has a non-finite vertex");
  if (h_err) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "hierarchy build failed (%u)", h_err);
  return SDFB_OK;
}
