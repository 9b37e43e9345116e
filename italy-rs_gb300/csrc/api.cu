// C ABI of the bake (include/sdfb.h): context, device workspace, and the plain single-mesh bake.
//
// One bake on a stream (run_bake): reset the error word -> build the BVH (lbvh.cu) -> occupancy
// (occupancy.cu) -> parity crossing lists (parity.cu) or winding-number signs (gwn.cu) ->
// distance with fused sign (distance.cu). CUDA events bracket each stage for the per-stage
// times in sdfb_stats. After the stream drains, the device error word is read: bad indices and
// non-finite vertices become SDFB_ERR_BAD_MESH; a crossing list that outgrew its buffer is rebuilt
// once at its exact size.
//
// Replaces italy::bakeSdf (src/convert/sdf_baker.cpp:137-310), which builds an OptiX context,
// GAS, module, pipeline and SBT on every call and copies the grid back synchronously.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "host_mesh.h"
#include "kernels.h"

using namespace sdfb;

namespace sdfb {
static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace sdfb

// ---------------------------------------------------------------------------------------------
// Context plumbing.

bool DevBuf::ensure(size_t bytes) {
  if (bytes <= cap) return true;
  release();
  const size_t want = std::max<size_t>(bytes + bytes / 8, 4096);
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return false;
  }
  cap = want;
  return true;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

sdfb_status ctx_fail(sdfb_ctx *ctx, sdfb_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return st;
}

sdfb_status ctx_cuda(sdfb_ctx *ctx, cudaError_t e, const char *what) {
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "%s: out of device memory", what);
  return ctx_fail(ctx, SDFB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                                  \
  do {                                                            \
    const cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call);       \
  } while (0)

#define ENSURE(buf, bytes)                                                                       \
  do {                                                                                           \
    if (!(buf).ensure(bytes))                                                                    \
      return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of device memory", \
                      static_cast<size_t>(bytes));                                               \
  } while (0)

bool grid_ok(const sdfb_grid_desc *g) {
  if (!g) return false;
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) return false;
  if (!(g->voxel_size > 0.0f) || !std::isfinite(g->voxel_size)) return false;
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(g->origin[a])) return false;
  const double cells = double(g->nx) * g->ny * g->nz;
  return cells <= double(1ull << 36);
}

GridDev to_dev(const sdfb_grid_desc &g) {
  return GridDev{g.origin[0], g.origin[1], g.origin[2], g.voxel_size, g.nx, g.ny, g.nz};
}

void default_params(uint32_t T, uint64_t cells, int *leaf, int *tile) {
  (void)T;
  (void)cells;
  *leaf = 4;
  *tile = 2;
}

sdfb_opts opts_or_default(const sdfb_opts *o) {
  sdfb_opts r;
  std::memset(&r, 0, sizeof r);
  r.struct_size = sizeof r;
  if (o) std::memcpy(&r, o, std::min<size_t>(sizeof r, o->struct_size ? o->struct_size : sizeof r));
  if (!(r.band_voxels > 0.0f)) r.band_voxels = 1.0f;
  return r;
}

// ---------------------------------------------------------------------------------------------
// One bake on device buffers.

sdfb_status run_bake(sdfb_ctx *ctx, cudaStream_t st, const BakeInput &in, const sdfb_grid_desc &grid,
                     const sdfb_opts &opts, int sign, float *d_dist, uint8_t *d_occ, sdfb_stats *stats) {
  const uint32_t T = in.num_tris;
  const GridDev g = to_dev(grid);
  const uint64_t cells = uint64_t(grid.nx) * grid.ny * grid.nz;
  int leaf = opts.leaf_size, tile = opts.tile;
  int dleaf, dtile;
  default_params(T, cells, &dleaf, &dtile);
  if (leaf <= 0) leaf = dleaf;
  if (tile <= 0 || tile >= tile_shape_count()) tile = (opts.tile == 0) ? dtile : 0;
  leaf = std::max(1, std::min(leaf, 16));
  const bool want_dist = d_dist && !opts.no_distance;
  const bool want_occ = d_occ && !opts.no_occupancy;

  // Workspace.
  MeshDev m;
  m.num_verts = in.num_verts;
  m.num_tris = T;
  m.verts = in.verts;
  m.idx = in.idx;
  const bool moments = want_dist && sign == kSignGwn;
  ENSURE(ctx->mesh, lbvh_mesh_bytes(T, moments));
  lbvh_bind_mesh(m, ctx->mesh.p, moments);
  ctx->gwn_refined = 0;
  ENSURE(ctx->build_tmp, std::max(lbvh_temp_bytes(T), occupancy_temp_bytes(T)));
  ENSURE(ctx->misc, 256);
  uint32_t *d_err = static_cast<uint32_t *>(ctx->misc.p);
  unsigned long long *d_tile = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->misc.p) + 64);
  unsigned long long *d_work = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->misc.p) + 128);
  unsigned long long *d_sat = reinterpret_cast<unsigned long long *>(static_cast<char *>(ctx->misc.p) + 160);
  CK(cudaMemsetAsync(ctx->misc.p, 0, 256, st));

  const size_t ncols = size_t(grid.nx) * grid.ny;
  BakeInput pin = in;  // the mesh whose crossings decide parity (the welded mesh for soups)
  if (in.parity_verts) {
    pin.verts = in.parity_verts;
    pin.idx = in.parity_idx;
    pin.num_verts = in.parity_num_verts;
    pin.num_tris = in.parity_num_tris;
  }
  uint64_t capacity = 0;
  if (want_dist && sign == kSignParity) {
    ENSURE(ctx->par_tmp, parity_temp_bytes(pin.num_tris, grid.nx, grid.ny));
    ENSURE(ctx->col_start, (ncols + 1) * 8);
    capacity = std::max<uint64_t>(ctx->col_capacity_hint, std::max<uint64_t>(4 * ncols, 2 * uint64_t(pin.num_tris)));
    ENSURE(ctx->col_z, capacity * 4);
    capacity = ctx->col_z.cap / 4;
  }

  const uint64_t launches0 = launch_count();
  CK(cudaEventRecord(ctx->ev[0], st));
  CK(lbvh_build(m, leaf, ctx->build_tmp.p, ctx->build_tmp.cap, d_err, st));
  CK(cudaEventRecord(ctx->ev[1], st));
  if (want_occ)
    CK(occupancy_dense(in.verts, in.idx, in.num_verts, T, g, d_occ, ctx->build_tmp.p, ctx->build_tmp.cap, d_sat, st));
  CK(cudaEventRecord(ctx->ev[2], st));
  if (want_dist && sign == kSignParity)
    CK(parity_columns(pin.verts, pin.idx, pin.num_verts, pin.num_tris, g, static_cast<uint64_t *>(ctx->col_start.p),
                      static_cast<float *>(ctx->col_z.p), capacity, ctx->par_tmp.p, ctx->par_tmp.cap, d_err, st));
  CK(cudaEventRecord(ctx->ev[3], st));
  DistanceArgs da{};
  if (want_dist) {
    da.nodes = m.nodes;
    da.tris = m.tris;
    da.num_nodes = static_cast<int>(std::max<uint32_t>(T, 2) - 1);
    da.num_tris = static_cast<int>(T);
    da.g = g;
    da.sign = sign == kSignParity ? kSignParity : kSignNone;
    da.col_start = static_cast<const uint64_t *>(ctx->col_start.p);
    da.col_z = static_cast<const float *>(ctx->col_z.p);
    da.dist = d_dist;
    da.err = d_err;
    da.tile_counter = d_tile;
    da.work_counters = opts.count_work ? d_work : nullptr;
  }
  CK(cudaEventRecord(ctx->ev[4], st));
  if (want_dist) CK(distance_launch(da, tile, ctx->num_sms, st));
  if (want_dist && sign == kSignGwn) {
    CK(cudaEventRecord(ctx->ev[6], st));
    const sdfb_status gs = gwn_apply(ctx, st, m, in, grid, opts, d_dist, d_err);
    if (gs != SDFB_OK) return gs;
  } else {
    CK(cudaEventRecord(ctx->ev[6], st));
  }
  CK(cudaEventRecord(ctx->ev[5], st));

  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err & (kErrBadIndex | kErrNonFinite))
    return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "%s",
                    (h_err & kErrBadIndex) ? "triangle index out of range" : "mesh has a non-finite vertex");
  if (h_err & kErrStackOverflow)
    return ctx_fail(ctx, SDFB_ERR_OVERFLOW, "BVH traversal stack overflow (depth > 64)");
  if (h_err & kErrCorruptTree) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "BVH walk met an invalid reference");
  if (h_err & kErrCrossingOverflow) {
    // Rebuild the crossing list at its exact size, then rerun the distance pass.
    uint64_t need = 0;
    CK(cudaMemcpy(&need, static_cast<uint64_t *>(ctx->col_start.p) + ncols, 8, cudaMemcpyDeviceToHost));
    ctx->col_capacity_hint = need + need / 4;
    ENSURE(ctx->col_z, ctx->col_capacity_hint * 4);
    capacity = ctx->col_z.cap / 4;
    CK(cudaMemsetAsync(d_err, 0, 4, st));
    CK(parity_columns(pin.verts, pin.idx, pin.num_verts, pin.num_tris, g, static_cast<uint64_t *>(ctx->col_start.p),
                      static_cast<float *>(ctx->col_z.p), capacity, ctx->par_tmp.p, ctx->par_tmp.cap, d_err, st));
    da.col_z = static_cast<const float *>(ctx->col_z.p);
    CK(distance_launch(da, tile, ctx->num_sms, st));
    CK(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h_err) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "crossing list overflow after resize");
  }

  if (stats) {
    sdfb_stats s;
    std::memset(&s, 0, sizeof s);
    s.struct_size = sizeof s;
    s.sign_mode_used = sign == kSignParity ? SDFB_SIGN_PARITY : (sign == kSignGwn ? SDFB_SIGN_GWN : SDFB_SIGN_NONE);
    s.watertight = in.watertight;
    s.leaf_size_used = leaf;
    s.tile_used = tile;
    float ms[4], ms_dist = 0, ms_gwn = 0, tot = 0;
    for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&ms[i], ctx->ev[i], ctx->ev[i + 1]);
    cudaEventElapsedTime(&ms_dist, ctx->ev[4], ctx->ev[6]);
    cudaEventElapsedTime(&ms_gwn, ctx->ev[6], ctx->ev[5]);
    cudaEventElapsedTime(&tot, ctx->ev[0], ctx->ev[5]);
    s.ms_total = tot;
    s.ms_build = ms[0];
    s.ms_occupancy = ms[1];
    s.ms_sign = ms[2] + ms[3] + ms_gwn;
    s.ms_distance = ms_dist;
    s.voxels = cells;
    s.triangles = T;
    unsigned long long w[4] = {0, 0, 0, 0};
    cudaMemcpy(w, d_work, 32, cudaMemcpyDeviceToHost);
    s.box_tests = w[0];
    s.tri_tests = w[1];
    s.sat_tests = w[2];
    s.flops_distance = double(w[0]) * kFlopsPointBox + double(w[1]) * kFlopsPointTri;
    s.kernel_launches = launch_count() - launches0;
    s.gwn_fp64_cells = ctx->gwn_refined;
    if (want_dist && sign == kSignParity)
      cudaMemcpy(&s.crossings, static_cast<uint64_t *>(ctx->col_start.p) + ncols, 8, cudaMemcpyDeviceToHost);
    const size_t n = std::min<size_t>(stats->struct_size ? stats->struct_size : sizeof s, sizeof s);
    std::memcpy(stats, &s, n);
  }
  return SDFB_OK;
}

// Resolves AUTO: welds the mesh and runs the watertight test on the host copy.
int resolve_sign(const sdfb_opts &o, const float *h_verts, uint32_t V, const uint32_t *h_idx, uint32_t T,
                 int *watertight_out) {
  *watertight_out = -1;
  switch (o.sign_mode) {
    case SDFB_SIGN_PARITY: return kSignParity;
    case SDFB_SIGN_GWN: return kSignGwn;
    case SDFB_SIGN_NONE: return kSignNone;
    default: break;
  }
  const int w = indexed_mesh_watertight(h_verts, V, h_idx, T);
  *watertight_out = w == 1 ? 1 : 0;
  return w == 1 ? kSignParity : kSignGwn;
}

// ---------------------------------------------------------------------------------------------
// C ABI.

extern "C" {

int32_t sdfb_abi_version(void) { return SDFB_ABI_VERSION; }

sdfb_status sdfb_ctx_create(int32_t device, sdfb_ctx **out) {
  if (!out) return SDFB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return SDFB_ERR_NO_DEVICE;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
    cudaGetLastError();
    return SDFB_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess) return SDFB_ERR_NO_DEVICE;
  sdfb_ctx *ctx = new sdfb_ctx();
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return SDFB_ERR_CUDA;
  }
  for (auto &e : ctx->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete ctx;
      return SDFB_ERR_CUDA;
    }
  *out = ctx;
  return SDFB_OK;
}

void sdfb_ctx_destroy(sdfb_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
}

const char *sdfb_last_error(const sdfb_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

sdfb_status sdfb_ctx_trim(sdfb_ctx *ctx) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->release_all();
  return SDFB_OK;
}

uint64_t sdfb_ctx_device_bytes(const sdfb_ctx *ctx) { return ctx ? ctx->device_bytes() : 0; }

sdfb_status sdfb_grid_from_bounds_res(const float bmin[3], const float bmax[3], int32_t resolution,
                                      sdfb_grid_desc *out) {
  if (!bmin || !bmax || !out) return SDFB_ERR_INVALID_ARGUMENT;
  // sdf_baker.cpp:139-148, FP32 in the reference's operation order.
  const float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  float longest = ex;
  if (longest < ey) longest = ey;
  if (longest < ez) longest = ez;
  if (longest < 1e-6f) longest = 1e-6f;
  const float voxel = longest / static_cast<float>(resolution > 1 ? resolution : 1);
  const float pad = voxel * 2.0f;
  const float pad2 = voxel * 2.0f * 2.0f;
  const float e[3] = {ex, ey, ez};
  int32_t n[3];
  for (int a = 0; a < 3; ++a) {
    out->origin[a] = bmin[a] - pad;
    const float q = std::ceil((e[a] + pad2) / voxel);
    if (!(q < 2147483000.0f)) return SDFB_ERR_INVALID_ARGUMENT;
    n[a] = static_cast<int32_t>(q) + 1;
  }
  out->voxel_size = voxel;
  out->nx = n[0];
  out->ny = n[1];
  out->nz = n[2];
  return SDFB_OK;
}

sdfb_status sdfb_bake_device(sdfb_ctx *ctx, const float *d_verts, uint32_t num_verts, const uint32_t *d_idx,
                             uint32_t num_tris, const sdfb_grid_desc *grid, const sdfb_opts *opts, float *d_dist_out,
                             uint8_t *d_occ_out, void *stream, sdfb_stats *stats) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!d_verts || !d_idx || !grid_ok(grid))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null mesh pointer or invalid grid");
  if (num_tris == 0 || num_verts == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh has no triangles");
  cudaSetDevice(ctx->device);
  const sdfb_opts o = opts_or_default(opts);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  int watertight = -1;
  int sign;
  if (o.sign_mode == SDFB_SIGN_AUTO) {
    std::vector<float> hv(size_t(num_verts) * 3);
    std::vector<uint32_t> hi(size_t(num_tris) * 3);
    CK(cudaMemcpyAsync(hv.data(), d_verts, hv.size() * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hi.data(), d_idx, hi.size() * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    sign = resolve_sign(o, hv.data(), num_verts, hi.data(), num_tris, &watertight);
  } else {
    sign = resolve_sign(o, nullptr, 0, nullptr, 0, &watertight);
  }
  BakeInput in{d_verts, d_idx, num_verts, num_tris, nullptr, nullptr, 0, 0, watertight};
  return run_bake(ctx, st, in, *grid, o, sign, d_dist_out, d_occ_out, stats);
}

sdfb_status sdfb_bake(sdfb_ctx *ctx, const float *verts, uint32_t num_verts, const uint32_t *idx, uint32_t num_tris,
                      const sdfb_grid_desc *grid, const sdfb_opts *opts, float *dist_out, uint8_t *occ_out,
                      sdfb_stats *stats) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!verts || !idx || !grid_ok(grid))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null mesh pointer or invalid grid");
  if (num_tris == 0 || num_verts == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh has no triangles");
  cudaSetDevice(ctx->device);
  const sdfb_opts o = opts_or_default(opts);
  int watertight = -1;
  const int sign = resolve_sign(o, verts, num_verts, idx, num_tris, &watertight);
  if (watertight == -1 && o.sign_mode == SDFB_SIGN_AUTO)
    return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "triangle index out of range");
  const cudaStream_t st = ctx->stream;
  const uint64_t cells = uint64_t(grid->nx) * grid->ny * grid->nz;
  ENSURE(ctx->in_verts, size_t(num_verts) * 12);
  ENSURE(ctx->in_idx, size_t(num_tris) * 12);
  const bool want_dist = dist_out && !o.no_distance, want_occ = occ_out && !o.no_occupancy;
  if (want_dist) ENSURE(ctx->out_dist, cells * 4);
  if (want_occ) ENSURE(ctx->out_occ, cells);
  CK(cudaMemcpyAsync(ctx->in_verts.p, verts, size_t(num_verts) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, idx, size_t(num_tris) * 12, cudaMemcpyHostToDevice, st));
  BakeInput in{static_cast<const float *>(ctx->in_verts.p), static_cast<const uint32_t *>(ctx->in_idx.p), num_verts,
               num_tris, nullptr, nullptr, 0, 0, watertight};
  sdfb_status s = run_bake(ctx, st, in, *grid, o, sign, want_dist ? static_cast<float *>(ctx->out_dist.p) : nullptr,
                           want_occ ? static_cast<uint8_t *>(ctx->out_occ.p) : nullptr, stats);
  if (s != SDFB_OK) return s;
  if (want_dist) CK(cudaMemcpyAsync(dist_out, ctx->out_dist.p, cells * 4, cudaMemcpyDeviceToHost, st));
  if (want_occ) CK(cudaMemcpyAsync(occ_out, ctx->out_occ.p, cells, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

sdfb_status sdfb_bake_soup(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                           const float bounds_max[3], int32_t resolution, const sdfb_opts *opts,
                           sdfb_grid_desc *grid_out, float *dist_out, uint8_t *occ_out, sdfb_stats *stats) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!positions || !bounds_min || !bounds_max || !grid_out)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  sdfb_status s = sdfb_grid_from_bounds_res(bounds_min, bounds_max, resolution, grid_out);
  if (s != SDFB_OK) return ctx_fail(ctx, s, "grid too large for the bounds and resolution");
  if (!dist_out && !occ_out) return SDFB_OK;
  if (!grid_ok(grid_out)) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "grid too large");
  if (num_tris == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh has no triangles");
  cudaSetDevice(ctx->device);
  sdfb_opts o = opts_or_default(opts);
  const uint32_t V = 3 * num_tris;
  // Weld for the watertight gate and for a crack-free parity mesh (first occurrence kept).
  std::vector<uint32_t> welded(V);
  const uint32_t U = weld_positions(positions, V, bounds_min, bounds_max, welded.data());
  std::vector<float> uniq(size_t(U) * 3);
  std::vector<uint8_t> seen(U, 0);
  for (uint32_t i = 0; i < V; ++i)
    if (!seen[welded[i]]) {
      seen[welded[i]] = 1;
      std::memcpy(&uniq[size_t(welded[i]) * 3], positions + size_t(i) * 3, 12);
    }
  int watertight = -1;
  int sign;
  if (o.sign_mode == SDFB_SIGN_AUTO) {
    uint64_t b, m;
    watertight = watertight_flag(welded.data(), num_tris, &b, &m);
    sign = watertight == 1 ? kSignParity : kSignGwn;
  } else {
    sign = resolve_sign(o, nullptr, 0, nullptr, 0, &watertight);
  }
  std::vector<uint32_t> ident(V);
  for (uint32_t i = 0; i < V; ++i) ident[i] = i;
  const cudaStream_t st = ctx->stream;
  const uint64_t cells = uint64_t(grid_out->nx) * grid_out->ny * grid_out->nz;
  ENSURE(ctx->in_verts, size_t(V) * 12);
  ENSURE(ctx->in_idx, size_t(V) * 4);
  ENSURE(ctx->in_verts2, size_t(U) * 12);
  ENSURE(ctx->in_idx2, size_t(V) * 4);
  const bool want_dist = dist_out && !o.no_distance, want_occ = occ_out && !o.no_occupancy;
  if (want_dist) ENSURE(ctx->out_dist, cells * 4);
  if (want_occ) ENSURE(ctx->out_occ, cells);
  CK(cudaMemcpyAsync(ctx->in_verts.p, positions, size_t(V) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, ident.data(), size_t(V) * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_verts2.p, uniq.data(), size_t(U) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx2.p, welded.data(), size_t(V) * 4, cudaMemcpyHostToDevice, st));
  BakeInput in{static_cast<const float *>(ctx->in_verts.p),
               static_cast<const uint32_t *>(ctx->in_idx.p),
               V,
               num_tris,
               static_cast<const float *>(ctx->in_verts2.p),
               static_cast<const uint32_t *>(ctx->in_idx2.p),
               U,
               num_tris,
               watertight};
  s = run_bake(ctx, st, in, *grid_out, o, sign, want_dist ? static_cast<float *>(ctx->out_dist.p) : nullptr,
               want_occ ? static_cast<uint8_t *>(ctx->out_occ.p) : nullptr, stats);
  if (s != SDFB_OK) return s;
  if (want_dist) CK(cudaMemcpyAsync(dist_out, ctx->out_dist.p, cells * 4, cudaMemcpyDeviceToHost, st));
  if (want_occ) CK(cudaMemcpyAsync(occ_out, ctx->out_occ.p, cells, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

sdfb_status sdfb_weld(sdfb_ctx *ctx, const float *positions, uint32_t num_positions, const float bounds_min[3],
                      const float bounds_max[3], uint32_t *welded_out, uint32_t *num_unique) {
  if (!positions || !bounds_min || !bounds_max || !welded_out || !num_unique)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  *num_unique = weld_positions(positions, num_positions, bounds_min, bounds_max, welded_out);
  return SDFB_OK;
}

sdfb_status sdfb_is_watertight(sdfb_ctx *ctx, const uint32_t *welded_idx, uint32_t num_tris, int32_t *watertight_out,
                               uint64_t *boundary_edges, uint64_t *nonmanifold_edges) {
  if (!welded_idx || !watertight_out) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  uint64_t b = 0, m = 0;
  const int w = watertight_flag(welded_idx, num_tris, &b, &m);
  *watertight_out = w == 1 ? 1 : 0;
  if (boundary_edges) *boundary_edges = b;
  if (nonmanifold_edges) *nonmanifold_edges = m;
  return SDFB_OK;
}

sdfb_status sdfb_voxelize_sparse(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                                 const float bounds_max[3], int32_t resolution, int32_t *cells_out, uint64_t cap,
                                 uint64_t *count, float origin_out[3], float *voxel_out) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (!positions || !bounds_min || !bounds_max || !count || (cap && !cells_out) || resolution < 1)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument or resolution < 1");
  if (uint64_t(resolution) * resolution * resolution >= (1ull << 32))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "resolution too large for the sparse voxelizer (max 1625)");
  cudaSetDevice(ctx->device);
  // voxelize.cpp:54-57: origin = boundsMin (no pad), voxel = longest / res, cells clamped to res - 1.
  const float ex = bounds_max[0] - bounds_min[0], ey = bounds_max[1] - bounds_min[1],
              ez = bounds_max[2] - bounds_min[2];
  float longest = ex;
  if (longest < ey) longest = ey;
  if (longest < ez) longest = ez;
  if (longest < 1e-6f) longest = 1e-6f;
  const float voxel = longest / static_cast<float>(resolution);
  sdfb_grid_desc g;
  g.origin[0] = bounds_min[0];
  g.origin[1] = bounds_min[1];
  g.origin[2] = bounds_min[2];
  g.voxel_size = voxel;
  g.nx = g.ny = g.nz = resolution;
  if (origin_out) std::memcpy(origin_out, g.origin, 12);
  if (voxel_out) *voxel_out = voxel;
  *count = 0;
  if (num_tris == 0) return SDFB_OK;
  const uint32_t V = 3 * num_tris;
  const size_t cells = size_t(resolution) * resolution * resolution;
  const cudaStream_t st = ctx->stream;
  std::vector<uint32_t> ident(V);
  for (uint32_t i = 0; i < V; ++i) ident[i] = i;
  ENSURE(ctx->in_verts, size_t(V) * 12);
  ENSURE(ctx->in_idx, size_t(V) * 4);
  ENSURE(ctx->out_occ, cells);
  ENSURE(ctx->first_tri, cells * 4);
  ENSURE(ctx->build_tmp, occupancy_temp_bytes(num_tris));
  CK(cudaMemcpyAsync(ctx->in_verts.p, positions, size_t(V) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, ident.data(), size_t(V) * 4, cudaMemcpyHostToDevice, st));
  CK(occupancy_dense_first(static_cast<const float *>(ctx->in_verts.p), static_cast<const uint32_t *>(ctx->in_idx.p),
                           V, num_tris, to_dev(g), static_cast<uint8_t *>(ctx->out_occ.p),
                           static_cast<uint32_t *>(ctx->first_tri.p), ctx->build_tmp.p, ctx->build_tmp.cap, st));
  ENSURE(ctx->par_tmp, sparse_temp_bytes(cells, 0));
  uint64_t total = 0;
  CK(sparse_count(static_cast<const uint8_t *>(ctx->out_occ.p), cells, ctx->par_tmp.p, ctx->par_tmp.cap, &total, st));
  *count = total;
  if (total == 0) return SDFB_OK;
  ENSURE(ctx->par_tmp, sparse_temp_bytes(cells, total));
  ENSURE(ctx->col_z, total * 4);
  int bits = 1;
  while (bits < 32 && (uint64_t(1) << bits) < num_tris) ++bits;
  CK(sparse_emit(static_cast<const uint8_t *>(ctx->out_occ.p), static_cast<const uint32_t *>(ctx->first_tri.p), cells,
                 total, bits, ctx->par_tmp.p, ctx->par_tmp.cap, static_cast<uint32_t *>(ctx->col_z.p), st));
  const uint64_t n = std::min<uint64_t>(total, cap);
  std::vector<uint32_t> lin(n);
  if (n) CK(cudaMemcpyAsync(lin.data(), ctx->col_z.p, n * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const uint64_t r = uint64_t(resolution);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t c = lin[i];
    cells_out[3 * i] = static_cast<int32_t>(c % r);
    cells_out[3 * i + 1] = static_cast<int32_t>((c / r) % r);
    cells_out[3 * i + 2] = static_cast<int32_t>(c / (r * r));
  }
  return SDFB_OK;
}

}  // extern "C"
