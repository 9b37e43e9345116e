// C ABI of the bake (include/sdfb.h): context, buffers and every entry point. Each entry point
// resolves sign modes on the host (the reference's weld + watertight gate,
// src/io/mesh_weld.cpp:26-48 and src/io/mesh_validate.cpp:21-59), caps non-watertight meshes for
// the winding number, places inputs and outputs in device memory and hands the meshes to
// run_batch (orchestrate.cu).
//
// Replaces italy::bakeSdf (src/convert/sdf_baker.cpp:137-310) and italy::voxelizeMesh
// (src/convert/voxelize.cpp:52-107).
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
// Buffers, errors, context.

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

bool PinBuf::ensure(size_t bytes) {
  if (bytes <= cap) return true;
  release();
  const size_t want = std::max<size_t>(bytes + bytes / 8, 4096);
  if (cudaMallocHost(&p, want) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return false;
  }
  cap = want;
  return true;
}

void PinBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
}

sdfb_ctx::~sdfb_ctx() {
  if (stream) cudaStreamDestroy(stream);
}

DevBuf *sdfb_ctx::all_bufs(int i) {
  DevBuf *b[] = {&in_verts, &in_idx,   &in_verts2, &in_idx2,    &in_caps,   &in_capidx, &out_dist,
                 &out_occ,  &first_tri, &sparse_tmp, &sparse_out, &mat_rec,  &mat_in,    &mat_tri,
                 &hit_keys, &hit_vals,  &hit_alt,   &mat_cells, &cons_grid, &cons_io,    &weld_tmp,
                 &caps_tmp, &caps_misc};
  return i < int(sizeof b / sizeof b[0]) ? b[i] : nullptr;
}

void sdfb_ctx::release_all() {
  for (int i = 0; DevBuf *b = all_bufs(i); ++i) b->release();
  ws.release();
  staging_small.release();
}

uint64_t sdfb_ctx::device_bytes() const {
  uint64_t s = ws.bytes();
  for (int i = 0; const DevBuf *b = const_cast<sdfb_ctx *>(this)->all_bufs(i); ++i) s += b->cap;
  return s;
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

sdfb_opts opts_or_default(const sdfb_opts *o) {
  sdfb_opts r;
  std::memset(&r, 0, sizeof r);
  r.struct_size = sizeof r;
  if (o) std::memcpy(&r, o, std::min<size_t>(sizeof r, o->struct_size ? o->struct_size : sizeof r));
  if (!(r.band_voxels > 0.0f)) r.band_voxels = 1.0f;
  return r;
}

// ---------------------------------------------------------------------------------------------
// Host-side preparation.

namespace {

// Sign of one mesh from the options and, for AUTO, the watertight gate on the host copy.
// Returns -1 when an index is out of range (AUTO only).
int resolve_sign(const sdfb_opts &o, const float *hv, uint32_t V, const uint32_t *hi, uint32_t T, int *watertight) {
  *watertight = -1;
  switch (o.sign_mode) {
    case SDFB_SIGN_PARITY: return kSignParity;
    case SDFB_SIGN_GWN: return kSignGwn;
    case SDFB_SIGN_NONE: return kSignNone;
    default: break;
  }
  const int w = indexed_mesh_watertight(hv, V, hi, T);
  if (w == -2) return -1;
  *watertight = w == 1 ? 1 : 0;
  return w == 1 ? kSignParity : kSignGwn;
}


// The device address of a page-locked host buffer (cudaHostAlloc, cudaHostRegister, a pinned
// tensor), or null for pageable memory. The distance kernel writes such a distance output
// directly: the GPU reaches host memory coherently over NVLink-C2C, so the grid streams to the
// host while the bake computes instead of in a copy after it. Winding-number meshes keep device
// outputs, because their band pass reads the distances back; occupancy is always copied (its
// clear writes single bytes).
void *mapped_host(void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

}  // namespace

sdfb_status device_caps(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &ms, bool every_gwn) {
  // Regions sized for the most caps a mesh can have (3T boundary half-edges, 3T loops).
  size_t nv = 0, np = 0, tmax = 0, ng = 0;
  for (const PlanMesh &p : ms)
    if (p.sign == kSignGwn && (p.dist || every_gwn)) {
      const size_t V = p.pverts ? p.pV : p.V, T = p.pverts ? p.pT : p.T;
      nv += 3 * (V + 3 * T);
      np += 3 * (T + 3 * T);
      tmax = std::max<size_t>(tmax, T);
      ++ng;
    }
  if (ng == 0) return SDFB_OK;
  // Cap vertices are numbered V + loop and half-edges are labelled by 32-bit indices.
  for (const PlanMesh &p : ms)
    if (p.sign == kSignGwn && (p.dist || every_gwn)) {
      const uint64_t V = p.pverts ? p.pV : p.V, T = p.pverts ? p.pT : p.T;
      if (V + 3 * T >= (uint64_t(1) << 32))
        return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "mesh too large for winding-number caps (V + 3T >= 2^32)");
    }
  ENSURE(ctx->in_caps, nv * 4);
  ENSURE(ctx->in_capidx, np * 4);
  ENSURE(ctx->caps_tmp, caps_temp_bytes(tmax));
  ENSURE(ctx->caps_misc, 256 + ng * 16);
  uint32_t *d_err = static_cast<uint32_t *>(ctx->caps_misc.p);
  uint64_t *d_tot = reinterpret_cast<uint64_t *>(static_cast<char *>(ctx->caps_misc.p) + 256);
  CK(cudaMemsetAsync(d_err, 0, 4, st));
  size_t ov = 0, op = 0, k = 0;
  std::vector<size_t> at(ms.size(), 0);
  for (size_t m = 0; m < ms.size(); ++m) {
    PlanMesh &p = ms[m];
    if (p.sign != kSignGwn || !(p.dist || every_gwn)) continue;
    const float *bv = p.pverts ? p.pverts : p.verts;
    const uint32_t *bi = p.pverts ? p.pidx : p.idx;
    const uint32_t V = p.pverts ? p.pV : p.V, T = p.pverts ? p.pT : p.T;
    float *dv = static_cast<float *>(ctx->in_caps.p) + ov;
    uint32_t *dp = static_cast<uint32_t *>(ctx->in_capidx.p) + op;
    CK(cudaMemcpyAsync(dv, bv, size_t(V) * 12, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(dp, bi, size_t(T) * 12, cudaMemcpyDeviceToDevice, st));
    CK(caps_device(bv, V, bi, T, ctx->caps_tmp.p, ctx->caps_tmp.cap, dv + 3 * size_t(V), dp + 3 * size_t(T),
                   d_tot + 2 * k, d_err, ctx->num_sms, st));
    p.pverts = p.cverts = dv;
    p.pidx = dp;
    p.cidx = dp + 3 * size_t(T);
    p.pV = V;
    p.pT = T;
    at[m] = k++;
    ov += 3 * (size_t(V) + 3 * size_t(T));
    op += 3 * (size_t(T) + 3 * size_t(T));
  }
  std::vector<uint64_t> tot(2 * ng);
  uint32_t h_err = 0;
  CK(cudaMemcpyAsync(tot.data(), d_tot, tot.size() * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err & kErrBadIndex) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "triangle index out of range");
  if (h_err) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "boundary loops of a winding-number mesh do not close");
  for (size_t m = 0; m < ms.size(); ++m) {
    PlanMesh &p = ms[m];
    if (p.sign != kSignGwn || !(p.dist || every_gwn)) continue;
    const uint64_t caps = tot[2 * at[m]], loops = tot[2 * at[m] + 1];
    p.pV += static_cast<uint32_t>(loops);
    p.pT += static_cast<uint32_t>(caps);
    p.cT = static_cast<uint32_t>(caps);
  }
  return SDFB_OK;
}

sdfb_status device_sign(sdfb_ctx *ctx, const sdfb_opts &o, const float *d_verts, uint32_t V, const uint32_t *d_idx,
                        uint32_t T, cudaStream_t st, int *sign, int *watertight) {
  *watertight = -1;
  if (o.sign_mode != SDFB_SIGN_AUTO) {
    *sign = resolve_sign(o, nullptr, 0, nullptr, 0, watertight);
    return SDFB_OK;
  }
  ENSURE(ctx->weld_tmp, indexed_gate_temp_bytes(V, T));
  int w = 0;
  CK(indexed_watertight_device(d_verts, V, d_idx, T, ctx->weld_tmp.p, ctx->weld_tmp.cap, &w, ctx->num_sms, st));
  if (w == -2) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "triangle index out of range");
  *watertight = w == 1 ? 1 : 0;
  *sign = w == 1 ? kSignParity : kSignGwn;
  return SDFB_OK;
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
  if (!ctx->ws.init()) {
    delete ctx;
    return SDFB_ERR_CUDA;
  }
  load_tuning(ctx);
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
  std::vector<PlanMesh> ms(1);
  PlanMesh &p = ms[0];
  p.verts = d_verts;
  p.idx = d_idx;
  p.V = num_verts;
  p.T = num_tris;
  p.grid = *grid;
  p.dist = o.no_distance ? nullptr : d_dist_out;
  p.occ = o.no_occupancy ? nullptr : d_occ_out;
  sdfb_status s = device_sign(ctx, o, d_verts, num_verts, d_idx, num_tris, st, &p.sign, &p.watertight);
  if (s != SDFB_OK) return s;
  if ((s = device_caps(ctx, st, ms)) != SDFB_OK) return s;
  return run_batch(ctx, st, ms, o, false, stats);
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
  const cudaStream_t st = ctx->stream;
  std::vector<PlanMesh> ms(1);
  PlanMesh &p = ms[0];
  const uint64_t cells = uint64_t(grid->nx) * grid->ny * grid->nz;
  const bool want_dist = dist_out && !o.no_distance, want_occ = occ_out && !o.no_occupancy;
  ENSURE(ctx->in_verts, size_t(num_verts) * 12);
  ENSURE(ctx->in_idx, size_t(num_tris) * 12);
  if (want_dist) ENSURE(ctx->out_dist, cells * 4);
  if (want_occ) ENSURE(ctx->out_occ, cells);
  CK(cudaMemcpyAsync(ctx->in_verts.p, verts, size_t(num_verts) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, idx, size_t(num_tris) * 12, cudaMemcpyHostToDevice, st));
  sdfb_status sg = device_sign(ctx, o, static_cast<const float *>(ctx->in_verts.p), num_verts,
                               static_cast<const uint32_t *>(ctx->in_idx.p), num_tris, st, &p.sign, &p.watertight);
  if (sg != SDFB_OK) return sg;
  p.verts = static_cast<const float *>(ctx->in_verts.p);
  p.idx = static_cast<const uint32_t *>(ctx->in_idx.p);
  p.V = num_verts;
  p.T = num_tris;
  p.grid = *grid;
  float *const direct_dist =
      (want_dist && p.sign != kSignGwn) ? static_cast<float *>(mapped_host(dist_out)) : nullptr;
  uint8_t *const direct_occ = nullptr;
  p.dist = want_dist ? (direct_dist ? direct_dist : static_cast<float *>(ctx->out_dist.p)) : nullptr;
  p.occ = want_occ ? (direct_occ ? direct_occ : static_cast<uint8_t *>(ctx->out_occ.p)) : nullptr;
  sdfb_status s = device_caps(ctx, st, ms);
  if (s != SDFB_OK) return s;
  s = run_batch(ctx, st, ms, o, false, stats);
  if (s != SDFB_OK) return s;
  if (want_dist && !direct_dist)
    CK(cudaMemcpyAsync(dist_out, ctx->out_dist.p, cells * 4, cudaMemcpyDeviceToHost, st));
  if (want_occ && !direct_occ) CK(cudaMemcpyAsync(occ_out, ctx->out_occ.p, cells, cudaMemcpyDeviceToHost, st));
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
  const sdfb_opts o = opts_or_default(opts);
  const uint32_t V = 3 * num_tris;
  const cudaStream_t st = ctx->stream;
  const uint64_t cells = uint64_t(grid_out->nx) * grid_out->ny * grid_out->nz;
  const bool want_dist = dist_out && !o.no_distance, want_occ = occ_out && !o.no_occupancy;
  std::vector<uint32_t> ident(V);
  for (uint32_t i = 0; i < V; ++i) ident[i] = i;
  ENSURE(ctx->in_verts, size_t(V) * 12);
  ENSURE(ctx->in_idx, size_t(V) * 4);
  if (want_dist) ENSURE(ctx->out_dist, cells * 4);
  if (want_occ) ENSURE(ctx->out_occ, cells);
  CK(cudaMemcpyAsync(ctx->in_verts.p, positions, size_t(V) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, ident.data(), size_t(V) * 4, cudaMemcpyHostToDevice, st));
  // Weld on the device (first occurrence kept) for the watertight gate and for a crack-free
  // crossing mesh: welded indices in in_idx2, unique positions in in_verts2.
  ENSURE(ctx->in_idx2, size_t(V) * 4);
  ENSURE(ctx->in_verts2, size_t(V) * 12);
  ENSURE(ctx->weld_tmp, std::max(weld_temp_bytes(V) + size_t(V) * 4 + 256, watertight_temp_bytes(num_tris)));
  uint32_t *d_welded = static_cast<uint32_t *>(ctx->in_idx2.p);
  uint32_t *d_first = reinterpret_cast<uint32_t *>(static_cast<char *>(ctx->weld_tmp.p) + weld_temp_bytes(V));
  uint32_t U = 0;
  CK(weld_device(static_cast<const float *>(ctx->in_verts.p), V, weld_cell(bounds_min, bounds_max), d_welded, d_first,
                 ctx->weld_tmp.p, weld_temp_bytes(V), &U, ctx->num_sms, st));
  CK(gather_unique(static_cast<const float *>(ctx->in_verts.p), d_first, U, static_cast<float *>(ctx->in_verts2.p),
                   ctx->num_sms, st));
  std::vector<PlanMesh> ms(1);
  PlanMesh &p = ms[0];
  if (o.sign_mode == SDFB_SIGN_AUTO) {
    uint64_t b = 0, m = 0;
    CK(watertight_device(d_welded, num_tris, U, ctx->weld_tmp.p, ctx->weld_tmp.cap, &b, &m, ctx->num_sms, st));
    p.watertight = (b == 0 && m == 0) ? 1 : 0;
    p.sign = p.watertight ? kSignParity : kSignGwn;
  } else {
    p.sign = resolve_sign(o, nullptr, 0, nullptr, 0, &p.watertight);
  }
  p.verts = static_cast<const float *>(ctx->in_verts.p);
  p.idx = static_cast<const uint32_t *>(ctx->in_idx.p);
  p.V = V;
  p.T = num_tris;
  p.grid = *grid_out;
  float *const direct_dist =
      (want_dist && p.sign != kSignGwn) ? static_cast<float *>(mapped_host(dist_out)) : nullptr;
  p.dist = want_dist ? (direct_dist ? direct_dist : static_cast<float *>(ctx->out_dist.p)) : nullptr;
  p.occ = want_occ ? static_cast<uint8_t *>(ctx->out_occ.p) : nullptr;
  if (p.sign == kSignGwn && want_dist) {
    // the caps close the welded mesh
    p.pverts = static_cast<const float *>(ctx->in_verts2.p);
    p.pidx = d_welded;
    p.pV = U;
    p.pT = num_tris;
    if ((s = device_caps(ctx, st, ms)) != SDFB_OK) return s;
  } else if (p.sign == kSignParity && want_dist) {
    p.pverts = static_cast<const float *>(ctx->in_verts2.p);
    p.pidx = static_cast<const uint32_t *>(ctx->in_idx2.p);
    p.pV = U;
    p.pT = num_tris;
  }
  s = run_batch(ctx, st, ms, o, false, stats);
  if (s != SDFB_OK) return s;
  if (want_dist && !direct_dist)
    CK(cudaMemcpyAsync(dist_out, ctx->out_dist.p, cells * 4, cudaMemcpyDeviceToHost, st));
  if (want_occ) CK(cudaMemcpyAsync(occ_out, ctx->out_occ.p, cells, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

sdfb_status sdfb_weld_device(sdfb_ctx *ctx, const float *d_positions, uint32_t num_positions,
                             const float bounds_min[3], const float bounds_max[3], uint32_t *d_welded_out,
                             uint32_t *num_unique, void *stream) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if ((num_positions && (!d_positions || !d_welded_out)) || !bounds_min || !bounds_max || !num_unique)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  cudaSetDevice(ctx->device);
  const cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  ENSURE(ctx->weld_tmp, weld_temp_bytes(num_positions));
  CK(weld_device(d_positions, num_positions, weld_cell(bounds_min, bounds_max), d_welded_out, nullptr, ctx->weld_tmp.p,
                 ctx->weld_tmp.cap, num_unique, ctx->num_sms, st));
  return SDFB_OK;
}

sdfb_status sdfb_is_watertight_device(sdfb_ctx *ctx, const uint32_t *d_welded_idx, uint32_t num_tris,
                                      int32_t *watertight_out, uint64_t *boundary_edges, uint64_t *nonmanifold_edges,
                                      void *stream) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if ((num_tris && !d_welded_idx) || !watertight_out) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  cudaSetDevice(ctx->device);
  const cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  uint64_t b = 0, m = 0;
  if (num_tris) {
    ENSURE(ctx->weld_tmp, watertight_temp_bytes(num_tris));
    CK(watertight_device(d_welded_idx, num_tris, 0, ctx->weld_tmp.p, ctx->weld_tmp.cap, &b, &m,
                         ctx->num_sms, st));
  }
  *watertight_out = (num_tris && b == 0 && m == 0) ? 1 : 0;  // no triangles: not watertight
  if (boundary_edges) *boundary_edges = b;
  if (nonmanifold_edges) *nonmanifold_edges = m;
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
  return voxelize_sparse_run(ctx, positions, num_tris, bounds_min, bounds_max, resolution, cells_out, cap, count,
                             origin_out, voxel_out, nullptr, nullptr);
}

}  // extern "C"

sdfb_status voxelize_sparse_run(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                                const float bounds_max[3], int32_t resolution, int32_t *cells_out, uint64_t cap,
                                uint64_t *count, float origin_out[3], float *voxel_out, const uint32_t **d_list,
                                sdfb_grid_desc *grid_out) {
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
  if (grid_out) *grid_out = g;
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
  ENSURE(ctx->sparse_tmp, std::max(occupancy_temp_bytes(num_tris), sparse_temp_bytes(cells, 0)));
  CK(cudaMemcpyAsync(ctx->in_verts.p, positions, size_t(V) * 12, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->in_idx.p, ident.data(), size_t(V) * 4, cudaMemcpyHostToDevice, st));
  // a batch of one mesh with an occupancy output only
  MeshRec r;
  std::memset(&r, 0, sizeof r);
  r.verts = static_cast<const float *>(ctx->in_verts.p);
  r.idx = static_cast<const uint32_t *>(ctx->in_idx.p);
  r.num_verts = V;
  r.num_tris = num_tris;
  r.occ = static_cast<uint8_t *>(ctx->out_occ.p);
  r.g = to_dev(g);
  r.leaf_size = 1;
  const uint64_t tables[2][2] = {{0, num_tris}, {0, cells}};
  const uint64_t zero[2] = {0, 0};
  const size_t bytes = 256 * 4;
  ENSURE(ctx->sparse_out, bytes);
  if (!ctx->staging_small.ensure(bytes)) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "pinned staging");
  char *hs = static_cast<char *>(ctx->staging_small.p);
  std::memcpy(hs, &r, sizeof r);
  std::memcpy(hs + 256, tables[0], 16);
  std::memcpy(hs + 512, tables[1], 16);
  std::memcpy(hs + 768, zero, 16);
  CK(cudaMemcpyAsync(ctx->sparse_out.p, hs, bytes, cudaMemcpyHostToDevice, st));
  char *d = static_cast<char *>(ctx->sparse_out.p);
  BatchDev B;
  B.num_meshes = 1;
  B.recs = reinterpret_cast<const MeshRec *>(d);
  B.tri_starts = reinterpret_cast<const uint64_t *>(d + 256);
  B.cell_starts = reinterpret_cast<const uint64_t *>(d + 512);
  B.ptri_starts = B.tile_starts = B.gwn_tile_starts = reinterpret_cast<const uint64_t *>(d + 768);
  B.total_tris = num_tris;
  B.total_cells = cells;
  CK(occupancy_batch(B, static_cast<uint32_t *>(ctx->first_tri.p), ctx->sparse_tmp.p, ctx->sparse_tmp.cap, nullptr,
                     ctx->num_sms, st));
  uint64_t total = 0;
  CK(sparse_count(static_cast<const uint8_t *>(ctx->out_occ.p), cells, ctx->sparse_tmp.p, ctx->sparse_tmp.cap, &total,
                  st));
  *count = total;
  if (total == 0) return SDFB_OK;
  ENSURE(ctx->sparse_tmp, sparse_temp_bytes(cells, total));
  ENSURE(ctx->out_dist, total * 4);
  int bits = 1;
  while (bits < 32 && (uint64_t(1) << bits) < num_tris) ++bits;
  CK(sparse_emit(static_cast<const uint8_t *>(ctx->out_occ.p), static_cast<const uint32_t *>(ctx->first_tri.p), cells,
                 total, bits, ctx->sparse_tmp.p, ctx->sparse_tmp.cap, static_cast<uint32_t *>(ctx->out_dist.p), st));
  if (d_list) *d_list = static_cast<const uint32_t *>(ctx->out_dist.p);
  const uint64_t n = std::min<uint64_t>(total, cap);
  std::vector<uint32_t> lin(n);
  if (n) CK(cudaMemcpyAsync(lin.data(), ctx->out_dist.p, n * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const uint64_t rr = uint64_t(resolution);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t c = lin[i];
    cells_out[3 * i] = static_cast<int32_t>(c % rr);
    cells_out[3 * i + 1] = static_cast<int32_t>((c / rr) % rr);
    cells_out[3 * i + 2] = static_cast<int32_t>(c / (rr * rr));
  }
  return SDFB_OK;
}

extern "C" {

// ---- batched bake ------------------------------------------------------------------------------

sdfb_status sdfb_bake_batch_device(sdfb_ctx *ctx, uint32_t count, const sdfb_mesh_desc *meshes,
                                   const sdfb_grid_desc *grids, const sdfb_opts *opts, float *const *dist_outs,
                                   uint8_t *const *occ_outs, void *stream, sdfb_stats *stats) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (count == 0 || !meshes || !grids) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "empty batch");
  cudaSetDevice(ctx->device);
  const sdfb_opts o = opts_or_default(opts);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  std::vector<PlanMesh> ms(count);
  for (uint32_t m = 0; m < count; ++m) {
    const sdfb_mesh_desc &d = meshes[m];
    if (!d.verts || !d.idx || !grid_ok(&grids[m]))
      return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "mesh %u: null pointer or invalid grid", m);
    if (d.num_tris == 0 || d.num_verts == 0) return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh %u has no triangles", m);
    PlanMesh &p = ms[m];
    p.verts = d.verts;
    p.idx = d.idx;
    p.V = d.num_verts;
    p.T = d.num_tris;
    p.grid = grids[m];
    p.dist = (o.no_distance || !dist_outs) ? nullptr : dist_outs[m];
    p.occ = (o.no_occupancy || !occ_outs) ? nullptr : occ_outs[m];
    const sdfb_status sg = device_sign(ctx, o, d.verts, d.num_verts, d.idx, d.num_tris, st, &p.sign, &p.watertight);
    if (sg != SDFB_OK) {
      const std::string e = ctx->err;
      return ctx_fail(ctx, sg, "mesh %u: %s", m, e.c_str());
    }
  }
  const sdfb_status s = device_caps(ctx, st, ms);
  if (s != SDFB_OK) return s;
  return run_batch(ctx, st, ms, o, true, stats);
}

sdfb_status sdfb_bake_batch(sdfb_ctx *ctx, uint32_t count, const sdfb_mesh_desc *meshes, const sdfb_grid_desc *grids,
                            const sdfb_opts *opts, float *const *dist_outs, uint8_t *const *occ_outs,
                            sdfb_stats *stats) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (count == 0 || !meshes || !grids) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "empty batch");
  cudaSetDevice(ctx->device);
  const sdfb_opts o = opts_or_default(opts);
  const cudaStream_t st = ctx->stream;
  size_t nv = 0, ni = 0;
  for (uint32_t m = 0; m < count; ++m) {
    if (!meshes[m].verts || !meshes[m].idx || !grid_ok(&grids[m]))
      return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "mesh %u: null pointer or invalid grid", m);
    if (meshes[m].num_tris == 0 || meshes[m].num_verts == 0)
      return ctx_fail(ctx, SDFB_ERR_BAD_MESH, "mesh %u has no triangles", m);
    nv += size_t(meshes[m].num_verts) * 3;
    ni += size_t(meshes[m].num_tris) * 3;
  }
  const bool want_dist = dist_outs && !o.no_distance, want_occ = occ_outs && !o.no_occupancy;
  ENSURE(ctx->in_verts, nv * 4);
  ENSURE(ctx->in_idx, ni * 4);
  std::vector<PlanMesh> ms(count);
  std::vector<float *> direct_dist(count, nullptr);
  std::vector<uint8_t *> direct_occ(count, nullptr);
  size_t ov = 0, oi = 0;
  uint64_t occ_off = 0;
  for (uint32_t m = 0; m < count; ++m) {
    const sdfb_mesh_desc &d = meshes[m];
    PlanMesh &p = ms[m];
    float *dv = static_cast<float *>(ctx->in_verts.p) + ov;
    uint32_t *di = static_cast<uint32_t *>(ctx->in_idx.p) + oi;
    CK(cudaMemcpyAsync(dv, d.verts, size_t(d.num_verts) * 12, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(di, d.idx, size_t(d.num_tris) * 12, cudaMemcpyHostToDevice, st));
    const sdfb_status sg = device_sign(ctx, o, dv, d.num_verts, di, d.num_tris, st, &p.sign, &p.watertight);
    if (sg != SDFB_OK) {
      const std::string e = ctx->err;
      return ctx_fail(ctx, sg, "mesh %u: %s", m, e.c_str());
    }
    p.verts = dv;
    p.idx = di;
    p.V = d.num_verts;
    p.T = d.num_tris;
    p.grid = grids[m];
    if (want_dist && dist_outs[m] && p.sign != kSignGwn)
      direct_dist[m] = static_cast<float *>(mapped_host(dist_outs[m]));
    ov += size_t(d.num_verts) * 3;
    oi += size_t(d.num_tris) * 3;
  }
  // Outputs: pinned caller buffers directly, the rest through device buffers copied out afterwards.
  uint64_t staged = 0;
  for (uint32_t m = 0; m < count; ++m) {
    const uint64_t cells = uint64_t(grids[m].nx) * grids[m].ny * grids[m].nz;
    if ((want_dist && dist_outs[m] && !direct_dist[m]) || (want_occ && occ_outs[m] && !direct_occ[m]))
      staged += cells;
  }
  if (staged > 0 && want_dist) ENSURE(ctx->out_dist, staged * 4);
  if (staged > 0 && want_occ) ENSURE(ctx->out_occ, staged);
  for (uint32_t m = 0; m < count; ++m) {
    PlanMesh &p = ms[m];
    const uint64_t cells = uint64_t(p.grid.nx) * p.grid.ny * p.grid.nz;
    const bool stage = (want_dist && dist_outs[m] && !direct_dist[m]) || (want_occ && occ_outs[m] && !direct_occ[m]);
    if (want_dist && dist_outs[m])
      p.dist = direct_dist[m] ? direct_dist[m] : static_cast<float *>(ctx->out_dist.p) + occ_off;
    if (want_occ && occ_outs[m])
      p.occ = direct_occ[m] ? direct_occ[m] : static_cast<uint8_t *>(ctx->out_occ.p) + occ_off;
    if (stage) occ_off += cells;
  }
  sdfb_status s = device_caps(ctx, st, ms);
  if (s != SDFB_OK) return s;
  s = run_batch(ctx, st, ms, o, true, stats);
  if (s != SDFB_OK) return s;
  for (uint32_t m = 0; m < count; ++m) {
    const uint64_t cells = uint64_t(ms[m].grid.nx) * ms[m].grid.ny * ms[m].grid.nz;
    if (ms[m].dist && !direct_dist[m])
      CK(cudaMemcpyAsync(dist_outs[m], ms[m].dist, cells * 4, cudaMemcpyDeviceToHost, st));
    if (ms[m].occ && !direct_occ[m]) CK(cudaMemcpyAsync(occ_outs[m], ms[m].occ, cells, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

}  // extern "C"
