// Internal host-side types shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/sdfb.h"
#include "kernels.h"

// Grow-only device buffer.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  bool ensure(size_t bytes);
  void release();
};

// The mesh of one bake. parity_* (optional) name a second mesh whose crossings decide parity:
// the welded copy of a soup, so that near-coincident duplicates cannot leak the ray.
struct BakeInput {
  const float *verts;
  const uint32_t *idx;
  uint32_t num_verts, num_tris;
  const float *parity_verts;
  const uint32_t *parity_idx;
  uint32_t parity_num_verts, parity_num_tris;
  int watertight;  // 1, 0, -1 (not evaluated)
};

struct sdfb_ctx {
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[7] = {};
  std::string err;
  // inputs / outputs of host-buffer calls
  DevBuf in_verts, in_idx, in_verts2, in_idx2, out_dist, out_occ, first_tri;
  // workspace of one bake
  DevBuf mesh, build_tmp, par_tmp, col_start, col_z, misc, gwn_tmp;
  uint64_t col_capacity_hint = 0;
  uint64_t gwn_refined = 0;  // cells of the last bake that took the FP64 winding-number pass

  ~sdfb_ctx() {
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
  DevBuf *all_bufs(int i) {
    DevBuf *b[] = {&in_verts, &in_idx, &in_verts2, &in_idx2, &out_dist, &out_occ, &first_tri,
                   &mesh,     &build_tmp, &par_tmp, &col_start, &col_z,   &misc,    &gwn_tmp};
    return i < int(sizeof b / sizeof b[0]) ? b[i] : nullptr;
  }
  void release_all() {
    for (int i = 0; DevBuf *b = all_bufs(i); ++i) b->release();
  }
  uint64_t device_bytes() const {
    uint64_t s = 0;
    for (int i = 0; const DevBuf *b = const_cast<sdfb_ctx *>(this)->all_bufs(i); ++i) s += b->cap;
    return s;
  }
};

sdfb_status ctx_fail(sdfb_ctx *ctx, sdfb_status st, const char *fmt, ...);
sdfb_status ctx_cuda(sdfb_ctx *ctx, cudaError_t e, const char *what);
bool grid_ok(const sdfb_grid_desc *g);
sdfb::GridDev to_dev(const sdfb_grid_desc &g);
sdfb_opts opts_or_default(const sdfb_opts *o);

// One bake on device buffers; synchronises `st` and reads the device error word.
sdfb_status run_bake(sdfb_ctx *ctx, cudaStream_t st, const BakeInput &in, const sdfb_grid_desc &grid,
                     const sdfb_opts &opts, int sign, float *d_dist, uint8_t *d_occ, sdfb_stats *stats);

// gwn.cu: flips the sign of cells whose generalized winding number says inside, computing the
// winding number in FP64 for cells within opts.band_voxels of the surface and FP32 elsewhere.
sdfb_status gwn_apply(sdfb_ctx *ctx, cudaStream_t st, const sdfb::MeshDev &m, const BakeInput &in,
                      const sdfb_grid_desc &grid, const sdfb_opts &opts, float *d_dist, uint32_t *d_err);
