// Internal host-side types shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

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

// Grow-only pinned host buffer.
struct PinBuf {
  void *p = nullptr;
  size_t cap = 0;
  PinBuf() = default;
  PinBuf(const PinBuf &) = delete;
  PinBuf &operator=(const PinBuf &) = delete;
  ~PinBuf() { release(); }
  bool ensure(size_t bytes);
  void release();
};

// One mesh of a bake as the orchestrator sees it (every pointer is device memory).
struct PlanMesh {
  const float *verts = nullptr;   // geometry: BVH, occupancy, distance
  const uint32_t *idx = nullptr;
  uint32_t V = 0, T = 0;
  const float *pverts = nullptr;  // crossing mesh: parity, or mesh + caps for the winding number
  const uint32_t *pidx = nullptr;
  uint32_t pV = 0, pT = 0;
  const float *cverts = nullptr;  // winding number: the caps alone (indices into cverts)
  const uint32_t *cidx = nullptr;
  uint32_t cT = 0;
  sdfb_grid_desc grid{};
  int sign = sdfb::kSignNone;
  int leaf = 0;                   // 0 = tuned default
  float *dist = nullptr;
  uint8_t *occ = nullptr;
  int watertight = -1;
};

// Host-side result of capping a mesh for the winding-number sign.
struct CapBuild {
  std::vector<float> verts;    // mesh vertices followed by the loop centres
  std::vector<uint32_t> pidx;  // mesh triangles followed by the cap triangles
  std::vector<uint32_t> cidx;  // cap triangles alone
  size_t loops = 0;
};
// Builds the crossing mesh (mesh + caps) and the caps of an indexed mesh.
void build_caps(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, CapBuild &out);

struct GwnInput {
  sdfb::BatchDev batch;
  const uint64_t *col_start;
  const float *col_z;
  const int8_t *col_s;
  sdfb::BvhDev caps;
  uint64_t cap_total_tris;
  float band_voxels;
  uint32_t *err;
  uint64_t gwn_cells;  // cells of the winding-number meshes (refine list capacity)
};

struct GraphEntry;

struct sdfb_ctx {
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  std::string err;
  // inputs / outputs of host-buffer calls
  DevBuf in_verts, in_idx, in_verts2, in_idx2, in_caps, in_capidx, out_dist, out_occ, first_tri;
  // workspace of one bake
  DevBuf batch_buf, bvh, build_tmp, par_tmp, col_start, col_z, col_s, caps_bvh, caps_tmp, misc, gwn_tmp;
  PinBuf staging, staging_out;
  uint64_t col_capacity_hint = 0;
  uint64_t gwn_refined = 0;  // cells of the last bake that took the FP64 winding-number pass
  // CUDA graph of the last batch shape (replayed when the same batch comes again)
  cudaGraphExec_t graph = nullptr;
  std::vector<uint8_t> graph_key;
  uint64_t graph_launches = 0;  // kernels inside the cached graph
  int tuned_leaf[32][8];  // [log2 T][log2 n - 4]
  int tuned_tile[32][8];
  int tuned_stack[32][8];

  ~sdfb_ctx();
  DevBuf *all_bufs(int i);
  void release_all();
  uint64_t device_bytes() const;
};

// Reads the tuned leaf / tile / stack table (orchestrate.cu).
void load_tuning(sdfb_ctx *ctx);

sdfb_status ctx_fail(sdfb_ctx *ctx, sdfb_status st, const char *fmt, ...);
sdfb_status ctx_cuda(sdfb_ctx *ctx, cudaError_t e, const char *what);
bool grid_ok(const sdfb_grid_desc *g);
sdfb::GridDev to_dev(const sdfb_grid_desc &g);
sdfb_opts opts_or_default(const sdfb_opts *o);

// Runs every stage of a bake for `meshes` on stream `st` and waits for it. use_graph: capture the
// launch sequence into a CUDA graph and replay it while the batch is unchanged.
sdfb_status run_batch(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &meshes, const sdfb_opts &opts,
                      bool use_graph, sdfb_stats *stats);

// gwn.cu: flips the sign of cells whose generalized winding number says inside.
sdfb_status gwn_apply(sdfb_ctx *ctx, cudaStream_t st, const GwnInput &in);
