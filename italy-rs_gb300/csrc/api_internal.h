// Internal host-side types shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/sdfb.h"
#include "kernels.h"

// NVTX range in the "sdfb" domain for one bake stage (build, occupancy, crossings, distance,
// winding number, ...): a profiler attributes the kernels launched inside it to the stage. The
// header-only NVTX3 API costs a branch when no tool is attached.
inline nvtxDomainHandle_t nvtx_domain() {
  static const nvtxDomainHandle_t d = nvtxDomainCreateA("sdfb");
  return d;
}
struct NvtxRange {
  explicit NvtxRange(const char *name) {
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = name;
    nvtxDomainRangePushEx(nvtx_domain(), &a);
  }
  ~NvtxRange() { nvtxDomainRangePop(nvtx_domain()); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

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

// A mesh hierarchy resident in device memory (built once, reused by later bakes).
struct ResidentBvh {
  const sdfb::Node *nodes = nullptr;
  const sdfb::DistTri *dtris = nullptr;  // distance hierarchy
  const sdfb::TriRec *tris = nullptr;    // winding-number hierarchy
  const uint32_t *leaf_order = nullptr;
  const float4 *node_moment = nullptr;
  int num_nodes = 0, num_inner = 0, num_tris = 0, root = 0;
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
  const ResidentBvh *bvh = nullptr;   // set: use this hierarchy instead of building one
  const ResidentBvh *caps = nullptr;  // set: the caps hierarchy of a resident winding-number mesh
};


struct GwnInput {
  sdfb::BatchDev batch;
  const uint64_t *col_start;
  const float *col_z;
  const int8_t *col_s;
  float band_voxels;
  uint32_t *err;
  uint64_t gwn_cells;  // cells of the winding-number meshes (refine list capacity)
};

// Workspace::misc (256 bytes, zeroed before every bake): error flags at 0, the distance tile
// counter at 64, work counters at 128 (box, triangle, SAT, plane tests), the deferral counters at
// 160.
constexpr size_t kMiscDeferOffset = 192;
// Traversal steps a distance tile may take before it is deferred to the block-per-tile pass.
constexpr int kDefaultStepBudget = 1024;

// Device workspace of one bake in flight. The context owns one; the serving loop owns one per
// stream so consecutive waves overlap.
struct Workspace {
  DevBuf batch_buf, bvh, build_tmp, par_tmp, col_start, col_z, col_s, caps_bvh, caps_tmp, misc, gwn_tmp, defer;
  PinBuf staging;
  cudaEvent_t ev[8] = {};
  uint64_t col_capacity_hint = 0;
  cudaGraphExec_t graph = nullptr;  // the last batch's launch sequence, replayed while it repeats
  std::vector<uint8_t> graph_key;
  uint64_t graph_launches = 0;
  bool init();
  ~Workspace();
  void release();
  uint64_t bytes() const;
};

// What enqueue_batch leaves for finish_batch.
struct BatchState {
  uint64_t capacity = 0, total_cols = 0, total_cells = 0, total_tris = 0, launched = 0;
  bool any_cross = false, any_gwn = false, graphed = false;
  int tile_id = 0, stack = 64, leaf0 = 0;
};


struct sdfb_ctx {
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // inputs / outputs of host-buffer calls
  DevBuf in_verts, in_idx, in_verts2, in_idx2, in_caps, in_capidx, out_dist, out_occ, first_tri, sparse_tmp,
      sparse_out;
  // materials: the batch record, material tables and texels, per-triangle materials, sorted hits,
  // per-cell outputs
  DevBuf mat_rec, mat_in, mat_tri, hit_keys, hit_vals, hit_alt, mat_cells;
  DevBuf cons_grid, cons_io;  // consumer check: a grid and its queries / results
  DevBuf weld_tmp;            // device weld / watertight census
  DevBuf caps_tmp, caps_misc; // device-built winding-number caps: temporaries, totals and error word
  PinBuf staging_small;
  Workspace ws;
  int tuned_leaf[32][8];  // [log2 T][log2 n - 4]
  int tuned_tile[32][8];
  int tuned_stack[32][8];
  int tuned_budget[32][8];  // distance pass: steps before a tile is deferred (0 = never)
  // Batch-wide override for bakes of more than one mesh ("batch tile stack budget" in the table;
  // tile -1 = none): a batch otherwise takes the bucket of its mesh with the most cells.
  int batch_tile = -1, batch_stack = 64, batch_budget = 0;

  ~sdfb_ctx();
  DevBuf *all_bufs(int i);
  void release_all();
  uint64_t device_bytes() const;
};

int bucket_tris(uint64_t T);
int bucket_grid(const sdfb_grid_desc &g);

// Reads the tuned leaf / tile / stack table (orchestrate.cu).
void load_tuning(sdfb_ctx *ctx);

sdfb_status ctx_fail(sdfb_ctx *ctx, sdfb_status st, const char *fmt, ...);
sdfb_status ctx_cuda(sdfb_ctx *ctx, cudaError_t e, const char *what);
// Sign mode of a mesh in device memory: forced modes pass through; AUTO runs the weld + watertight
// gate on the device (parity when watertight, else the winding number). Fails with BAD_MESH on an
// index out of range.
sdfb_status device_sign(sdfb_ctx *ctx, const sdfb_opts &o, const float *d_verts, uint32_t V, const uint32_t *d_idx,
                        uint32_t T, cudaStream_t st, int *sign, int *watertight);
// sdfb_voxelize_sparse; also returns the device list of the count occupied cells' linear indices
// (valid until the context's next call) and the grid it used.
sdfb_status voxelize_sparse_run(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                                const float bounds_max[3], int32_t resolution, int32_t *cells_out, uint64_t cap,
                                uint64_t *count, float origin_out[3], float *voxel_out, const uint32_t **d_list,
                                sdfb_grid_desc *grid_out);
bool grid_ok(const sdfb_grid_desc *g);
sdfb::GridDev to_dev(const sdfb_grid_desc &g);
sdfb_opts opts_or_default(const sdfb_opts *o);

// Enqueues every stage of a bake for `meshes` on `st` (nothing waits). Meshes either all carry a
// resident hierarchy or none does (then one hierarchy over all of them is built). use_graph:
// capture the launch sequence into a CUDA graph and replay it while the batch is unchanged.
sdfb_status enqueue_batch(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, std::vector<PlanMesh> &meshes,
                          const sdfb_opts &opts, bool use_graph, BatchState &state);
// Waits for the stream, reads the device error word and fills stats. SDFB_ERR_BUSY means the
// crossing list outgrew its buffer: enqueue the same batch again (the buffer has been resized).
sdfb_status finish_batch(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, const BatchState &state,
                         const std::vector<PlanMesh> &meshes, sdfb_stats *stats);
// enqueue + finish, retrying a crossing-list overflow and a shallow-stack overflow.
sdfb_status run_batch(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &meshes, const sdfb_opts &opts,
                      bool use_graph, sdfb_stats *stats);
// Builds the hierarchy of one mesh (and of its caps when cT > 0) into `mem` / `cap_mem`, which
// must hold resident_bytes(T) / resident_bytes(cT, true). Enqueued on st with ws's temporaries.
size_t resident_bytes(uint64_t tris, bool winding = false);
sdfb_status build_resident(sdfb_ctx *ctx, Workspace &ws, cudaStream_t st, const PlanMesh &mesh, void *mem,
                           ResidentBvh &out, void *cap_mem, ResidentBvh &cap_out);

// caps.cu: boundary caps of an indexed mesh on the device. centres receives up to 3T loop centres
// (3 floats each), cap_tris up to 3T cap triangles (indices; centre c is vertex V + c); totals[0] =
// cap triangles (boundary half-edges), totals[1] = loops. Enqueued only.
size_t caps_temp_bytes(uint64_t T);
cudaError_t caps_device(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, void *temp,
                        size_t temp_bytes, float *centres, uint32_t *cap_tris, uint64_t *totals, uint32_t *err,
                        int num_sms, cudaStream_t st);
// The crossing mesh (mesh + caps) and the caps of every winding-number mesh of ms that has a
// distance output, built on the device into the context's buffers; sets their pverts / pidx /
// cverts / cidx and counts. The caps close the crossing mesh already set (pverts / pidx, as the
// soup bake's welded mesh), else the mesh itself. One read of the totals synchronises the stream.
// every_gwn: also the winding-number meshes without a distance output (resident meshes).
sdfb_status device_caps(sdfb_ctx *ctx, cudaStream_t st, std::vector<PlanMesh> &ms, bool every_gwn = false);

// Winding-number pass 1 tiles: 4 x 4 x (2 kGwnCellsPerLane) cells, kGwnCellsPerLane per lane.
constexpr int kGwnCellsPerLane = 4;
constexpr int kGwnTileZ = 2 * kGwnCellsPerLane;
// gwn.cu: flips the sign of cells whose generalized winding number says inside (enqueued only).
size_t gwn_temp_bytes(uint64_t gwn_cells);
cudaError_t gwn_enqueue(const GwnInput &in, void *temp, int num_sms, cudaStream_t st);
uint64_t *gwn_refine_counter(void *temp);
// Cells whose sign needed the direct FP64 sum over every cap triangle (the last pass).
uint64_t *gwn_direct_counter(void *temp);
