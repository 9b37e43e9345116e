// Host-side launch interface of the bake kernels. Every launcher enqueues work on the given
// stream and returns the launch error (cudaSuccess when it was enqueued).
//
// All stages work on a batch of meshes at once: triangles, cells, columns and tiles of the meshes
// are numbered consecutively ("global" indices), each kernel finds the mesh of a global index by
// binary search over a prefix table, and a single mesh is simply a batch of one.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sdfb {

struct TriRec;
struct DistTri;
struct Node;

// Count of kernel launches issued by this library (every launcher calls note_launch once per
// <<<...>>>); the bake reports the launches of one call in sdfb_stats.
void note_launch();
uint64_t launch_count();

// Device scratch for the device-wide primitives.
struct Scratch {
  void *ptr = nullptr;
  size_t bytes = 0;
};

// ---- primitives.cu ----------------------------------------------------------------------------
// Exclusive scan of n uint32 counts into uint64 starts; out[n] receives the total, so `out` must
// hold n + 1 values. Scratch need: scan_scratch_bytes(n).
size_t scan_scratch_bytes(size_t n);
cudaError_t exclusive_scan_u32(const uint32_t *in, uint64_t *out, size_t n, Scratch s, cudaStream_t st);
// The same for uint64 counts (per-triangle candidate counts, which can pass 2^32 on large grids).
cudaError_t exclusive_scan_u64(const uint64_t *in, uint64_t *out, size_t n, Scratch s, cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on bits [0, bits) of the keys, 8 bits per pass.
// keys/vals hold the input and receive the result; keys_alt/vals_alt are same-size temporaries.
size_t sort_scratch_bytes(size_t n);
cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                             int bits, Scratch s, cudaStream_t st);

// ---- the batch ---------------------------------------------------------------------------------
struct GridDev {
  float ox, oy, oz, voxel;
  int nx, ny, nz;
};

enum SignKind : int { kSignNone = 0, kSignParity = 1, kSignGwn = 2 };

// Device-side record of one mesh of a batch.
struct MeshRec {
  const float *verts;     // V x 3, original positions (occupancy, parity and FP64 winding read these)
  const uint32_t *idx;    // T x 3, local vertex indices
  const float *pverts;    // the mesh whose crossings decide parity (== verts unless a welded copy)
  const uint32_t *pidx;
  float *dist;            // cell outputs (either may be null)
  uint8_t *occ;
  uint32_t num_verts, num_tris, pnum_verts, pnum_tris;
  uint64_t tri_base;      // first global triangle = first sorted position of this mesh
  uint64_t cell_base;     // first global cell
  uint64_t col_base;      // first global column (parity meshes only)
  GridDev g;
  int sign;               // SignKind
  int leaf_size;          // 1..16
  int root;               // virtual root node of this mesh (see lbvh.cu)
  int cap_root;           // GWN: virtual root of this mesh's caps in the caps hierarchy, -1 if none
  const float *cverts;    // GWN: vertices of the caps (the parity mesh's vertices + loop centres)
  const uint32_t *cidx;   // GWN: cap triangles
  uint32_t cap_tris;      // GWN: number of cap triangles
  int bvh_nodes;          // node count of the hierarchy holding this mesh (root < bvh_nodes)
  // The hierarchy holding this mesh: the batch's combined tree, or the mesh's resident tree.
  const Node *nodes;
  const DistTri *tris;
  int bvh_tris;           // records in that hierarchy
  // GWN: the hierarchy holding this mesh's caps
  int cap_nodes_n, cap_inner_n, cap_recs_n;
  const Node *cap_nodes;
  const TriRec *cap_trec;
  const float4 *cap_moment;  // per inner cap node: (area-weighted normal sum, total area)
  const uint32_t *cap_order;
};

// Prefix tables of a batch (device): starts[m] of each numbering, starts[M] = total.
struct BatchDev {
  int num_meshes = 0;
  const MeshRec *recs = nullptr;
  const uint64_t *tri_starts = nullptr;       // triangles (BVH, occupancy)
  const uint64_t *ptri_starts = nullptr;      // triangles of the parity meshes
  const uint64_t *tile_starts = nullptr;      // distance tiles
  const uint64_t *gwn_tile_starts = nullptr;  // winding-number tiles (only GWN meshes have any)
  const uint64_t *cell_starts = nullptr;      // cells
  uint64_t total_tris = 0, total_ptris = 0, total_cells = 0, total_cols = 0, total_tiles = 0, total_gwn_tiles = 0;
};

// Largest m in [0, n) with starts[m] <= x (starts[0] = 0).
__host__ __device__ __forceinline__ int find_mesh(const uint64_t *starts, int n, uint64_t x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (starts[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// ---- lbvh.cu ----------------------------------------------------------------------------------
// The batch's acceleration structure: every mesh's triangles, sorted by (mesh, Morton code), under
// one binary radix tree; each mesh's subtree is entered through its virtual root node, stored
// after the inner nodes.
struct BvhDev {
  DistTri *dtris = nullptr;        // distance hierarchy: T_total records in leaf order
  TriRec *tris = nullptr;          // winding-number hierarchy: T_total records in leaf order
  Node *nodes = nullptr;           // (T_total - 1) inner nodes + M virtual roots
  uint32_t *leaf_order = nullptr;  // local (per-mesh) triangle index of each record
  uint32_t *bounds = nullptr;      // 6 ordered-uint words per mesh: centroid min xyz, max xyz
  float4 *node_moment = nullptr;   // winding-number hierarchy, per inner node: (sum of area x unit
                                   // normal over its triangles, their total area)
  int num_inner = 0;               // max(T_total - 1, 0)
  int num_nodes = 0;               // num_inner + M
};

size_t lbvh_temp_bytes(uint64_t total_tris, int num_meshes);
// winding = false: the distance hierarchy (DistTri records); true: the winding-number hierarchy
// (TriRec records and per-node triangle areas).
size_t lbvh_bytes(uint64_t total_tris, int num_meshes, bool winding);
void lbvh_bind(BvhDev &b, void *mem, uint64_t total_tris, int num_meshes, bool winding);
cudaError_t lbvh_build(const BatchDev &batch, BvhDev &b, void *temp, size_t temp_bytes, uint32_t *err,
                       cudaStream_t st);

// ---- occupancy.cu -----------------------------------------------------------------------------
size_t occupancy_temp_bytes(uint64_t total_tris);
// Clears and fills every mesh's occ grid (meshes with occ == null are skipped). first_tri
// (optional, for a batch of one) receives per cell the smallest triangle index that hits it.
cudaError_t occupancy_batch(const BatchDev &batch, uint32_t *first_tri, void *temp, size_t temp_bytes,
                            unsigned long long *sat_tests, int num_sms, cudaStream_t st);

// ---- parity.cu --------------------------------------------------------------------------------
// Column crossing lists along +z over the parity and winding-number meshes (their pverts / pidx):
// col_start[total_cols + 1] (uint64 starts), col_z[capacity] heights, col_s[capacity] orientations.
size_t parity_temp_bytes(uint64_t total_ptris, uint64_t total_cols);
cudaError_t parity_columns(const BatchDev &batch, uint64_t *col_start, float *col_z, int8_t *col_s,
                           uint64_t capacity, void *temp, size_t temp_bytes, uint32_t *err, int num_sms,
                           cudaStream_t st);

// ---- distance.cu ------------------------------------------------------------------------------
struct DistanceArgs {
  BatchDev batch;             // each mesh record names its hierarchy and root
  const uint64_t *col_start;  // parity
  const float *col_z;
  uint32_t *err;
  unsigned long long *tile_counter;   // pass A's chunk counter, zeroed by the launcher
  unsigned long long chunk_tiles;     // tiles per chunk (set by the launcher)
  unsigned long long *work_counters;  // optional: [0] box, [1] triangle, [3] plane, [4] rectangle tests (lanes)
  // Deferral of long tiles (none when defer_list is null or step_budget <= 0): every step_budget
  // traversal steps a walk checks whether all tiles have been handed out and, if so, defers its
  // tile. The list holds defer_capacity tile indices; defer_counters[0] counts deferred tiles (it
  // may pass the capacity), [1] is the second pass's tile counter. Both counters are zeroed by the
  // launcher.
  unsigned long long *defer_list;
  unsigned long long defer_capacity;
  unsigned long long *defer_counters;
  long long step_budget;
  int fault;  // sdfb_opts.fault_inject bits (testing only; 0 in normal use)
};

int tile_shape_count();
// FP32 flops of the counted distance work (counters as in DistanceArgs::work_counters).
double distance_work_flops(int tile_id, const unsigned long long *counters);
// tile shape id -> (tx, ty, tz)
void tile_shape(int id, int &tx, int &ty, int &tz);
uint64_t tiles_for(const GridDev &g, int tile_id);
// stack_depth: 32 or 64 entries (32 keeps the stack in one register per lane).
// Deferred-list capacity for a launch of total_tiles tiles.
uint64_t defer_capacity_for(uint64_t total_tiles);
cudaError_t distance_launch(const DistanceArgs &a, int tile_id, int stack_depth, int num_sms, cudaStream_t st);

// Every (cell, triangle) pair of a ONE-mesh batch that passes the occupancy rule, as keys
// (cell << tri_bits) | local triangle, appended in no particular order (the mesh's occupancy grid
// is written as well). *hit_count (device) receives the number of hits, also when it exceeds
// `capacity` (then only `capacity` keys are written).
cudaError_t occupancy_hits(const BatchDev &B, void *temp, size_t temp_bytes, uint64_t *keys, uint64_t capacity,
                           unsigned long long *hit_count, int tri_bits, int num_sms, cudaStream_t st);

// ---- weld.cu ----------------------------------------------------------------------------------
// weldPositions on the device: welded[i] = the first-occurrence number of position i's lattice key
// (cell: the weld lattice, weld_cell in host_mesh.h); first_of (optional, num_unique entries) gets
// each number's first position. Synchronises the stream (*num_unique is host memory).
size_t weld_temp_bytes(uint64_t n);
cudaError_t weld_device(const float *pos, uint64_t n, float cell, uint32_t *welded, uint32_t *first_of, void *temp,
                        size_t temp_bytes, uint32_t *num_unique, int num_sms, cudaStream_t st);
// out[u] = pos[first_of[u]] (3 floats) for u < U.
cudaError_t gather_unique(const float *pos, const uint32_t *first_of, uint64_t U, float *out, int num_sms,
                          cudaStream_t st);
// Edge census of a welded triangle list (degenerate triangles skipped); every index must be below
// num_unique (0: unknown). Synchronises the stream.
size_t watertight_temp_bytes(uint64_t T);
cudaError_t watertight_device(const uint32_t *welded, uint64_t T, uint32_t num_unique, void *temp, size_t temp_bytes,
                              uint64_t *boundary, uint64_t *nonmanifold, int num_sms, cudaStream_t st);

// The watertight gate of an indexed mesh on the device (the weld of its vertices over their
// bounds, then the edge census of the welded triangles; equivalent to the reference's test on the
// de-indexed soup). *result: 1 watertight, 0 not, -2 an index >= V. Synchronises the stream.
size_t indexed_gate_temp_bytes(uint64_t V, uint64_t T);
cudaError_t indexed_watertight_device(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, void *temp,
                                      size_t temp_bytes, int *result, int num_sms, cudaStream_t st);

// ---- sparse.cu --------------------------------------------------------------------------------
size_t sparse_temp_bytes(size_t cells, size_t max_out);
// Counts occupied cells (synchronises the stream; *h_total is host memory).
cudaError_t sparse_count(const uint8_t *occ, size_t cells, void *temp, size_t temp_bytes, uint64_t *h_total,
                         cudaStream_t st);
// Writes the occupied cell indices ordered by (first triangle, cell index) into cells_out.
cudaError_t sparse_emit(const uint8_t *occ, const uint32_t *first_tri, size_t cells, uint64_t total, int tri_bits,
                        void *temp, size_t temp_bytes, uint32_t *cells_out, cudaStream_t st);

}  // namespace sdfb
