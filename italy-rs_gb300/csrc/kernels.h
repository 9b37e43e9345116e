// Host-side launch interface of the bake kernels. Every launcher enqueues work on the given
// stream and returns the launch error (cudaSuccess when it was enqueued).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sdfb {

struct TriRec;
struct Node;

// Device scratch for the device-wide primitives; grown by the caller (see Workspace in api.cu).
struct Scratch {
  void *ptr = nullptr;
  size_t bytes = 0;
};

// Count of kernel launches issued by this library (every launcher calls note_launch once per
// <<<...>>>); the bake reports the launches of one call in sdfb_stats.
void note_launch();
uint64_t launch_count();

// ---- primitives.cu ----------------------------------------------------------------------------
// Exclusive scan of n uint32 counts into uint64 starts; starts[n] receives the total, so `out`
// must hold n + 1 values. Scratch need: scan_scratch_bytes(n).
size_t scan_scratch_bytes(size_t n);
cudaError_t exclusive_scan_u32(const uint32_t *in, uint64_t *out, size_t n, Scratch s, cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on bits [0, bits) of the keys, 8 bits per pass.
// keys/vals hold the input and receive the result; keys_alt/vals_alt are same-size temporaries.
size_t sort_scratch_bytes(size_t n);
cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                             int bits, Scratch s, cudaStream_t st);

// ---- lbvh.cu ----------------------------------------------------------------------------------
// One mesh's device-resident acceleration structure.
struct MeshDev {
  uint32_t num_verts = 0, num_tris = 0;
  const float *verts = nullptr;     // V x 3 (original positions; occupancy and parity read these)
  const uint32_t *idx = nullptr;    // T x 3
  TriRec *tris = nullptr;           // T records in leaf order
  Node *nodes = nullptr;            // max(T - 1, 1) nodes, root = 0
  uint32_t *leaf_order = nullptr;   // original triangle index of each record
  uint32_t *bounds = nullptr;       // 6 ordered-uint words: min xyz, max xyz
  float4 *moments = nullptr;        // optional: 4 float4 per inner node (winding-number expansion)
  int leaf_size = 1;
};

// Temporaries of one build, sized by lbvh_temp_bytes(T).
size_t lbvh_temp_bytes(uint32_t num_tris);
// tris + nodes + leaf_order + bounds (+ moments when with_moments)
size_t lbvh_mesh_bytes(uint32_t num_tris, bool with_moments = false);
// Carves a MeshDev's arrays out of `mem` (lbvh_mesh_bytes(T, with_moments) bytes, 256-aligned).
void lbvh_bind_mesh(MeshDev &m, void *mem, bool with_moments = false);
// Builds the hierarchy; when m.moments is set it also fills the winding-number moments.
cudaError_t lbvh_build(MeshDev &m, int leaf_size, void *temp, size_t temp_bytes, uint32_t *err, cudaStream_t st);

// ---- occupancy.cu -----------------------------------------------------------------------------
struct GridDev {
  float ox, oy, oz, voxel;
  int nx, ny, nz;
};

size_t occupancy_temp_bytes(uint32_t num_tris);
// occ must hold nx * ny * nz bytes; it is cleared and then filled. sat_tests (optional device
// uint64) receives the number of SAT tests.
cudaError_t occupancy_dense(const float *verts, const uint32_t *idx, uint32_t num_verts, uint32_t num_tris, GridDev g,
                            uint8_t *occ, void *temp, size_t temp_bytes, unsigned long long *sat_tests,
                            cudaStream_t st);
// Variant that also records, per occupied cell, the smallest triangle index that hits it
// (first_tri must hold nx*ny*nz uint32 and is initialised here).
cudaError_t occupancy_dense_first(const float *verts, const uint32_t *idx, uint32_t num_verts, uint32_t num_tris,
                                  GridDev g, uint8_t *occ, uint32_t *first_tri, void *temp, size_t temp_bytes,
                                  cudaStream_t st);

// ---- parity.cu --------------------------------------------------------------------------------
// Column crossing lists for +z parity: col_start[nx*ny + 1] (uint64 starts), col_z[capacity].
size_t parity_temp_bytes(uint32_t num_tris, int nx, int ny);
cudaError_t parity_columns(const float *verts, const uint32_t *idx, uint32_t num_verts, uint32_t num_tris, GridDev g,
                           uint64_t *col_start,
                           float *col_z, uint64_t capacity, void *temp, size_t temp_bytes, uint32_t *err,
                           cudaStream_t st);

// ---- distance.cu ------------------------------------------------------------------------------
enum SignKind : int { kSignNone = 0, kSignParity = 1, kSignGwn = 2 };

struct DistanceArgs {
  const Node *nodes;
  const TriRec *tris;
  int num_nodes;  // inner nodes (max(T - 1, 1))
  int num_tris;
  GridDev g;
  int sign;
  const uint64_t *col_start;  // parity
  const float *col_z;
  float *dist;
  uint32_t *err;
  unsigned long long *tile_counter;      // zeroed by the launcher
  unsigned long long *work_counters;     // optional: [0] box tests, [1] triangle tests (lanes)
};

int tile_shape_count();
// tile shape id -> (tx, ty, tz)
void tile_shape(int id, int &tx, int &ty, int &tz);
cudaError_t distance_launch(const DistanceArgs &a, int tile_id, int num_sms, cudaStream_t st);

// ---- sparse.cu --------------------------------------------------------------------------------
size_t sparse_temp_bytes(size_t cells, size_t max_out);
// Counts occupied cells (synchronises the stream; *h_total is host memory).
cudaError_t sparse_count(const uint8_t *occ, size_t cells, void *temp, size_t temp_bytes, uint64_t *h_total,
                         cudaStream_t st);
// Writes the occupied cell indices ordered by (first triangle, cell index) into cells_out.
cudaError_t sparse_emit(const uint8_t *occ, const uint32_t *first_tri, size_t cells, uint64_t total, int tri_bits,
                        void *temp, size_t temp_bytes, uint32_t *cells_out, cudaStream_t st);

}  // namespace sdfb
