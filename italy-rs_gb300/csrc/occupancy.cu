// Dense occupancy: the reference's candidate-cell loop (src/convert/sdf_baker.cpp:89-118) as a
// load-balanced expansion over (triangle, candidate cell) items.
//
// k_occ_items counts each triangle's clamped candidate box with the reference's FP32 rounding;
// an exclusive scan turns the counts into item starts; k_occ_test takes chunks of items, runs the
// exact-rounding SAT test (common.cuh) and stores 1 for hits. Several triangles may store 1 into
// the same byte; the stores carry the same value, so no atomics are needed and the result does
// not depend on their order.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "expand.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct TriCells {
  f3 a, b, c;
  int lo[3], hi[3];
  int mesh;
};

__device__ __forceinline__ f3 vload(const float *v, uint32_t i) {
  return {__ldg(v + 3ull * i), __ldg(v + 3ull * i + 1), __ldg(v + 3ull * i + 2)};
}

// Triangle t (global) with its mesh's clamped candidate box. Out-of-range indices read vertex 0
// (the bake reports the mesh as bad; reads stay in bounds). A mesh without an occupancy output
// gets an empty box.
__device__ __forceinline__ TriCells tri_cells(const BatchDev &B, uint64_t t) {
  TriCells r;
  r.mesh = find_mesh(B.tri_starts, B.num_meshes, t);
  const MeshRec &M = B.recs[r.mesh];
  const uint64_t lt = t - B.tri_starts[r.mesh];
  const uint32_t V = M.num_verts;
  const uint32_t i0 = __ldg(M.idx + 3 * lt), i1 = __ldg(M.idx + 3 * lt + 1), i2 = __ldg(M.idx + 3 * lt + 2);
  r.a = vload(M.verts, i0 < V ? i0 : 0);
  r.b = vload(M.verts, i1 < V ? i1 : 0);
  r.c = vload(M.verts, i2 < V ? i2 : 0);
  const GridDev &g = M.g;
  const float mn[3] = {min_ref(min_ref(r.a.x, r.b.x), r.c.x), min_ref(min_ref(r.a.y, r.b.y), r.c.y),
                       min_ref(min_ref(r.a.z, r.b.z), r.c.z)};
  const float mx[3] = {max_ref(max_ref(r.a.x, r.b.x), r.c.x), max_ref(max_ref(r.a.y, r.b.y), r.c.y),
                       max_ref(max_ref(r.a.z, r.b.z), r.c.z)};
  const float o[3] = {g.ox, g.oy, g.oz};
  const int nmax[3] = {g.nx - 1, g.ny - 1, g.nz - 1};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = cell_index_clamped(mn[k], o[k], g.voxel, nmax[k]);
    r.hi[k] = cell_index_clamped(mx[k], o[k], g.voxel, nmax[k]);
  }
  if (!M.occ) {
    r.lo[0] = 0;
    r.hi[0] = -1;
  }
  return r;
}

// Candidate cells per triangle, as 64-bit counts: one triangle across a large grid can have more
// than 2^32 candidate cells.
__global__ __launch_bounds__(kThreads) void k_occ_items(BatchDev B, uint64_t *__restrict__ items) {
  const uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (t >= B.total_tris) return;
  const TriCells tc = tri_cells(B, t);
  if (tc.hi[0] < tc.lo[0]) {
    items[t] = 0;
    return;
  }
  items[t] = uint64_t(tc.hi[0] - tc.lo[0] + 1) * uint64_t(tc.hi[1] - tc.lo[1] + 1) * uint64_t(tc.hi[2] - tc.lo[2] + 1);
}

// Clears the occupancy grids of the batch (one pass over the global cells). A thread clears 16
// consecutive cells, with one 16-byte store where they lie in one mesh's grid at an aligned
// address (so a warp writes 512 contiguous bytes), else byte by byte.
__global__ __launch_bounds__(kThreads) void k_occ_clear(BatchDev B) {
  const uint64_t stride = uint64_t(gridDim.x) * kThreads * 16;
  for (uint64_t c0 = (uint64_t(blockIdx.x) * kThreads + threadIdx.x) * 16; c0 < B.total_cells; c0 += stride) {
    int m = find_mesh(B.cell_starts, B.num_meshes, c0);
    if (c0 + 16 <= B.cell_starts[m + 1]) {
      uint8_t *occ = B.recs[m].occ;
      if (!occ) continue;
      uint8_t *p = occ + (c0 - B.cell_starts[m]);
      if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        *reinterpret_cast<uint4 *>(p) = make_uint4(0u, 0u, 0u, 0u);
        continue;
      }
    }
    for (uint64_t c = c0; c < c0 + 16 && c < B.total_cells; ++c) {
      while (c >= B.cell_starts[m + 1]) ++m;
      uint8_t *occ = B.recs[m].occ;
      if (occ) occ[c - B.cell_starts[m]] = 0;
    }
  }
}

// Appends of (cell, triangle) hits: a warp-aggregated atomic reserves the slots of the lanes that
// hit together; keys past the capacity are counted but not written.
struct HitSink {
  uint64_t *keys = nullptr;
  uint64_t capacity = 0;
  unsigned long long *count = nullptr;
  int tri_bits = 0;
};

__device__ __forceinline__ void append_hit(const HitSink &h, bool hit, uint64_t key) {
  const unsigned mask = __activemask();
  const unsigned ballot = __ballot_sync(mask, hit);
  if (!ballot) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(ballot) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(h.count, static_cast<unsigned long long>(__popc(ballot)));
  base = __shfl_sync(mask, base, leader);
  if (hit) {
    const unsigned long long pos = base + __popc(ballot & ((1u << lane) - 1u));
    if (pos < h.capacity) h.keys[pos] = key;
  }
}

template <bool FIRST, bool HITS>
__global__ __launch_bounds__(kThreads) void k_occ_test(BatchDev B, const uint64_t *__restrict__ starts,
                                                       uint32_t *__restrict__ first_tri,
                                                       unsigned long long *__restrict__ sat_tests, HitSink sink) {
  const uint64_t T = B.total_tris;
  const uint64_t total = starts[T];
  const uint64_t stride = uint64_t(gridDim.x) * kThreads * kExpandChunk;
  unsigned long long tests = 0;
  for (uint64_t w0 = (uint64_t(blockIdx.x) * kThreads + threadIdx.x) * kExpandChunk; w0 < total; w0 += stride) {
    uint64_t t = item_owner(starts, static_cast<uint32_t>(T), w0);
    TriCells tc = tri_cells(B, t);
    uint64_t tstart = starts[t], tend = starts[t + 1];
    const uint64_t wend = min(w0 + kExpandChunk, total);
    for (uint64_t w = w0; w < wend; ++w) {
      while (w >= tend) {
        ++t;
        tstart = tend;
        tend = starts[t + 1];
        if (tend > tstart) tc = tri_cells(B, t);
      }
      const MeshRec &M = B.recs[tc.mesh];
      const GridDev &g = M.g;
      const uint64_t k = w - tstart;
      const uint32_t sx = tc.hi[0] - tc.lo[0] + 1, sy = tc.hi[1] - tc.lo[1] + 1;
      const int x = tc.lo[0] + static_cast<int>(k % sx);
      const int y = tc.lo[1] + static_cast<int>((k / sx) % sy);
      const int z = tc.lo[2] + static_cast<int>(k / (uint64_t(sx) * sy));
      const f3 c = {cell_center(g.ox, x, g.voxel), cell_center(g.oy, y, g.voxel), cell_center(g.oz, z, g.voxel)};
      ++tests;
      const bool hit = sat_overlap(c, __fmul_rn(g.voxel, 0.5f), tc.a, tc.b, tc.c);
      const uint64_t cell = (uint64_t(z) * g.ny + y) * g.nx + x;
      if (hit) {
        M.occ[cell] = 1;
        if (FIRST) atomicMin(first_tri + cell, static_cast<uint32_t>(t - B.tri_starts[tc.mesh]));
      }
      if (HITS) append_hit(sink, hit, (cell << sink.tri_bits) | (t - B.tri_starts[tc.mesh]));
    }
  }
  if (sat_tests) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tests += __shfl_xor_sync(kFull, tests, o);
    if ((threadIdx.x & 31) == 0 && tests) atomicAdd(sat_tests, tests);
  }
}

struct OccTemp {
  uint64_t *items;
  uint64_t *starts;
  void *scratch;
  size_t scratch_bytes;
};

size_t occ_layout(uint64_t T, char *base, OccTemp *o) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  OccTemp x;
  x.items = reinterpret_cast<uint64_t *>(take(size_t(T) * 8 + 8));
  x.starts = reinterpret_cast<uint64_t *>(take((size_t(T) + 1) * 8));
  x.scratch_bytes = scan_scratch_bytes(T);
  x.scratch = take(x.scratch_bytes);
  if (o) *o = x;
  return off;
}

}  // namespace

size_t occupancy_temp_bytes(uint64_t total_tris) { return occ_layout(total_tris, nullptr, nullptr); }

cudaError_t occupancy_batch(const BatchDev &B, uint32_t *first_tri, void *temp, size_t temp_bytes,
                            unsigned long long *sat_tests, int num_sms, cudaStream_t st) {
  const uint64_t T = B.total_tris;
  cudaError_t e;
  if (B.total_cells) {
    const uint64_t blocks = std::min<uint64_t>((B.total_cells + kThreads * 16 - 1) / (kThreads * 16), uint64_t(num_sms) * 16);
    k_occ_clear<<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(B);
    note_launch();
  }
  if (first_tri) {
    if (B.num_meshes != 1) return cudaErrorInvalidValue;
    if ((e = cudaMemsetAsync(first_tri, 0xff, B.total_cells * 4, st)) != cudaSuccess) return e;
  }
  if (T == 0) return cudaGetLastError();
  OccTemp o;
  if (occ_layout(T, static_cast<char *>(temp), &o) > temp_bytes) return cudaErrorMemoryAllocation;
  k_occ_items<<<static_cast<unsigned>((T + kThreads - 1) / kThreads), kThreads, 0, st>>>(B, o.items);
  note_launch();
  if ((e = exclusive_scan_u64(o.items, o.starts, T, Scratch{o.scratch, o.scratch_bytes}, st)) != cudaSuccess) return e;
  if (first_tri)
    k_occ_test<true, false><<<num_sms * 8, kThreads, 0, st>>>(B, o.starts, first_tri, sat_tests, HitSink());
  else
    k_occ_test<false, false><<<num_sms * 8, kThreads, 0, st>>>(B, o.starts, nullptr, sat_tests, HitSink());
  note_launch();
  return cudaGetLastError();
}

cudaError_t occupancy_hits(const BatchDev &B, void *temp, size_t temp_bytes, uint64_t *keys, uint64_t capacity,
                           unsigned long long *hit_count, int tri_bits, int num_sms, cudaStream_t st) {
  if (B.num_meshes != 1) return cudaErrorInvalidValue;
  const uint64_t T = B.total_tris;
  cudaError_t e = cudaMemsetAsync(hit_count, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  if (B.total_cells) {
    const uint64_t blocks = std::min<uint64_t>((B.total_cells + kThreads * 16 - 1) / (kThreads * 16), uint64_t(num_sms) * 16);
    k_occ_clear<<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(B);
    note_launch();
  }
  if (T == 0) return cudaGetLastError();
  OccTemp o;
  if (occ_layout(T, static_cast<char *>(temp), &o) > temp_bytes) return cudaErrorMemoryAllocation;
  k_occ_items<<<static_cast<unsigned>((T + kThreads - 1) / kThreads), kThreads, 0, st>>>(B, o.items);
  note_launch();
  if ((e = exclusive_scan_u64(o.items, o.starts, T, Scratch{o.scratch, o.scratch_bytes}, st)) != cudaSuccess) return e;
  HitSink sink;
  sink.keys = keys;
  sink.capacity = capacity;
  sink.count = hit_count;
  sink.tri_bits = tri_bits;
  k_occ_test<false, true><<<num_sms * 8, kThreads, 0, st>>>(B, o.starts, nullptr, nullptr, sink);
  note_launch();
  return cudaGetLastError();
}

}  // namespace sdfb
