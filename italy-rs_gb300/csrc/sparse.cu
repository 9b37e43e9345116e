// Sparse voxel list from a dense occupancy grid (the cell list of voxelizeMesh,
// src/convert/voxelize.cpp:52-107).
//
// Atomics-free per-tile compaction: k_tile_count counts occupied cells per 1024-cell tile; a scan
// gives each tile its output offset; k_tile_write re-scans its tile inside the block and writes
// (first triangle, cell) pairs in cell order. A stable radix sort by first triangle then yields the
// reference's insertion order: a cell is inserted by the first triangle that hits it, and one
// triangle inserts its cells in z, y, x loop order, which is increasing cell index.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr size_t kTile = size_t(kThreads) * kItems;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

__global__ __launch_bounds__(kThreads) void k_tile_count(const uint8_t *__restrict__ occ, size_t cells,
                                                         uint32_t *__restrict__ counts) {
  __shared__ uint32_t warp_sum[kThreads / kWarp];
  const size_t base = size_t(blockIdx.x) * kTile;
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const size_t k = base + size_t(i) * kThreads + threadIdx.x;
    c += (k < cells && occ[k]) ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kThreads / kWarp; ++w) s += warp_sum[w];
    counts[blockIdx.x] = s;
  }
}

__global__ __launch_bounds__(kThreads) void k_tile_write(const uint8_t *__restrict__ occ,
                                                         const uint32_t *__restrict__ first_tri, size_t cells,
                                                         const uint64_t *__restrict__ tile_start,
                                                         uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  __shared__ uint32_t warp_sum[kThreads / kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t out = tile_start[blockIdx.x];
  const size_t base = size_t(blockIdx.x) * kTile;
  for (int i = 0; i < kItems; ++i) {
    const size_t k = base + size_t(i) * kThreads + threadIdx.x;
    const bool hit = k < cells && occ[k];
    const uint32_t ballot = __ballot_sync(kFull, hit);
    if (lane == 0) warp_sum[warp] = __popc(ballot);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kThreads / kWarp; ++w) {
      const uint32_t s = warp_sum[w];
      before += w < warp ? s : 0;
      total += s;
    }
    if (hit) {
      const uint64_t at = out + before + __popc(ballot & ((1u << lane) - 1u));
      keys[at] = first_tri[k];
      vals[at] = static_cast<uint32_t>(k);
    }
    out += total;
    __syncthreads();
  }
}

struct SparseTemp {
  uint32_t *counts;
  uint64_t *starts;
  uint64_t *keys, *keys_alt;
  uint32_t *vals_alt;
  void *scratch;
  size_t scratch_bytes;
};

size_t sparse_layout(size_t cells, size_t max_out, char *base, SparseTemp *o) {
  const size_t tiles = (cells + kTile - 1) / kTile;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  SparseTemp x;
  x.counts = reinterpret_cast<uint32_t *>(take(tiles * 4 + 4));
  x.starts = reinterpret_cast<uint64_t *>(take((tiles + 1) * 8));
  x.keys = reinterpret_cast<uint64_t *>(take(max_out * 8 + 8));
  x.keys_alt = reinterpret_cast<uint64_t *>(take(max_out * 8 + 8));
  x.vals_alt = reinterpret_cast<uint32_t *>(take(max_out * 4 + 4));
  x.scratch_bytes = std::max(scan_scratch_bytes(tiles), sort_scratch_bytes(max_out));
  x.scratch = take(x.scratch_bytes);
  if (o) *o = x;
  return off;
}

}  // namespace

size_t sparse_temp_bytes(size_t cells, size_t max_out) { return sparse_layout(cells, max_out, nullptr, nullptr); }

cudaError_t sparse_count(const uint8_t *occ, size_t cells, void *temp, size_t temp_bytes, uint64_t *h_total,
                         cudaStream_t st) {
  SparseTemp o;
  if (sparse_layout(cells, 0, static_cast<char *>(temp), &o) > temp_bytes) return cudaErrorMemoryAllocation;
  const size_t tiles = (cells + kTile - 1) / kTile;
  k_tile_count<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(occ, cells, o.counts);
  note_launch();
  cudaError_t e = exclusive_scan_u32(o.counts, o.starts, tiles, Scratch{o.scratch, o.scratch_bytes}, st);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(h_total, o.starts + tiles, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

// After sparse_count: writes the `total` occupied cell indices, ordered by (first triangle, cell),
// into cells_out (device, total uint32). tri_bits = bits needed for a triangle index.
cudaError_t sparse_emit(const uint8_t *occ, const uint32_t *first_tri, size_t cells, uint64_t total, int tri_bits,
                        void *temp, size_t temp_bytes, uint32_t *cells_out, cudaStream_t st) {
  SparseTemp o;
  if (sparse_layout(cells, total, static_cast<char *>(temp), &o) > temp_bytes) return cudaErrorMemoryAllocation;
  const size_t tiles = (cells + kTile - 1) / kTile;
  // recount: the workspace may have been reallocated since sparse_count
  k_tile_count<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(occ, cells, o.counts);
  note_launch();
  cudaError_t e0 = exclusive_scan_u32(o.counts, o.starts, tiles, Scratch{o.scratch, o.scratch_bytes}, st);
  if (e0 != cudaSuccess) return e0;
  k_tile_write<<<static_cast<unsigned>(tiles), kThreads, 0, st>>>(occ, first_tri, cells, o.starts, o.keys, cells_out);
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return radix_sort_pairs(o.keys, cells_out, o.keys_alt, o.vals_alt, total, tri_bits,
                          Scratch{o.scratch, o.scratch_bytes}, st);
}

}  // namespace sdfb
