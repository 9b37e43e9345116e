// Sparse voxel list from a dense occupancy grid (the cell list of voxelizeMesh,
// src/convert/voxelize.cpp:52-107).
//
// Atomics-free per-tile compaction: k_tile_count counts occupied cells per 4096-cell tile (16 cells
// per thread, one 16-byte load each); a scan gives each tile its output offset; k_tile_write scans
// its tile inside the block and writes (first triangle, cell) pairs in cell order. A stable radix sort by first triangle then yields the
// reference's insertion order: a cell is inserted by the first triangle that hits it, and one
// triangle inserts its cells in z, y, x loop order, which is increasing cell index.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 16;  // one 16-byte load of the occupancy grid per thread
constexpr size_t kTile = size_t(kThreads) * kCellsPerThread;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Bit j set when cell base + j (j < 16) is occupied. The grid's base address is 256-byte aligned
// and base a multiple of 16, so a whole run of 16 cells is one aligned 16-byte load; a run that
// crosses the end of the grid is read byte by byte.
__device__ __forceinline__ uint32_t occupied_mask(const uint8_t *__restrict__ occ, size_t base, size_t cells) {
  uint32_t m = 0;
  if (base + kCellsPerThread <= cells) {
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(occ + base));
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const uint32_t ne = __vcmpne4(w[i], 0u);  // 0xff in every nonzero byte
#pragma unroll
      for (int b = 0; b < 4; ++b) m |= ((ne >> (8 * b + 7)) & 1u) << (4 * i + b);
    }
  } else {
    for (int j = 0; j < kCellsPerThread; ++j)
      if (base + j < cells && occ[base + j]) m |= 1u << j;
  }
  return m;
}

// Sum of v over the block; the result is valid in thread 0.
__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t *warp_sum) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / kWarp; ++w) s += warp_sum[w];
  return s;
}

__global__ __launch_bounds__(kThreads) void k_tile_count(const uint8_t *__restrict__ occ, size_t cells,
                                                         uint32_t *__restrict__ counts) {
  __shared__ uint32_t warp_sum[kThreads / kWarp];
  const size_t base = size_t(blockIdx.x) * kTile + size_t(threadIdx.x) * kCellsPerThread;
  uint32_t c;
  if (base + kCellsPerThread <= cells) {
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(occ + base));
    // 8 set bits per nonzero byte
    c = (__popc(__vcmpne4(q.x, 0u)) + __popc(__vcmpne4(q.y, 0u)) + __popc(__vcmpne4(q.z, 0u)) +
         __popc(__vcmpne4(q.w, 0u))) >> 3;
  } else {
    c = __popc(occupied_mask(occ, base, cells));
  }
  const uint32_t s = block_sum(c, warp_sum);
  if (threadIdx.x == 0) counts[blockIdx.x] = s;
}

// Each thread writes the (first triangle, cell) pairs of its 16 cells at its offset: the tile's
// start plus the occupied cells of the threads before it (a block-wide exclusive scan), so the
// pairs come out in cell order without atomics.
__global__ __launch_bounds__(kThreads) void k_tile_write(const uint8_t *__restrict__ occ,
                                                         const uint32_t *__restrict__ first_tri, size_t cells,
                                                         const uint64_t *__restrict__ tile_start,
                                                         uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  __shared__ uint32_t warp_sum[kThreads / kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t base = size_t(blockIdx.x) * kTile + size_t(threadIdx.x) * kCellsPerThread;
  uint32_t m = occupied_mask(occ, base, cells);
  const uint32_t c = __popc(m);
  uint32_t incl = c;  // inclusive scan within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t x = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += x;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  uint32_t before = incl - c;
  for (int w = 0; w < warp; ++w) before += warp_sum[w];
  uint64_t at = tile_start[blockIdx.x] + before;
  while (m) {
    const int j = __ffs(m) - 1;
    m &= m - 1;
    const size_t k = base + j;
    keys[at] = first_tri[k];
    vals[at] = static_cast<uint32_t>(k);
    ++at;
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
