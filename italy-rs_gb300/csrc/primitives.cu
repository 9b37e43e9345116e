// Device-wide primitives used by the bake: exclusive scan and a stable LSD radix sort.
//
// Scan: tiles of 4096 counts (256 threads x 16), scanned per block, tile sums scanned
// recursively, then added back. Radix sort: 8-bit digits; per pass a per-tile histogram, one
// scan of the digit-major histogram matrix, and a stable scatter in which every tile walks its
// keys in 8 rounds of 256 (coalesced loads, positions increasing with round then thread) and
// ranks equal digits with __match_any_sync inside a warp plus per-warp counts across the block.
#include <algorithm>
#include <cstdint>
#include <utility>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr size_t kScanTile = size_t(kScanThreads) * kScanItems;

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr size_t kSortTile = size_t(kSortThreads) * kSortRounds;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Bump {
  char *p;
  size_t left;
  template <typename T> T *take(size_t count) {
    const size_t b = align256(count * sizeof(T));
    if (b > left) return nullptr;
    T *r = reinterpret_cast<T *>(p);
    p += b;
    left -= b;
    return r;
  }
};

// Block-wide exclusive scan of one uint64 per thread; returns the block total in *total.
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t *total) {
  __shared__ uint64_t warp_tot[kScanThreads / kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t n = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < kScanThreads / kWarp ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t n = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += n;
    }
    if (lane < kScanThreads / kWarp) warp_tot[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const uint64_t warp_base = warp ? warp_tot[warp - 1] : 0;
  *total = warp_tot[kScanThreads / kWarp - 1];
  return warp_base + incl - v;
}

template <typename Tin>
__global__ __launch_bounds__(kScanThreads) void k_scan_tiles(const Tin *__restrict__ in, uint64_t *__restrict__ out,
                                                             uint64_t *__restrict__ tile_sums, size_t n) {
  const size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanItems;
  uint64_t v[kScanItems];
  uint64_t sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    const size_t k = base + i;
    v[i] = k < n ? static_cast<uint64_t>(in[k]) : 0;
    sum += v[i];
  }
  uint64_t total;
  uint64_t run = block_exclusive_scan(sum, &total);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    const size_t k = base + i;
    if (k < n) out[k] = run;
    run += v[i];
  }
  if (threadIdx.x == 0) {
    if (tile_sums) tile_sums[blockIdx.x] = total;
    if (gridDim.x == 1) out[n] = total;
  }
}

__global__ void k_add_tile_offsets(uint64_t *__restrict__ out, const uint64_t *__restrict__ offs, size_t n,
                                   size_t ntiles) {
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) out[i] += offs[i / kScanTile];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = offs[ntiles];
}

template <typename Tin>
cudaError_t scan_impl(const Tin *in, uint64_t *out, size_t n, Bump &b, cudaStream_t st) {
  if (n == 0) return cudaMemsetAsync(out, 0, sizeof(uint64_t), st);
  const size_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 1) {
    k_scan_tiles<Tin><<<1, kScanThreads, 0, st>>>(in, out, nullptr, n);
    note_launch();
    return cudaGetLastError();
  }
  uint64_t *sums = b.take<uint64_t>(ntiles);
  uint64_t *offs = b.take<uint64_t>(ntiles + 1);
  if (!sums || !offs) return cudaErrorMemoryAllocation;
  k_scan_tiles<Tin><<<static_cast<unsigned>(ntiles), kScanThreads, 0, st>>>(in, out, sums, n);
  note_launch();
  cudaError_t e = scan_impl<uint64_t>(sums, offs, ntiles, b, st);
  if (e != cudaSuccess) return e;
  const unsigned blocks = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, 4096));
  k_add_tile_offsets<<<blocks, 256, 0, st>>>(out, offs, n, ntiles);
  note_launch();
  return cudaGetLastError();
}

// ---- radix sort -------------------------------------------------------------------------------

__global__ __launch_bounds__(kSortThreads) void k_sort_hist(const uint64_t *__restrict__ keys, size_t n, int shift,
                                                            uint32_t *__restrict__ hist, size_t ntiles) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = size_t(blockIdx.x) * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    const size_t pos = base + size_t(r) * kSortThreads + threadIdx.x;
    if (pos < n) atomicAdd(&cnt[(keys[pos] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[size_t(threadIdx.x) * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ __launch_bounds__(kSortThreads) void k_sort_scatter(const uint64_t *__restrict__ kin,
                                                               const uint32_t *__restrict__ vin,
                                                               uint64_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                               size_t n, int shift, const uint64_t *__restrict__ offs,
                                                               size_t ntiles) {
  constexpr int kWarps = kSortThreads / kWarp;
  __shared__ uint64_t running[256];
  __shared__ uint32_t wcnt[kWarps][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  running[tid] = offs[size_t(tid) * ntiles + blockIdx.x];
#pragma unroll
  for (int w = 0; w < kWarps; ++w) wcnt[w][tid] = 0;
  __syncthreads();
  const size_t base = size_t(blockIdx.x) * kSortTile;
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortRounds; ++r) {
    const size_t pos = base + size_t(r) * kSortThreads + tid;
    const bool valid = pos < n;
    uint64_t key = 0;
    uint32_t val = 0;
    if (valid) {
      key = kin[pos];
      val = vin[pos];
    }
    const uint32_t digit = valid ? static_cast<uint32_t>((key >> shift) & 255u) : 256u;
    const uint32_t peers = __match_any_sync(kFull, digit);
    const uint32_t rank = __popc(peers & lt_mask);
    const bool leader = (__ffs(peers) - 1) == lane;
    if (leader && valid) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint64_t off = running[digit] + rank;
      for (int w = 0; w < warp; ++w) off += wcnt[w][digit];
      kout[off] = key;
      vout[off] = val;
    }
    __syncthreads();
    uint32_t add = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      add += wcnt[w][tid];
      wcnt[w][tid] = 0;
    }
    running[tid] += add;
    __syncthreads();
  }
}

}  // namespace

size_t scan_scratch_bytes(size_t n) {
  size_t total = 0;
  size_t m = n;
  while (m > kScanTile) {
    const size_t t = (m + kScanTile - 1) / kScanTile;
    total += align256(t * sizeof(uint64_t)) + align256((t + 1) * sizeof(uint64_t));
    m = t;
  }
  return total + 1024;
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint64_t *out, size_t n, Scratch s, cudaStream_t st) {
  Bump b{static_cast<char *>(s.ptr), s.bytes};
  return scan_impl<uint32_t>(in, out, n, b, st);
}

cudaError_t exclusive_scan_u64(const uint64_t *in, uint64_t *out, size_t n, Scratch s, cudaStream_t st) {
  Bump b{static_cast<char *>(s.ptr), s.bytes};
  return scan_impl<uint64_t>(in, out, n, b, st);
}

size_t sort_scratch_bytes(size_t n) {
  const size_t ntiles = (n + kSortTile - 1) / kSortTile;
  const size_t cells = ntiles * 256;
  return align256(cells * sizeof(uint32_t)) + align256((cells + 1) * sizeof(uint64_t)) + scan_scratch_bytes(cells);
}

cudaError_t radix_sort_pairs(uint64_t *keys, uint32_t *vals, uint64_t *keys_alt, uint32_t *vals_alt, size_t n,
                             int bits, Scratch s, cudaStream_t st) {
  if (n <= 1 || bits <= 0) return cudaSuccess;
  const size_t ntiles = (n + kSortTile - 1) / kSortTile;
  const size_t cells = ntiles * 256;
  Bump b{static_cast<char *>(s.ptr), s.bytes};
  uint32_t *hist = b.take<uint32_t>(cells);
  uint64_t *offs = b.take<uint64_t>(cells + 1);
  if (!hist || !offs) return cudaErrorMemoryAllocation;
  uint64_t *ka = keys, *kb = keys_alt;
  uint32_t *va = vals, *vb = vals_alt;
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, ++passes) {
    k_sort_hist<<<static_cast<unsigned>(ntiles), kSortThreads, 0, st>>>(ka, n, shift, hist, ntiles);
    note_launch();
    Bump bs = b;
    cudaError_t e = scan_impl<uint32_t>(hist, offs, cells, bs, st);
    if (e != cudaSuccess) return e;
    k_sort_scatter<<<static_cast<unsigned>(ntiles), kSortThreads, 0, st>>>(ka, va, kb, vb, n, shift, offs, ntiles);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (passes & 1) {
    cudaError_t e = cudaMemcpyAsync(keys, ka, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  }
  return cudaSuccess;
}

}  // namespace sdfb
