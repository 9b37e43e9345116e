// Soup -> indexed weld and the watertight gate on the device (weldPositions,
// src/io/mesh_weld.cpp:26-48; isWatertight, src/io/mesh_validate.cpp:21-59), so that large soups
// are welded where they already are.
//
// Weld: every position gets the lattice key lround(p / cell) per axis (FP32 division, round half
// away from zero, as std::lround); three stable LSD radix sorts -- by z, then y, then x key, each
// biased to unsigned and cut to the bits its range needs -- order the positions by key with equal
// keys in position order. The first position of each run of equal keys is the key's first
// occurrence; an exclusive scan of first-occurrence flags in position order numbers the unique
// keys in first-occurrence order, which is the reference's numbering (a hash map filled in
// position order). Every position of a run takes its first position's number.
//
// Watertight: each non-degenerate triangle contributes its three undirected edges
// (min << b | max, b = bits of the unique count); degenerate ones contribute a sentinel above
// every edge. After a radix sort, each run of equal edges is one edge with its use count:
// 1 = boundary, > 2 = non-manifold.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "api_internal.h"
#include "common.cuh"
#include "host_mesh.h"
#include "kernels.h"

using namespace sdfb;

namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

inline unsigned grid_for(uint64_t n, int num_sms) {
  return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + kThreads - 1) / kThreads,
                                                                         uint64_t(num_sms) * 16)));
}

// Lattice keys and their per-axis minimum / maximum (as order-preserving unsigned values).
__global__ __launch_bounds__(kThreads) void k_weld_keys(const float *__restrict__ pos, uint64_t n, float cell,
                                                        long long *__restrict__ keys,
                                                        unsigned long long *__restrict__ range) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const long long k = llroundf(__fdiv_rn(pos[3 * i + a], cell));
      keys[a * n + i] = k;
      const unsigned long long u = static_cast<unsigned long long>(k) ^ (1ull << 63);
      lo[a] = min(lo[a], u);
      hi[a] = max(hi[a], u);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = min(lo[a], __shfl_xor_sync(kFull, lo[a], o));
      hi[a] = max(hi[a], __shfl_xor_sync(kFull, hi[a], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(range + 2 * a, lo[a]);
      atomicMax(range + 2 * a + 1, hi[a]);
    }
  }
}

__global__ __launch_bounds__(kThreads) void k_iota(uint32_t *__restrict__ v, uint64_t n) {
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads)
    v[i] = static_cast<uint32_t>(i);
}

// sort key of axis `a` for the positions in the current order: (key - min) as unsigned
__global__ __launch_bounds__(kThreads) void k_axis_keys(const long long *__restrict__ keys, uint64_t n, int a,
                                                        const unsigned long long *__restrict__ range,
                                                        const uint32_t *__restrict__ order,
                                                        uint64_t *__restrict__ out) {
  const unsigned long long lo = range[2 * a];
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const unsigned long long u = static_cast<unsigned long long>(keys[a * n + order[r]]) ^ (1ull << 63);
    out[r] = u - lo;
  }
}

__device__ __forceinline__ bool same_key(const long long *keys, uint64_t n, uint32_t i, uint32_t j) {
  return keys[i] == keys[j] && keys[n + i] == keys[n + j] && keys[2 * n + i] == keys[2 * n + j];
}

// flag[first position of each run] = 1 (the runs' first elements have the smallest index).
__global__ __launch_bounds__(kThreads) void k_first(const long long *__restrict__ keys, uint64_t n,
                                                    const uint32_t *__restrict__ order, uint32_t *__restrict__ flag) {
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const uint32_t i = order[r];
    flag[i] = (r == 0 || !same_key(keys, n, i, order[r - 1])) ? 1u : 0u;
  }
}

// Every position of a run takes the number of the run's first position.
// first_of[id] (optional) receives the position index of the id's first occurrence.
__global__ __launch_bounds__(kThreads) void k_assign(const long long *__restrict__ keys, uint64_t n,
                                                     const uint32_t *__restrict__ order,
                                                     const uint64_t *__restrict__ number,
                                                     uint32_t *__restrict__ welded, uint32_t *__restrict__ first_of) {
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const uint32_t i = order[r];
    if (r > 0 && same_key(keys, n, i, order[r - 1])) continue;
    const uint32_t id = static_cast<uint32_t>(number[i]);
    if (first_of) first_of[id] = i;
    for (uint64_t j = r; j < n && (j == r || same_key(keys, n, i, order[j])); ++j) welded[order[j]] = id;
  }
}

// Edge key (lo << b) | hi with b bits per index; the sentinel 1 << 2b sorts after every edge.
__global__ __launch_bounds__(kThreads) void k_edges(const uint32_t *__restrict__ w, uint64_t T, int bits,
                                                    uint64_t *__restrict__ edges, uint32_t *__restrict__ vals) {
  for (uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x; t < T; t += uint64_t(gridDim.x) * kThreads) {
    const uint32_t a = w[3 * t], b = w[3 * t + 1], c = w[3 * t + 2];
    const bool degenerate = a == b || b == c || c == a;
    const uint32_t v[3][2] = {{a, b}, {b, c}, {c, a}};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint32_t lo = min(v[k][0], v[k][1]), hi = max(v[k][0], v[k][1]);
      edges[3 * t + k] = degenerate ? (bits == 32 ? ~0ull : (1ull << (2 * bits))) : ((uint64_t(lo) << bits) | hi);
      vals[3 * t + k] = 0;
    }
  }
}

// counts[0] = boundary edges (used once), counts[1] = non-manifold edges (used more than twice)
__global__ __launch_bounds__(kThreads) void k_edge_runs(const uint64_t *__restrict__ e, uint64_t n, uint64_t sentinel,
                                                        unsigned long long *__restrict__ counts) {
  unsigned long long bnd = 0, nm = 0;
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const uint64_t k = e[r];
    if (k == sentinel || (r > 0 && e[r - 1] == k)) continue;
    uint64_t j = r + 1;
    while (j < n && e[j] == k && j - r <= 2) ++j;
    const uint64_t c = j - r;
    bnd += c == 1;
    nm += c > 2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    bnd += __shfl_xor_sync(kFull, bnd, o);
    nm += __shfl_xor_sync(kFull, nm, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bnd) atomicAdd(counts, bnd);
    if (nm) atomicAdd(counts + 1, nm);
  }
}

int bits_of(unsigned long long range) {
  int b = 0;
  while (b < 64 && (range >> b) != 0) ++b;
  return b;
}

// Vertex bounds as order-preserving unsigned values: out[0..2] minima, out[3..5] maxima.
__global__ __launch_bounds__(kThreads) void k_bounds(const float *__restrict__ v, uint64_t n,
                                                     unsigned int *__restrict__ out) {
  unsigned int lo[3] = {~0u, ~0u, ~0u}, hi[3] = {0, 0, 0};
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const unsigned int u = float_to_ordered(v[3 * i + a]);
      lo[a] = min(lo[a], u);
      hi[a] = max(hi[a], u);
    }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = min(lo[a], __shfl_xor_sync(kFull, lo[a], o));
      hi[a] = max(hi[a], __shfl_xor_sync(kFull, hi[a], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(out + a, lo[a]);
      atomicMax(out + 3 + a, hi[a]);
    }
  }
}

// Triangle corners through the vertex weld; err = 1 when an index is out of range.
__global__ __launch_bounds__(kThreads) void k_map_tris(const uint32_t *__restrict__ idx, uint64_t n, uint32_t V,
                                                       const uint32_t *__restrict__ wv, uint32_t *__restrict__ tri,
                                                       unsigned int *__restrict__ err) {
  for (uint64_t k = uint64_t(blockIdx.x) * kThreads + threadIdx.x; k < n; k += uint64_t(gridDim.x) * kThreads) {
    const uint32_t i = idx[k];
    if (i >= V) {
      *err = 1;
      tri[k] = 0;
    } else {
      tri[k] = wv[i];
    }
  }
}

__global__ __launch_bounds__(kThreads) void k_gather_unique(const float *__restrict__ pos,
                                                            const uint32_t *__restrict__ first_of, uint64_t U,
                                                            float *__restrict__ out) {
  for (uint64_t u = uint64_t(blockIdx.x) * kThreads + threadIdx.x; u < U; u += uint64_t(gridDim.x) * kThreads) {
    const uint64_t i = first_of[u];
    out[3 * u] = pos[3 * i];
    out[3 * u + 1] = pos[3 * i + 1];
    out[3 * u + 2] = pos[3 * i + 2];
  }
}

}  // namespace

namespace sdfb {

cudaError_t gather_unique(const float *pos, const uint32_t *first_of, uint64_t U, float *out, int num_sms,
                          cudaStream_t st) {
  if (U == 0) return cudaSuccess;
  k_gather_unique<<<grid_for(U, num_sms), kThreads, 0, st>>>(pos, first_of, U, out);
  note_launch();
  return cudaGetLastError();
}


size_t weld_temp_bytes(uint64_t n) {
  return align256(n * 24) + align256(48) + 2 * align256(n * 8) + 2 * align256(n * 4) + align256(n * 4) +
         align256((n + 1) * 8) + std::max(sort_scratch_bytes(n), scan_scratch_bytes(n));
}

cudaError_t weld_device(const float *pos, uint64_t n, float cell, uint32_t *welded, uint32_t *first_of, void *temp,
                        size_t temp_bytes, uint32_t *num_unique, int num_sms, cudaStream_t st) {
  *num_unique = 0;
  if (n == 0) return cudaSuccess;
  if (temp_bytes < weld_temp_bytes(n)) return cudaErrorMemoryAllocation;
  char *p = static_cast<char *>(temp);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += align256(bytes);
    return r;
  };
  long long *keys = reinterpret_cast<long long *>(take(n * 24));
  unsigned long long *range = reinterpret_cast<unsigned long long *>(take(48));
  uint64_t *sk = reinterpret_cast<uint64_t *>(take(n * 8));
  uint64_t *sk_alt = reinterpret_cast<uint64_t *>(take(n * 8));
  uint32_t *order = reinterpret_cast<uint32_t *>(take(n * 4));
  uint32_t *order_alt = reinterpret_cast<uint32_t *>(take(n * 4));
  uint32_t *flag = reinterpret_cast<uint32_t *>(take(n * 4));
  uint64_t *number = reinterpret_cast<uint64_t *>(take((n + 1) * 8));
  Scratch scratch{p, temp_bytes - size_t(p - static_cast<char *>(temp))};
  const unsigned long long init[6] = {~0ull, 0, ~0ull, 0, ~0ull, 0};
  cudaError_t e = cudaMemcpyAsync(range, init, sizeof init, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  k_weld_keys<<<grid_for(n, num_sms), kThreads, 0, st>>>(pos, n, cell, keys, range);
  note_launch();
  unsigned long long h_range[6];
  if ((e = cudaMemcpyAsync(h_range, range, sizeof h_range, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  k_iota<<<grid_for(n, num_sms), kThreads, 0, st>>>(order, n);
  note_launch();
  for (int a = 2; a >= 0; --a) {  // z, then y, then x: LSD order over the three fields
    const int bits = bits_of(h_range[2 * a + 1] - h_range[2 * a]);
    if (bits == 0) continue;
    k_axis_keys<<<grid_for(n, num_sms), kThreads, 0, st>>>(keys, n, a, range, order, sk);
    note_launch();
    if ((e = radix_sort_pairs(sk, order, sk_alt, order_alt, n, bits, scratch, st)) != cudaSuccess) return e;
  }
  k_first<<<grid_for(n, num_sms), kThreads, 0, st>>>(keys, n, order, flag);
  note_launch();
  if ((e = exclusive_scan_u32(flag, number, n, scratch, st)) != cudaSuccess) return e;
  k_assign<<<grid_for(n, num_sms), kThreads, 0, st>>>(keys, n, order, number, welded, first_of);
  note_launch();
  uint64_t total = 0;
  if ((e = cudaMemcpyAsync(&total, number + n, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *num_unique = static_cast<uint32_t>(total);
  return cudaGetLastError();
}

size_t indexed_gate_temp_bytes(uint64_t V, uint64_t T) {
  return align256(64) + align256(V * 4) + align256(T * 12) + std::max(weld_temp_bytes(V), watertight_temp_bytes(T));
}

cudaError_t indexed_watertight_device(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, void *temp,
                                      size_t temp_bytes, int *result, int num_sms, cudaStream_t st) {
  *result = 0;
  if (V == 0 || T == 0) return cudaSuccess;
  if (temp_bytes < indexed_gate_temp_bytes(V, T)) return cudaErrorMemoryAllocation;
  char *p = static_cast<char *>(temp);
  unsigned int *misc = reinterpret_cast<unsigned int *>(p);  // bounds [6], error flag [6]
  uint32_t *wv = reinterpret_cast<uint32_t *>(p + align256(64));
  uint32_t *tri = reinterpret_cast<uint32_t *>(p + align256(64) + align256(uint64_t(V) * 4));
  char *rest = p + align256(64) + align256(uint64_t(V) * 4) + align256(uint64_t(T) * 12);
  const size_t rest_bytes = temp_bytes - size_t(rest - p);
  const unsigned int init[7] = {~0u, ~0u, ~0u, 0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(misc, init, sizeof init, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  k_bounds<<<grid_for(V, num_sms), kThreads, 0, st>>>(verts, V, misc);
  note_launch();
  unsigned int hb[6];
  if ((e = cudaMemcpyAsync(hb, misc, sizeof hb, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  float bmin[3], bmax[3];
  for (int a = 0; a < 3; ++a) {
    bmin[a] = ordered_to_float(hb[a]);
    bmax[a] = ordered_to_float(hb[3 + a]);
  }
  uint32_t U = 0;
  if ((e = weld_device(verts, V, weld_cell(bmin, bmax), wv, nullptr, rest, rest_bytes, &U, num_sms, st)) != cudaSuccess)
    return e;
  k_map_tris<<<grid_for(uint64_t(T) * 3, num_sms), kThreads, 0, st>>>(idx, uint64_t(T) * 3, V, wv, tri, misc + 6);
  note_launch();
  unsigned int bad = 0;
  if ((e = cudaMemcpyAsync(&bad, misc + 6, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  if (bad) {
    *result = -2;
    return cudaSuccess;
  }
  uint64_t b = 0, m = 0;
  if ((e = watertight_device(tri, T, U, rest, rest_bytes, &b, &m, num_sms, st)) != cudaSuccess) return e;
  *result = (b == 0 && m == 0) ? 1 : 0;
  return cudaSuccess;
}

size_t watertight_temp_bytes(uint64_t T) {
  const uint64_t n = 3 * T;
  return 2 * align256(n * 8) + 2 * align256(n * 4) + align256(16) + sort_scratch_bytes(n);
}

cudaError_t watertight_device(const uint32_t *welded, uint64_t T, uint32_t num_unique, void *temp, size_t temp_bytes,
                              uint64_t *boundary, uint64_t *nonmanifold, int num_sms, cudaStream_t st) {
  *boundary = *nonmanifold = 0;
  if (T == 0) return cudaSuccess;
  if (temp_bytes < watertight_temp_bytes(T)) return cudaErrorMemoryAllocation;
  const uint64_t n = 3 * T;
  char *p = static_cast<char *>(temp);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += align256(bytes);
    return r;
  };
  uint64_t *edges = reinterpret_cast<uint64_t *>(take(n * 8));
  uint64_t *edges_alt = reinterpret_cast<uint64_t *>(take(n * 8));
  uint32_t *vals = reinterpret_cast<uint32_t *>(take(n * 4));
  uint32_t *vals_alt = reinterpret_cast<uint32_t *>(take(n * 4));
  unsigned long long *counts = reinterpret_cast<unsigned long long *>(take(16));
  Scratch scratch{p, temp_bytes - size_t(p - static_cast<char *>(temp))};
  cudaError_t e = cudaMemsetAsync(counts, 0, 16, st);
  if (e != cudaSuccess) return e;
  // b bits per index when every index is below num_unique; 0 = unknown: full 32-bit indices (a
  // non-degenerate edge has lo < hi, so its key stays below the all-ones sentinel)
  int b = 1;
  while (b < 31 && (uint64_t(1) << b) < num_unique) ++b;
  if (num_unique == 0 || num_unique > (1u << 30)) b = 32;
  k_edges<<<grid_for(T, num_sms), kThreads, 0, st>>>(welded, T, b, edges, vals);
  note_launch();
  const int key_bits = b == 32 ? 64 : 2 * b + 1;
  const uint64_t sentinel = b == 32 ? ~0ull : (1ull << (2 * b));
  if ((e = radix_sort_pairs(edges, vals, edges_alt, vals_alt, n, key_bits, scratch, st)) != cudaSuccess) return e;
  k_edge_runs<<<grid_for(n, num_sms), kThreads, 0, st>>>(edges, n, sentinel, counts);
  note_launch();
  unsigned long long h[2];
  if ((e = cudaMemcpyAsync(h, counts, sizeof h, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *boundary = h[0];
  *nonmanifold = h[1];
  return cudaGetLastError();
}

}  // namespace sdfb
