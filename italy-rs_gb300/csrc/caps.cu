// Boundary caps of an indexed mesh, built on the device, for the winding-number sign.
//
// The caps close every boundary loop of the mesh with a fan around the loop's vertex mean, so that
// mesh + caps has no boundary and its winding number is the integer count of signed +z crossings
// (gwn.cu). The boundary is the net directed edge chain of the triangles' index topology (the
// edge rule of src/io/mesh_validate.cpp:21-59, with directions): an undirected edge {u, v} used n1
// times as u->v and n2 times as v->u leaves |n1 - n2| boundary half-edges. At every vertex as many
// boundary half-edges arrive as leave, so they form closed loops.
//
//   k_cap_edges     one key per directed edge (low index, high index) and its direction
//   radix sort      equal undirected edges become runs
//   k_cap_runs      net multiplicity of each run; scan -> boundary half-edge slots
//   k_cap_emit      boundary half-edges (tail, head)
//   2 radix sorts   half-edges by tail and by head
//   k_cap_pair      the successor of a half-edge arriving at x is the outgoing half-edge of x of
//                   the same rank (any pairing closes the loops; this one is deterministic)
//   k_cap_jump      pointer jumping: every half-edge learns the smallest index on its cycle
//   radix sort      half-edges grouped by cycle, in index order within a cycle
//   k_cap_loops     loop numbers (a scan over cycle starts), loop means summed in FP64 in that
//                   order, and one fan triangle (head, tail, centre) per half-edge
//
// Any closing caps give the same winding number of the mesh itself, so the pairing at vertices
// where several loops meet does not change a sign. Every size is bounded by 3T; kernels read the
// data-dependent counts from device memory, and the caller reads the two totals once.
#include <algorithm>
#include <cstdint>

#include "api_internal.h"
#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

inline unsigned grid_for(uint64_t n, int num_sms) {
  return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + kThreads - 1) / kThreads,
                                                                         uint64_t(num_sms) * 16)));
}

struct CapTemp {
  uint64_t *keys, *keys_alt;
  uint32_t *vals, *vals_alt;
  uint32_t *cnt;
  uint64_t *starts;
  uint2 *half;  // boundary half-edges (tail, head)
  uint32_t *out_order, *in_order;
  uint64_t *out_keys, *in_keys;
  uint32_t *succ, *nxt, *nxt2, *lab, *lab2;
  uint32_t *loop_flag;
  uint64_t *loop_start;
  void *scratch;
  size_t scratch_bytes;
};

size_t cap_layout(uint64_t T, char *base, CapTemp *o) {
  const uint64_t n = std::max<uint64_t>(3 * T, 1);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  CapTemp x;
  x.keys = reinterpret_cast<uint64_t *>(take(n * 8));
  x.keys_alt = reinterpret_cast<uint64_t *>(take(n * 8));
  x.vals = reinterpret_cast<uint32_t *>(take(n * 4));
  x.vals_alt = reinterpret_cast<uint32_t *>(take(n * 4));
  x.cnt = reinterpret_cast<uint32_t *>(take(n * 4));
  x.starts = reinterpret_cast<uint64_t *>(take((n + 1) * 8));
  x.half = reinterpret_cast<uint2 *>(take(n * 8));
  x.out_order = reinterpret_cast<uint32_t *>(take(n * 4));
  x.in_order = reinterpret_cast<uint32_t *>(take(n * 4));
  x.out_keys = reinterpret_cast<uint64_t *>(take(n * 8));
  x.in_keys = reinterpret_cast<uint64_t *>(take(n * 8));
  x.succ = reinterpret_cast<uint32_t *>(take(n * 4));
  x.nxt = reinterpret_cast<uint32_t *>(take(n * 4));
  x.nxt2 = reinterpret_cast<uint32_t *>(take(n * 4));
  x.lab = reinterpret_cast<uint32_t *>(take(n * 4));
  x.lab2 = reinterpret_cast<uint32_t *>(take(n * 4));
  x.loop_flag = reinterpret_cast<uint32_t *>(take(n * 4));
  x.loop_start = reinterpret_cast<uint64_t *>(take((n + 1) * 8));
  x.scratch_bytes = std::max(sort_scratch_bytes(n), scan_scratch_bytes(n));
  x.scratch = take(x.scratch_bytes);
  if (o) *o = x;
  return off;
}

// Directed edge a->b of every triangle as (lo << bits | hi, direction): 1 for lo->hi. Edges with a
// == b, or with an index >= V (flagged), get the sentinel key, which sorts last.
__global__ __launch_bounds__(kThreads) void k_cap_edges(const uint32_t *__restrict__ idx, uint64_t T, uint32_t V,
                                                        int bits, uint64_t sentinel, uint64_t *__restrict__ keys,
                                                        uint32_t *__restrict__ dir, uint32_t *__restrict__ err) {
  for (uint64_t e = uint64_t(blockIdx.x) * kThreads + threadIdx.x; e < 3 * T; e += uint64_t(gridDim.x) * kThreads) {
    const uint64_t t = e / 3;
    const int k = static_cast<int>(e % 3);
    const uint32_t a = __ldg(idx + 3 * t + k), b = __ldg(idx + 3 * t + (k + 1) % 3);
    const uint32_t lo = min(a, b), hi = max(a, b);
    const bool bad = a >= V || b >= V;
    if (bad) atomic_or_err(err, kErrBadIndex);
    keys[e] = (a == b || bad) ? sentinel : ((uint64_t(lo) << bits) | hi);
    dir[e] = a < b ? 1u : 0u;
  }
}

// At each run start of the sorted edges: the number of boundary half-edges |uses lo->hi - uses
// hi->lo| in cnt and their direction in sign (1: hi->lo); cnt is 0 elsewhere.
__global__ __launch_bounds__(kThreads) void k_cap_runs(const uint64_t *__restrict__ keys,
                                                       const uint32_t *__restrict__ dir, uint64_t n,
                                                       uint64_t sentinel, uint32_t *__restrict__ cnt,
                                                       uint32_t *__restrict__ sign) {
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const uint64_t k = keys[r];
    if (k == sentinel || (r > 0 && keys[r - 1] == k)) {
      cnt[r] = 0;
      continue;
    }
    long long net = 0;
    for (uint64_t j = r; j < n && keys[j] == k; ++j) net += dir[j] ? 1 : -1;
    cnt[r] = static_cast<uint32_t>(net < 0 ? -net : net);
    sign[r] = net < 0 ? 1u : 0u;
  }
}

__global__ __launch_bounds__(kThreads) void k_cap_emit(const uint64_t *__restrict__ keys,
                                                       const uint32_t *__restrict__ cnt,
                                                       const uint32_t *__restrict__ sign,
                                                       const uint64_t *__restrict__ starts, uint64_t n, int bits,
                                                       uint2 *__restrict__ half) {
  const uint64_t mask = (uint64_t(1) << bits) - 1;
  for (uint64_t r = uint64_t(blockIdx.x) * kThreads + threadIdx.x; r < n; r += uint64_t(gridDim.x) * kThreads) {
    const uint32_t c = cnt[r];
    if (c == 0) continue;
    const uint32_t lo = static_cast<uint32_t>(keys[r] >> bits), hi = static_cast<uint32_t>(keys[r] & mask);
    const uint2 h = sign[r] ? make_uint2(hi, lo) : make_uint2(lo, hi);
    for (uint32_t j = 0; j < c; ++j) half[starts[r] + j] = h;
  }
}

// Sort keys of the half-edges by tail (which = 0) or head (1); slots past the count sort last.
__global__ __launch_bounds__(kThreads) void k_cap_end_keys(const uint2 *__restrict__ half,
                                                           const uint64_t *__restrict__ total, uint64_t n, int which,
                                                           uint64_t sentinel, uint64_t *__restrict__ keys,
                                                           uint32_t *__restrict__ vals) {
  const uint64_t nb = *total;
  for (uint64_t h = uint64_t(blockIdx.x) * kThreads + threadIdx.x; h < n; h += uint64_t(gridDim.x) * kThreads) {
    keys[h] = h < nb ? uint64_t(which ? half[h].y : half[h].x) : sentinel;
    vals[h] = static_cast<uint32_t>(h);
  }
}

__device__ __forceinline__ uint64_t lower_bound64(const uint64_t *__restrict__ a, uint64_t n, uint64_t x) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The successor of the rank-r half-edge arriving at x is the rank-r half-edge leaving x. A vertex
// whose counts differ (impossible for index topology) raises the corrupt-tree flag and points the
// half-edge at itself.
__global__ __launch_bounds__(kThreads) void k_cap_pair(const uint64_t *__restrict__ in_keys,
                                                       const uint32_t *__restrict__ in_order,
                                                       const uint64_t *__restrict__ out_keys,
                                                       const uint32_t *__restrict__ out_order,
                                                       const uint64_t *__restrict__ total, uint32_t *__restrict__ succ,
                                                       uint32_t *__restrict__ lab, uint32_t *__restrict__ err) {
  const uint64_t nb = *total;
  for (uint64_t j = uint64_t(blockIdx.x) * kThreads + threadIdx.x; j < nb; j += uint64_t(gridDim.x) * kThreads) {
    const uint64_t x = in_keys[j];
    const uint64_t rank = j - lower_bound64(in_keys, nb, x);
    const uint64_t at = lower_bound64(out_keys, nb, x) + rank;
    const uint32_t h = in_order[j];
    if (at < nb && out_keys[at] == x) {
      succ[h] = out_order[at];
    } else {
      succ[h] = h;
      atomic_or_err(err, kErrCorruptTree);
    }
    lab[h] = h;
  }
}

// One doubling step: lab2 = min(lab, lab[nxt]), nxt2 = nxt[nxt].
__global__ __launch_bounds__(kThreads) void k_cap_jump(const uint32_t *__restrict__ nxt,
                                                       const uint32_t *__restrict__ lab,
                                                       const uint64_t *__restrict__ total, uint32_t *__restrict__ nxt2,
                                                       uint32_t *__restrict__ lab2) {
  const uint64_t nb = *total;
  for (uint64_t h = uint64_t(blockIdx.x) * kThreads + threadIdx.x; h < nb; h += uint64_t(gridDim.x) * kThreads) {
    const uint32_t m = nxt[h];
    lab2[h] = min(lab[h], lab[m]);
    nxt2[h] = nxt[m];
  }
}

__global__ __launch_bounds__(kThreads) void k_cap_cycle_keys(const uint32_t *__restrict__ lab,
                                                             const uint64_t *__restrict__ total, uint64_t n,
                                                             uint64_t sentinel, uint64_t *__restrict__ keys,
                                                             uint32_t *__restrict__ vals) {
  const uint64_t nb = *total;
  for (uint64_t h = uint64_t(blockIdx.x) * kThreads + threadIdx.x; h < n; h += uint64_t(gridDim.x) * kThreads) {
    keys[h] = h < nb ? uint64_t(lab[h]) : sentinel;
    vals[h] = static_cast<uint32_t>(h);
  }
}

__global__ __launch_bounds__(kThreads) void k_cap_loop_flags(const uint64_t *__restrict__ keys,
                                                             const uint64_t *__restrict__ total, uint64_t n,
                                                             uint32_t *__restrict__ flag) {
  const uint64_t nb = *total;
  for (uint64_t j = uint64_t(blockIdx.x) * kThreads + threadIdx.x; j < n; j += uint64_t(gridDim.x) * kThreads)
    flag[j] = (j < nb && (j == 0 || keys[j] != keys[j - 1])) ? 1u : 0u;
}

// Loop c starts at sorted position j (flag set): its centre, the mean of its half-edges' tails
// summed in FP64 in sorted order, becomes vertex V + c, and each of its half-edges (a -> b) gives
// the cap triangle (b, a, V + c).
__global__ __launch_bounds__(kThreads) void k_cap_loops(const float *__restrict__ verts, uint32_t V,
                                                        const uint2 *__restrict__ half,
                                                        const uint64_t *__restrict__ keys,
                                                        const uint32_t *__restrict__ order,
                                                        const uint32_t *__restrict__ flag,
                                                        const uint64_t *__restrict__ loop_start,
                                                        const uint64_t *__restrict__ total, float *__restrict__ centres,
                                                        uint32_t *__restrict__ cap_tris) {
  const uint64_t nb = *total;
  for (uint64_t j = uint64_t(blockIdx.x) * kThreads + threadIdx.x; j < nb; j += uint64_t(gridDim.x) * kThreads) {
    if (!flag[j]) continue;
    const uint64_t c = loop_start[j];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    uint64_t e = j;
    for (; e < nb && keys[e] == keys[j]; ++e) {
      const uint32_t t = half[order[e]].x;
      sx += double(verts[3ull * t]);
      sy += double(verts[3ull * t + 1]);
      sz += double(verts[3ull * t + 2]);
    }
    const double inv = 1.0 / double(e - j);
    centres[3 * c] = float(sx * inv);
    centres[3 * c + 1] = float(sy * inv);
    centres[3 * c + 2] = float(sz * inv);
    const uint32_t cv = V + static_cast<uint32_t>(c);
    for (uint64_t k = j; k < e; ++k) {
      const uint2 h = half[order[k]];
      cap_tris[3 * k] = h.y;
      cap_tris[3 * k + 1] = h.x;
      cap_tris[3 * k + 2] = cv;
    }
  }
}

__global__ void k_cap_totals(const uint64_t *__restrict__ starts, uint64_t n, const uint64_t *__restrict__ loop_start,
                             uint64_t *__restrict__ totals) {
  totals[0] = starts[n];
  totals[1] = loop_start[n];
}

int bits_for_index(uint64_t V) {
  int b = 1;
  while (b < 32 && (uint64_t(1) << b) < V) ++b;
  return b;
}

}  // namespace
}  // namespace sdfb

using namespace sdfb;

size_t caps_temp_bytes(uint64_t T) { return cap_layout(T, nullptr, nullptr) + 256; }

cudaError_t caps_device(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T, void *temp,
                        size_t temp_bytes, float *centres, uint32_t *cap_tris, uint64_t *totals, uint32_t *err,
                        int num_sms, cudaStream_t st) {
  if (T == 0) return cudaMemsetAsync(totals, 0, 16, st);
  CapTemp t;
  if (cap_layout(T, static_cast<char *>(temp), &t) > temp_bytes) return cudaErrorMemoryAllocation;
  const uint64_t n = 3 * uint64_t(T);
  const Scratch sc{t.scratch, t.scratch_bytes};
  const int bits = bits_for_index(V);
  // every (lo << bits | hi) is below 2^(2 bits): the sentinel sorts last
  const int edge_bits = bits < 32 ? 2 * bits + 1 : 64;
  const uint64_t edge_sentinel = bits < 32 ? (uint64_t(1) << (2 * bits)) : ~0ull;
  const uint64_t end_sentinel = uint64_t(1) << 32;  // above every vertex index and half-edge label
  cudaError_t e;
  uint32_t *sign = t.vals_alt;  // free once the edge sort is done
  k_cap_edges<<<grid_for(n, num_sms), kThreads, 0, st>>>(idx, T, V, bits, edge_sentinel, t.keys, t.vals, err);
  note_launch();
  if ((e = radix_sort_pairs(t.keys, t.vals, t.keys_alt, t.vals_alt, n, edge_bits, sc, st)) != cudaSuccess) return e;
  k_cap_runs<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.keys, t.vals, n, edge_sentinel, t.cnt, sign);
  note_launch();
  if ((e = exclusive_scan_u32(t.cnt, t.starts, n, sc, st)) != cudaSuccess) return e;
  k_cap_emit<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.keys, t.cnt, sign, t.starts, n, bits, t.half);
  note_launch();
  const uint64_t *nb = t.starts + n;  // boundary half-edges
  // by tail
  k_cap_end_keys<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.half, nb, n, 0, end_sentinel, t.out_keys, t.out_order);
  note_launch();
  if ((e = radix_sort_pairs(t.out_keys, t.out_order, t.keys_alt, t.vals_alt, n, 33, sc, st)) != cudaSuccess) return e;
  // by head
  k_cap_end_keys<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.half, nb, n, 1, end_sentinel, t.in_keys, t.in_order);
  note_launch();
  if ((e = radix_sort_pairs(t.in_keys, t.in_order, t.keys_alt, t.vals_alt, n, 33, sc, st)) != cudaSuccess) return e;
  k_cap_pair<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.in_keys, t.in_order, t.out_keys, t.out_order, nb, t.succ,
                                                        t.lab, err);
  note_launch();
  // pointer jumping: after r rounds every half-edge knows the smallest index among its next 2^r
  const uint32_t *nx = t.succ;
  uint32_t *lab = t.lab, *lab2 = t.lab2, *nxa = t.nxt, *nxb = t.nxt2;
  int rounds = 1;
  while (rounds < 40 && (uint64_t(1) << rounds) < n) ++rounds;
  for (int r = 0; r < rounds; ++r) {
    k_cap_jump<<<grid_for(n, num_sms), kThreads, 0, st>>>(nx, lab, nb, nxa, lab2);
    note_launch();
    std::swap(lab, lab2);
    nx = nxa;
    std::swap(nxa, nxb);
  }
  // group by cycle
  k_cap_cycle_keys<<<grid_for(n, num_sms), kThreads, 0, st>>>(lab, nb, n, end_sentinel, t.keys, t.vals);
  note_launch();
  if ((e = radix_sort_pairs(t.keys, t.vals, t.keys_alt, t.vals_alt, n, 33, sc, st)) != cudaSuccess) return e;
  k_cap_loop_flags<<<grid_for(n, num_sms), kThreads, 0, st>>>(t.keys, nb, n, t.loop_flag);
  note_launch();
  if ((e = exclusive_scan_u32(t.loop_flag, t.loop_start, n, sc, st)) != cudaSuccess) return e;
  k_cap_loops<<<grid_for(n, num_sms), kThreads, 0, st>>>(verts, V, t.half, t.keys, t.vals, t.loop_flag, t.loop_start,
                                                         nb, centres, cap_tris);
  note_launch();
  k_cap_totals<<<1, 1, 0, st>>>(t.starts, n, t.loop_start, totals);
  note_launch();
  return cudaGetLastError();
}
