// Device-built linear BVH over the triangles of a batch of meshes (replaces the OptiX GAS build
// of src/convert/sdf_baker.cpp:170-193, which builds one acceleration structure per call).
//
//   1. k_prep      gathers each indexed triangle of each mesh, checks indices and finiteness,
//                  writes its box (and, for the winding-number hierarchy, its 64-byte record), and
//                  reduces per-mesh centroid bounds.
//   2. k_morton    key = (mesh << 30) | 30-bit Morton code of the box centre in its mesh's bounds.
//   3. radix sort  (key, triangle) pairs, stable: meshes end up contiguous, each in Morton order.
//   4. k_hierarchy binary radix tree over all keys (Karras 2012, "Maximizing Parallelism in the
//                  Construction of BVHs, Octrees, and k-d Trees"; equal keys ordered by position).
//                  Since keys of one mesh share the mesh prefix, each mesh owns one subtree.
//   5. k_refit     bottom-up boxes: the second thread to reach a node merges its children.
//   6. k_layout    64-byte traversal nodes holding both child boxes; subtrees of at most the
//                  mesh's leaf size become leaves (their records are contiguous).
//   7. k_roots     one virtual root node per mesh, after the inner nodes, whose first child is
//                  the mesh's subtree (or leaf) and whose second child is empty; traversal of a
//                  mesh starts there.
//   8. k_gather    triangle records in leaf order: 80-byte frame records (DistTri) for the
//                  distance hierarchy, the k_prep records for the winding-number hierarchy.
//   9. k_moments   (optional) per inner node the sum of area x unit normal of its triangles and
//                  their total area (the winding number's far field, gwn.cu).
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct BuildTemp {
  TriRec *rec;      // T, global triangle order
  float4 *lo, *hi;  // T, triangle boxes (global triangle order)
  uint64_t *keys, *keys_alt;
  uint32_t *vals, *vals_alt;
  int2 *child;      // T - 1: (left, right); leaf children have the top bit set
  int2 *range;      // T - 1: covered sorted positions [first, last]
  int *iparent;     // T - 1
  int *lparent;     // T
  int *visits;      // T - 1
  float4 *ilo, *ihi;  // T - 1 inner boxes
  int *subtree;     // M: inner node covering exactly the mesh, -1 if none
  void *scratch;
  size_t scratch_bytes;
};

size_t temp_layout(uint64_t T, int M, char *base, BuildTemp *t) {
  const size_t n = std::max<uint64_t>(T, 1), m = std::max<uint64_t>(T, 2) - 1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  BuildTemp x;
  x.rec = reinterpret_cast<TriRec *>(take(n * sizeof(TriRec)));
  x.lo = reinterpret_cast<float4 *>(take(n * sizeof(float4)));
  x.hi = reinterpret_cast<float4 *>(take(n * sizeof(float4)));
  x.keys = reinterpret_cast<uint64_t *>(take(n * 8));
  x.keys_alt = reinterpret_cast<uint64_t *>(take(n * 8));
  x.vals = reinterpret_cast<uint32_t *>(take(n * 4));
  x.vals_alt = reinterpret_cast<uint32_t *>(take(n * 4));
  x.child = reinterpret_cast<int2 *>(take(m * sizeof(int2)));
  x.range = reinterpret_cast<int2 *>(take(m * sizeof(int2)));
  x.iparent = reinterpret_cast<int *>(take(m * 4));
  x.lparent = reinterpret_cast<int *>(take(n * 4));
  x.visits = reinterpret_cast<int *>(take(m * 4));
  x.ilo = reinterpret_cast<float4 *>(take(m * sizeof(float4)));
  x.ihi = reinterpret_cast<float4 *>(take(m * sizeof(float4)));
  x.subtree = reinterpret_cast<int *>(take(size_t(M) * 4));
  x.scratch_bytes = sort_scratch_bytes(n);
  x.scratch = take(x.scratch_bytes);
  if (t) *t = x;
  return off;
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ float3 load3(const float *v, uint32_t i) {
  return make_float3(__ldg(v + 3ull * i), __ldg(v + 3ull * i + 1), __ldg(v + 3ull * i + 2));
}

__global__ __launch_bounds__(kThreads) void k_prep(BatchDev B, TriRec *__restrict__ rec, float4 *__restrict__ lo,
                                                   float4 *__restrict__ hi, uint32_t *__restrict__ bounds,
                                                   uint32_t *__restrict__ err) {
  const uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
  float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  int mesh = -1;
  if (t < B.total_tris) {
    mesh = find_mesh(B.tri_starts, B.num_meshes, t);
    const MeshRec &M = B.recs[mesh];
    const uint64_t lt = t - B.tri_starts[mesh];
    const uint32_t V = M.num_verts;
    uint32_t i0 = __ldg(M.idx + 3 * lt), i1 = __ldg(M.idx + 3 * lt + 1), i2 = __ldg(M.idx + 3 * lt + 2);
    if (i0 >= V || i1 >= V || i2 >= V) {
      atomic_or_err(err, kErrBadIndex);
      i0 = i0 < V ? i0 : 0;
      i1 = i1 < V ? i1 : 0;
      i2 = i2 < V ? i2 : 0;
    }
    const float3 a = load3(M.verts, i0), b = load3(M.verts, i1), c = load3(M.verts, i2);
    const bool finite = isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) &&
                        isfinite(b.z) && isfinite(c.x) && isfinite(c.y) && isfinite(c.z);
    if (!finite) atomic_or_err(err, kErrNonFinite);
    if (rec) {
      const float e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
      const float e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
      const float e3x = c.x - b.x, e3y = c.y - b.y, e3z = c.z - b.z;
      const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
      TriRec r;
      r.r0 = make_float4(a.x, a.y, a.z, inv_or_zero(e1x * e1x + e1y * e1y + e1z * e1z));
      r.r1 = make_float4(e1x, e1y, e1z, inv_or_zero(e2x * e2x + e2y * e2y + e2z * e2z));
      r.r2 = make_float4(e2x, e2y, e2z, inv_or_zero(e3x * e3x + e3y * e3y + e3z * e3z));
      r.r3 = make_float4(nx, ny, nz, sqrtf(nx * nx + ny * ny + nz * nz));
      rec[t] = r;
    }
    const float4 l = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y),
                                 fminf(fminf(a.z, b.z), c.z), 0.0f);
    const float4 h = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y),
                                 fmaxf(fmaxf(a.z, b.z), c.z), 0.0f);
    lo[t] = l;
    hi[t] = h;
    if (finite) {
      cmin[0] = cmax[0] = 0.5f * (l.x + h.x);
      cmin[1] = cmax[1] = 0.5f * (l.y + h.y);
      cmin[2] = cmax[2] = 0.5f * (l.z + h.z);
    }
  }
  // Reduce over the warp when all its lanes hold the same mesh, else per lane.
  const int m0 = __shfl_sync(kFull, mesh, 0);
  if (__all_sync(kFull, mesh == m0)) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        cmin[a] = fminf(cmin[a], __shfl_xor_sync(kFull, cmin[a], o));
        cmax[a] = fmaxf(cmax[a], __shfl_xor_sync(kFull, cmax[a], o));
      }
    }
    if ((threadIdx.x & 31) != 0) mesh = -1;
  }
  if (mesh >= 0 && cmin[0] <= cmax[0]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(bounds + 6 * mesh + a, float_to_ordered(cmin[a]));
      atomicMax(bounds + 6 * mesh + 3 + a, float_to_ordered(cmax[a]));
    }
  }
}

__global__ void k_init_bounds(uint32_t *bounds, int M) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 6 * M) bounds[i] = (i % 6) < 3 ? 0xffffffffu : 0u;
}

__global__ __launch_bounds__(kThreads) void k_morton(BatchDev B, const float4 *__restrict__ lo,
                                                     const float4 *__restrict__ hi, const uint32_t *__restrict__ bounds,
                                                     uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  const uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (t >= B.total_tris) return;
  const int mesh = find_mesh(B.tri_starts, B.num_meshes, t);
  float bmin[3], ext[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    bmin[a] = ordered_to_float(bounds[6 * mesh + a]);
    ext[a] = ordered_to_float(bounds[6 * mesh + 3 + a]) - bmin[a];
  }
  const float4 l = lo[t], h = hi[t];
  const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float u = ext[a] > 0.0f ? (c[a] - bmin[a]) / ext[a] : 0.5f;
    const float s = fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f);
    q[a] = isfinite(s) ? static_cast<uint32_t>(s) : 0u;
  }
  keys[t] = (uint64_t(mesh) << 30) | (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  vals[t] = static_cast<uint32_t>(t);
}

// Length of the common prefix of sorted keys i and j (positions break ties); -1 outside.
__device__ __forceinline__ int prefix(const uint64_t *__restrict__ keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t a = keys[i], b = keys[j];
  if (a != b) return __clzll(a ^ b);
  return 64 + __clz(static_cast<uint32_t>(i ^ j));
}

__global__ __launch_bounds__(kThreads) void k_hierarchy(const uint64_t *__restrict__ keys, int n,
                                                        int2 *__restrict__ child, int2 *__restrict__ range,
                                                        int *__restrict__ iparent, int *__restrict__ lparent) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (prefix(keys, n, i, i + 1) - prefix(keys, n, i, i - 1)) > 0 ? 1 : -1;
  const int dmin = prefix(keys, n, i, i - d);
  int lmax = 2;
  while (prefix(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (prefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = prefix(keys, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (prefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int split = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  int left = split, right = split + 1;
  if (first == split) {
    lparent[split] = i;
    left = split | 0x80000000;
  } else {
    iparent[split] = i;
  }
  if (last == split + 1) {
    lparent[split + 1] = i;
    right = (split + 1) | 0x80000000;
  } else {
    iparent[split + 1] = i;
  }
  child[i] = make_int2(left, right);
  range[i] = make_int2(first, last);
  if (i == 0) iparent[0] = -1;
}

// The inner node whose range is exactly one mesh's triangles is that mesh's subtree root.
__global__ __launch_bounds__(kThreads) void k_find_subtrees(BatchDev B, const uint64_t *__restrict__ keys, int n,
                                                            const int2 *__restrict__ range, int *__restrict__ subtree) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  const int2 r = range[i];
  const int mesh = static_cast<int>(keys[r.x] >> 30);
  if (uint64_t(r.x) == B.tri_starts[mesh] && uint64_t(r.y) + 1 == B.tri_starts[mesh + 1]) subtree[mesh] = i;
}

__device__ __forceinline__ void child_box(int c, const uint32_t *__restrict__ vals, const float4 *__restrict__ lo,
                                          const float4 *__restrict__ hi, const float4 *ilo, const float4 *ihi,
                                          float4 &l, float4 &h) {
  if (c < 0) {
    const uint32_t t = vals[c & 0x7fffffff];
    l = lo[t];
    h = hi[t];
  } else {
    l = __ldcg(ilo + c);
    h = __ldcg(ihi + c);
  }
}

__global__ __launch_bounds__(kThreads) void k_refit(int n, const uint32_t *__restrict__ vals,
                                                    const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                                                    const int2 *__restrict__ child, const int *__restrict__ iparent,
                                                    const int *__restrict__ lparent, int *visits, float4 *ilo,
                                                    float4 *ihi) {
  const int leaf = blockIdx.x * kThreads + threadIdx.x;
  if (leaf >= n) return;
  int node = lparent[leaf];
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(visits + node, 1) == 0) return;  // the sibling's thread finishes this node
    __threadfence();
    const int2 c = child[node];
    float4 l0, h0, l1, h1;
    child_box(c.x, vals, lo, hi, ilo, ihi, l0, h0);
    child_box(c.y, vals, lo, hi, ilo, ihi, l1, h1);
    __stcg(ilo + node, make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f));
    __stcg(ihi + node, make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f));
    node = iparent[node];
  }
}

// A child box as centre and half extent (see Node), rounded outward: the half extent is rounded
// up from both sides of the rounded centre and widened by one part in 2^22, so that the traversal's
// box distance stays a lower bound of the distance to anything inside.
__device__ __forceinline__ void put_child(float *box, int which, float4 l, float4 h) {
  const float lo[3] = {l.x, l.y, l.z}, hi[3] = {h.x, h.y, h.z};
  const bool empty = !(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (empty) {
      box[which * 6 + a] = 0.0f;
      box[which * 6 + 3 + a] = -__int_as_float(0x7f800000);
      continue;
    }
    const float c = __fmul_rn(0.5f, __fadd_rn(lo[a], hi[a]));
    const float e = fmaxf(__fsub_ru(hi[a], c), __fsub_ru(c, lo[a]));
    box[which * 6 + a] = c;
    box[which * 6 + 3 + a] = __fmul_ru(e, 1.0f + 0x1p-22f);
  }
}

__device__ __forceinline__ void store_node(Node *nodes, int i, const float *b, int4 refs) {
  Node nd;
  nd.n0 = make_float4(b[0], b[1], b[2], b[3]);
  nd.n1 = make_float4(b[4], b[5], b[6], b[7]);
  nd.n2 = make_float4(b[8], b[9], b[10], b[11]);
  nd.n3 = refs;
  nodes[i] = nd;
}

__global__ __launch_bounds__(kThreads) void k_layout(BatchDev B, int n, const uint64_t *__restrict__ keys,
                                                     const uint32_t *__restrict__ vals, const float4 *__restrict__ lo,
                                                     const float4 *__restrict__ hi, const int2 *__restrict__ child,
                                                     const int2 *__restrict__ range, const float4 *__restrict__ ilo,
                                                     const float4 *__restrict__ ihi, Node *__restrict__ nodes) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  const int leaf_size = B.recs[keys[range[i].x] >> 30].leaf_size;
  float box[12];
  int ref[2], cnt[2];
  const int2 c = child[i];
  const int cs[2] = {c.x, c.y};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    float4 l, h;
    if (cs[k] < 0) {
      const int pos = cs[k] & 0x7fffffff;
      const uint32_t t = vals[pos];
      l = lo[t];
      h = hi[t];
      ref[k] = pos;
      cnt[k] = 1;
    } else {
      l = ilo[cs[k]];
      h = ihi[cs[k]];
      const int2 r = range[cs[k]];
      const int size = r.y - r.x + 1;
      if (size <= leaf_size) {
        ref[k] = r.x;
        cnt[k] = size;
      } else {
        ref[k] = cs[k];
        cnt[k] = 0;
      }
    }
    put_child(box, k, l, h);
  }
  store_node(nodes, i, box, make_int4(ref[0], ref[1], cnt[0], cnt[1]));
}

// Virtual root of each mesh: child 0 is the mesh's subtree (a leaf range when the mesh has at
// most leaf_size triangles), child 1 is empty.
__global__ void k_roots(BatchDev B, int num_inner, const uint32_t *__restrict__ vals, const float4 *__restrict__ lo,
                        const float4 *__restrict__ hi, const float4 *__restrict__ ilo,
                        const float4 *__restrict__ ihi, const int *__restrict__ subtree, Node *__restrict__ nodes,
                        uint32_t *__restrict__ err) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= B.num_meshes) return;
  const MeshRec &M = B.recs[m];
  const int first = static_cast<int>(B.tri_starts[m]);
  const int count = static_cast<int>(B.tri_starts[m + 1] - B.tri_starts[m]);
  float box[12];
  const float4 empty_lo = make_float4(INFINITY, INFINITY, INFINITY, 0), empty_hi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0);
  put_child(box, 1, empty_lo, empty_hi);
  int4 refs = make_int4(0, 0, -1, -1);
  if (count == 1) {
    const uint32_t t = vals[first];
    put_child(box, 0, lo[t], hi[t]);
    refs = make_int4(first, 0, 1, -1);
  } else if (count > 1) {
    const int s = subtree[m];
    if (s < 0) {
      atomic_or_err(err, kErrCorruptTree);
      put_child(box, 0, empty_lo, empty_hi);
    } else {
      put_child(box, 0, ilo[s], ihi[s]);
      refs = count <= M.leaf_size ? make_int4(first, 0, count, -1) : make_int4(s, 0, 0, -1);
    }
  } else {
    put_child(box, 0, empty_lo, empty_hi);
  }
  store_node(nodes, num_inner + m, box, refs);
}

__global__ __launch_bounds__(kThreads) void k_gather(BatchDev B, const uint32_t *__restrict__ vals,
                                                     const TriRec *__restrict__ rec, TriRec *__restrict__ out,
                                                     DistTri *__restrict__ dout, uint32_t *__restrict__ order) {
  const uint64_t k = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (k >= B.total_tris) return;
  const uint32_t t = vals ? vals[k] : static_cast<uint32_t>(k);
  const int mesh = find_mesh(B.tri_starts, B.num_meshes, t);
  const uint64_t lt = t - B.tri_starts[mesh];
  if (out) out[k] = rec[t];
  if (dout) {
    // The frame is built from the input vertices (k_prep has flagged bad indices already).
    const MeshRec &M = B.recs[mesh];
    const uint32_t V = M.num_verts;
    uint32_t i0 = __ldg(M.idx + 3 * lt), i1 = __ldg(M.idx + 3 * lt + 1), i2 = __ldg(M.idx + 3 * lt + 2);
    i0 = i0 < V ? i0 : 0;
    i1 = i1 < V ? i1 : 0;
    i2 = i2 < V ? i2 : 0;
    dout[k] = make_dist_tri(load3(M.verts, i0), load3(M.verts, i1), load3(M.verts, i2));
  }
  order[k] = static_cast<uint32_t>(lt);
}

// Far-field moments of every inner node, bottom-up like k_refit: (sum of a_i n_i, sum of a_i)
// over its triangles, a_i the area and n_i the unit normal. A triangle's a_i n_i is half its edge
// cross product, the r3 of its record (whose w is the product's length).
__device__ __forceinline__ float4 tri_moment(const TriRec &t) {
  return make_float4(0.5f * t.r3.x, 0.5f * t.r3.y, 0.5f * t.r3.z, 0.5f * t.r3.w);
}

__global__ __launch_bounds__(kThreads) void k_moments(int n, const TriRec *__restrict__ tris,
                                                      const int2 *__restrict__ child, const int *__restrict__ iparent,
                                                      const int *__restrict__ lparent, int *visits, float4 *mom) {
  const int leaf = blockIdx.x * kThreads + threadIdx.x;
  if (leaf >= n) return;
  int node = lparent[leaf];
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(visits + node, 1) == 0) return;
    __threadfence();
    const int2 c = child[node];
    const float4 a = c.x < 0 ? tri_moment(tris[c.x & 0x7fffffff]) : __ldcg(mom + c.x);
    const float4 b = c.y < 0 ? tri_moment(tris[c.y & 0x7fffffff]) : __ldcg(mom + c.y);
    __stcg(mom + node, make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w));
    node = iparent[node];
  }
}

inline unsigned blocks_for(size_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

}  // namespace

size_t lbvh_temp_bytes(uint64_t total_tris, int num_meshes) { return temp_layout(total_tris, num_meshes, nullptr, nullptr); }

size_t lbvh_bytes(uint64_t T, int M, bool winding) {
  const size_t n = std::max<uint64_t>(T, 1), m = std::max<uint64_t>(T, 2) - 1;
  return align256(n * (winding ? sizeof(TriRec) : sizeof(DistTri))) + align256((m + M) * sizeof(Node)) +
         align256(n * 4) + align256(size_t(M) * 6 * 4) + (winding ? align256(m * sizeof(float4)) : 0);
}

void lbvh_bind(BvhDev &b, void *mem, uint64_t T, int M, bool winding) {
  const size_t n = std::max<uint64_t>(T, 1), m = std::max<uint64_t>(T, 2) - 1;
  char *p = static_cast<char *>(mem);
  b.tris = winding ? reinterpret_cast<TriRec *>(p) : nullptr;
  b.dtris = winding ? nullptr : reinterpret_cast<DistTri *>(p);
  p += align256(n * (winding ? sizeof(TriRec) : sizeof(DistTri)));
  b.nodes = reinterpret_cast<Node *>(p);
  p += align256((m + M) * sizeof(Node));
  b.leaf_order = reinterpret_cast<uint32_t *>(p);
  p += align256(n * 4);
  b.bounds = reinterpret_cast<uint32_t *>(p);
  p += align256(size_t(M) * 6 * 4);
  b.node_moment = winding ? reinterpret_cast<float4 *>(p) : nullptr;
  b.num_inner = T >= 2 ? static_cast<int>(T - 1) : 0;
  b.num_nodes = b.num_inner + M;
}

cudaError_t lbvh_build(const BatchDev &B, BvhDev &b, void *temp, size_t temp_bytes, uint32_t *err, cudaStream_t st) {
  const uint64_t T = B.total_tris;
  const int M = B.num_meshes;
  if (T == 0 || M == 0) return cudaErrorInvalidValue;
  if (T >= (1ull << 31)) return cudaErrorInvalidValue;
  BuildTemp t;
  const size_t need = temp_layout(T, M, static_cast<char *>(temp), &t);
  if (need > temp_bytes) return cudaErrorMemoryAllocation;
  cudaError_t e;
  k_init_bounds<<<(6 * M + 255) / 256, 256, 0, st>>>(b.bounds, M);
  note_launch();
  k_prep<<<blocks_for(T), kThreads, 0, st>>>(B, b.tris ? t.rec : nullptr, t.lo, t.hi, b.bounds, err);
  note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int n = static_cast<int>(T);
  const uint32_t *vals = nullptr;
  if (T >= 2) {
    k_morton<<<blocks_for(T), kThreads, 0, st>>>(B, t.lo, t.hi, b.bounds, t.keys, t.vals);
    note_launch();
    int mesh_bits = 0;
    while ((1 << mesh_bits) < M) ++mesh_bits;
    if ((e = radix_sort_pairs(t.keys, t.vals, t.keys_alt, t.vals_alt, T, 30 + mesh_bits,
                              Scratch{t.scratch, t.scratch_bytes}, st)) != cudaSuccess)
      return e;
    k_hierarchy<<<blocks_for(T - 1), kThreads, 0, st>>>(t.keys, n, t.child, t.range, t.iparent, t.lparent);
    note_launch();
    if ((e = cudaMemsetAsync(t.subtree, 0xff, sizeof(int) * M, st)) != cudaSuccess) return e;
    k_find_subtrees<<<blocks_for(T - 1), kThreads, 0, st>>>(B, t.keys, n, t.range, t.subtree);
    note_launch();
    if ((e = cudaMemsetAsync(t.visits, 0, sizeof(int) * (T - 1), st)) != cudaSuccess) return e;
    k_refit<<<blocks_for(T), kThreads, 0, st>>>(n, t.vals, t.lo, t.hi, t.child, t.iparent, t.lparent, t.visits, t.ilo,
                                                 t.ihi);
    note_launch();
    k_layout<<<blocks_for(T - 1), kThreads, 0, st>>>(B, n, t.keys, t.vals, t.lo, t.hi, t.child, t.range, t.ilo, t.ihi,
                                                      b.nodes);
    note_launch();
    vals = t.vals;
  } else {
    // one triangle in the whole batch: its sorted position is 0
    if ((e = cudaMemsetAsync(t.vals, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    vals = t.vals;
  }
  k_roots<<<(M + 127) / 128, 128, 0, st>>>(B, b.num_inner, vals, t.lo, t.hi, t.ilo, t.ihi, t.subtree, b.nodes, err);
  note_launch();
  k_gather<<<blocks_for(T), kThreads, 0, st>>>(B, vals, t.rec, b.tris, b.dtris, b.leaf_order);
  note_launch();
  if (b.node_moment && T >= 2) {
    if ((e = cudaMemsetAsync(t.visits, 0, sizeof(int) * (T - 1), st)) != cudaSuccess) return e;
    k_moments<<<blocks_for(T), kThreads, 0, st>>>(n, b.tris, t.child, t.iparent, t.lparent, t.visits, b.node_moment);
    note_launch();
  }
  return cudaGetLastError();
}

}  // namespace sdfb
