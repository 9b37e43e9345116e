// Device-built linear BVH over one mesh's triangles (replaces the OptiX GAS build of
// src/convert/sdf_baker.cpp:170-193).
//
//   1. k_prep      gathers each indexed triangle, checks indices and finiteness, writes its
//                  64-byte distance record and bounds, and reduces the centroid bounds.
//   2. k_morton    30-bit Morton code of the box centre, normalised to the centroid bounds.
//   3. radix sort  (code, triangle) pairs, stable.
//   4. k_hierarchy binary radix tree over the sorted codes (Karras 2012, "Maximizing Parallelism
//                  in the Construction of BVHs, Octrees, and k-d Trees"; equal codes ordered by
//                  position), one thread per inner node.
//   5. k_refit     bottom-up boxes: the second thread to reach a node merges its children.
//   6. k_layout    64-byte traversal nodes holding both child boxes; subtrees of at most
//                  `leaf_size` triangles become leaves (their records are contiguous).
//   7. k_gather    triangle records in leaf order.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct BuildTemp {
  TriRec *rec;      // T, original order
  float4 *lo, *hi;  // T, triangle boxes (original order)
  uint64_t *keys, *keys_alt;
  uint32_t *vals, *vals_alt;
  int2 *child;      // T - 1: (left, right); leaf children have the top bit set
  int2 *range;      // T - 1: covered sorted positions [first, last]
  int *iparent;     // T - 1
  int *lparent;     // T
  int *visits;      // T - 1
  float4 *ilo, *ihi;  // T - 1 inner boxes
  void *scratch;
  size_t scratch_bytes;
};

size_t temp_layout(uint32_t T, char *base, BuildTemp *t) {
  const size_t n = std::max<uint32_t>(T, 1), m = std::max<uint32_t>(T, 2) - 1;
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

__global__ __launch_bounds__(kThreads) void k_prep(const float *__restrict__ verts, const uint32_t *__restrict__ idx,
                                                   uint32_t V, uint32_t T, TriRec *__restrict__ rec,
                                                   float4 *__restrict__ lo, float4 *__restrict__ hi,
                                                   uint32_t *__restrict__ bounds, uint32_t *__restrict__ err) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (t < T) {
    uint32_t i0 = __ldg(idx + 3ull * t), i1 = __ldg(idx + 3ull * t + 1), i2 = __ldg(idx + 3ull * t + 2);
    if (i0 >= V || i1 >= V || i2 >= V) {
      atomic_or_err(err, kErrBadIndex);
      i0 = i0 < V ? i0 : 0;
      i1 = i1 < V ? i1 : 0;
      i2 = i2 < V ? i2 : 0;
    }
    const float3 a = load3(verts, i0), b = load3(verts, i1), c = load3(verts, i2);
    const bool finite = isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) &&
                        isfinite(b.z) && isfinite(c.x) && isfinite(c.y) && isfinite(c.z);
    if (!finite) atomic_or_err(err, kErrNonFinite);
    const float e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
    const float e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
    const float e3x = c.x - b.x, e3y = c.y - b.y, e3z = c.z - b.z;
    const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    TriRec r;
    r.r0 = make_float4(a.x, a.y, a.z, inv_or_zero(e1x * e1x + e1y * e1y + e1z * e1z));
    r.r1 = make_float4(e1x, e1y, e1z, inv_or_zero(e2x * e2x + e2y * e2y + e2z * e2z));
    r.r2 = make_float4(e2x, e2y, e2z, inv_or_zero(e3x * e3x + e3y * e3y + e3z * e3z));
    const float n2 = nx * nx + ny * ny + nz * nz;
    // A face region is only used when the normal is well above rounding noise.
    const float scale = fmaxf(e1x * e1x + e1y * e1y + e1z * e1z, e2x * e2x + e2y * e2y + e2z * e2z);
    r.r3 = make_float4(nx, ny, nz, (n2 > 1e-12f * scale * scale) ? 1.0f / n2 : 0.0f);
    rec[t] = r;
    const float4 l = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y),
                                 fminf(fminf(a.z, b.z), c.z), 0.0f);
    const float4 h = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y),
                                 fmaxf(fmaxf(a.z, b.z), c.z), 0.0f);
    lo[t] = l;
    hi[t] = h;
    if (finite) {
      const float cx = 0.5f * (l.x + h.x), cy = 0.5f * (l.y + h.y), cz = 0.5f * (l.z + h.z);
      cmin[0] = cmax[0] = cx;
      cmin[1] = cmax[1] = cy;
      cmin[2] = cmax[2] = cz;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      cmin[a] = fminf(cmin[a], __shfl_xor_sync(kFull, cmin[a], o));
      cmax[a] = fmaxf(cmax[a], __shfl_xor_sync(kFull, cmax[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0 && cmin[0] <= cmax[0]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(bounds + a, float_to_ordered(cmin[a]));
      atomicMax(bounds + 3 + a, float_to_ordered(cmax[a]));
    }
  }
}

__global__ void k_init_bounds(uint32_t *bounds) {
  if (threadIdx.x < 3) bounds[threadIdx.x] = 0xffffffffu;       // min
  else if (threadIdx.x < 6) bounds[threadIdx.x] = 0u;           // max
}

__global__ __launch_bounds__(kThreads) void k_morton(const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                                                     uint32_t T, const uint32_t *__restrict__ bounds,
                                                     uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= T) return;
  float bmin[3], ext[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    bmin[a] = ordered_to_float(bounds[a]);
    const float bmax = ordered_to_float(bounds[3 + a]);
    ext[a] = bmax - bmin[a];
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
  keys[t] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  vals[t] = t;
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

__device__ __forceinline__ void put_child(float *box, int which, float4 l, float4 h) {
  box[which * 6 + 0] = l.x;
  box[which * 6 + 1] = l.y;
  box[which * 6 + 2] = l.z;
  box[which * 6 + 3] = h.x;
  box[which * 6 + 4] = h.y;
  box[which * 6 + 5] = h.z;
}

__device__ __forceinline__ void store_node(Node *nodes, int i, const float *b, int4 refs) {
  Node nd;
  nd.n0 = make_float4(b[0], b[1], b[2], b[3]);
  nd.n1 = make_float4(b[4], b[5], b[6], b[7]);
  nd.n2 = make_float4(b[8], b[9], b[10], b[11]);
  nd.n3 = refs;
  nodes[i] = nd;
}

__global__ __launch_bounds__(kThreads) void k_layout(int n, int leaf_size, const uint32_t *__restrict__ vals,
                                                     const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                                                     const int2 *__restrict__ child, const int2 *__restrict__ range,
                                                     const float4 *__restrict__ ilo, const float4 *__restrict__ ihi,
                                                     Node *__restrict__ nodes) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  float box[12];
  int ref[2], cnt[2];
  if (i == 0 && n <= leaf_size) {  // the whole mesh is one leaf
    put_child(box, 0, ilo[0], ihi[0]);
    put_child(box, 1, make_float4(INFINITY, INFINITY, INFINITY, 0), make_float4(-INFINITY, -INFINITY, -INFINITY, 0));
    store_node(nodes, 0, box, make_int4(0, 0, n, -1));
    return;
  }
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

__global__ void k_single(const float4 *lo, const float4 *hi, Node *nodes) {
  float box[12];
  put_child(box, 0, lo[0], hi[0]);
  put_child(box, 1, make_float4(INFINITY, INFINITY, INFINITY, 0), make_float4(-INFINITY, -INFINITY, -INFINITY, 0));
  store_node(nodes, 0, box, make_int4(0, 0, 1, -1));
}

__global__ __launch_bounds__(kThreads) void k_gather(uint32_t T, const uint32_t *__restrict__ vals,
                                                     const TriRec *__restrict__ rec, TriRec *__restrict__ out,
                                                     uint32_t *__restrict__ order) {
  const uint32_t k = blockIdx.x * kThreads + threadIdx.x;
  if (k >= T) return;
  const uint32_t t = vals ? vals[k] : k;
  out[k] = rec[t];
  order[k] = t;
}

// Winding-number moments of every inner node, bottom-up like k_refit (Barill et al. 2018, "Fast
// Winding Numbers for Soups and Clouds": each triangle is a dipole of area vector a = (e1 x e2)/2
// at its centroid c; a node keeps N = sum a, P = area-weighted centroid, M = sum a (c - P)^T and
// r = radius around P). Children combine as N = N0 + N1, P = (A0 P0 + A1 P1) / (A0 + A1),
// M = M0 + N0 (P0 - P)^T + M1 + N1 (P1 - P)^T, r = max(r0 + |P0 - P|, r1 + |P1 - P|).
struct Mom {
  float px, py, pz, r, nx, ny, nz, area;
  float m[9];
};

__device__ __forceinline__ Mom leaf_mom(const TriRec &t) {
  Mom o;
  const float cx = t.r0.x + (t.r1.x + t.r2.x) * (1.0f / 3.0f);
  const float cy = t.r0.y + (t.r1.y + t.r2.y) * (1.0f / 3.0f);
  const float cz = t.r0.z + (t.r1.z + t.r2.z) * (1.0f / 3.0f);
  o.px = cx;
  o.py = cy;
  o.pz = cz;
  o.nx = 0.5f * t.r3.x;
  o.ny = 0.5f * t.r3.y;
  o.nz = 0.5f * t.r3.z;
  o.area = sqrtf(o.nx * o.nx + o.ny * o.ny + o.nz * o.nz);
  const float ax = t.r0.x - cx, ay = t.r0.y - cy, az = t.r0.z - cz;
  const float bx = ax + t.r1.x, by = ay + t.r1.y, bz = az + t.r1.z;
  const float qx = ax + t.r2.x, qy = ay + t.r2.y, qz = az + t.r2.z;
  o.r = sqrtf(fmaxf(fmaxf(ax * ax + ay * ay + az * az, bx * bx + by * by + bz * bz), qx * qx + qy * qy + qz * qz));
#pragma unroll
  for (int k = 0; k < 9; ++k) o.m[k] = 0.0f;
  return o;
}

__device__ __forceinline__ Mom combine(const Mom &a, const Mom &b) {
  Mom o;
  const float A = a.area + b.area;
  const float wa = A > 0.0f ? a.area / A : 0.5f, wb = 1.0f - wa;
  o.px = wa * a.px + wb * b.px;
  o.py = wa * a.py + wb * b.py;
  o.pz = wa * a.pz + wb * b.pz;
  o.area = A;
  o.nx = a.nx + b.nx;
  o.ny = a.ny + b.ny;
  o.nz = a.nz + b.nz;
  const float da[3] = {a.px - o.px, a.py - o.py, a.pz - o.pz}, db[3] = {b.px - o.px, b.py - o.py, b.pz - o.pz};
  const float na[3] = {a.nx, a.ny, a.nz}, nb[3] = {b.nx, b.ny, b.nz};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.m[3 * i + j] = a.m[3 * i + j] + b.m[3 * i + j] + na[i] * da[j] + nb[i] * db[j];
  o.r = fmaxf(a.r + sqrtf(da[0] * da[0] + da[1] * da[1] + da[2] * da[2]),
              b.r + sqrtf(db[0] * db[0] + db[1] * db[1] + db[2] * db[2]));
  return o;
}

__device__ __forceinline__ void store_mom(float4 *mom, float *area, int i, const Mom &o) {
  __stcg(mom + 4 * i + 0, make_float4(o.px, o.py, o.pz, o.r));
  __stcg(mom + 4 * i + 1, make_float4(o.nx, o.ny, o.nz, o.m[0]));
  __stcg(mom + 4 * i + 2, make_float4(o.m[1], o.m[2], o.m[3], o.m[4]));
  __stcg(mom + 4 * i + 3, make_float4(o.m[5], o.m[6], o.m[7], o.m[8]));
  __stcg(area + i, o.area);
}

__device__ __forceinline__ Mom load_mom(const float4 *mom, const float *area, int i) {
  Mom o;
  const float4 a = __ldcg(mom + 4 * i), b = __ldcg(mom + 4 * i + 1), c = __ldcg(mom + 4 * i + 2),
               d = __ldcg(mom + 4 * i + 3);
  o.px = a.x; o.py = a.y; o.pz = a.z; o.r = a.w;
  o.nx = b.x; o.ny = b.y; o.nz = b.z; o.m[0] = b.w;
  o.m[1] = c.x; o.m[2] = c.y; o.m[3] = c.z; o.m[4] = c.w;
  o.m[5] = d.x; o.m[6] = d.y; o.m[7] = d.z; o.m[8] = d.w;
  o.area = __ldcg(area + i);
  return o;
}

__global__ __launch_bounds__(kThreads) void k_moments(int n, const TriRec *__restrict__ tris,
                                                      const int2 *__restrict__ child, const int *__restrict__ iparent,
                                                      const int *__restrict__ lparent, int *visits, float4 *mom,
                                                      float *area) {
  const int leaf = blockIdx.x * kThreads + threadIdx.x;
  if (leaf >= n) return;
  int node = lparent[leaf];
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(visits + node, 1) == 0) return;
    __threadfence();
    const int2 c = child[node];
    const Mom a = c.x < 0 ? leaf_mom(tris[c.x & 0x7fffffff]) : load_mom(mom, area, c.x);
    const Mom b = c.y < 0 ? leaf_mom(tris[c.y & 0x7fffffff]) : load_mom(mom, area, c.y);
    store_mom(mom, area, node, combine(a, b));
    node = iparent[node];
  }
}

__global__ void k_moments_single(const TriRec *tris, float4 *mom) {
  const Mom o = leaf_mom(tris[0]);
  mom[0] = make_float4(o.px, o.py, o.pz, o.r);
  mom[1] = make_float4(o.nx, o.ny, o.nz, 0.0f);
  mom[2] = make_float4(0, 0, 0, 0);
  mom[3] = make_float4(0, 0, 0, 0);
}

inline unsigned blocks_for(size_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

}  // namespace

size_t lbvh_temp_bytes(uint32_t num_tris) { return temp_layout(num_tris, nullptr, nullptr); }

size_t lbvh_mesh_bytes(uint32_t T, bool with_moments) {
  const size_t n = std::max<uint32_t>(T, 1), m = std::max<uint32_t>(T, 2) - 1;
  return align256(n * sizeof(TriRec)) + align256(m * sizeof(Node)) + align256(n * 4) + align256(6 * 4) +
         (with_moments ? align256(m * 4 * sizeof(float4)) : 0);
}

void lbvh_bind_mesh(MeshDev &m, void *mem, bool with_moments) {
  const size_t n = std::max<uint32_t>(m.num_tris, 1), k = std::max<uint32_t>(m.num_tris, 2) - 1;
  char *p = static_cast<char *>(mem);
  m.tris = reinterpret_cast<TriRec *>(p);
  p += align256(n * sizeof(TriRec));
  m.nodes = reinterpret_cast<Node *>(p);
  p += align256(k * sizeof(Node));
  m.leaf_order = reinterpret_cast<uint32_t *>(p);
  p += align256(n * 4);
  m.bounds = reinterpret_cast<uint32_t *>(p);
  p += align256(6 * 4);
  m.moments = with_moments ? reinterpret_cast<float4 *>(p) : nullptr;
}

cudaError_t lbvh_build(MeshDev &m, int leaf_size, void *temp, size_t temp_bytes, uint32_t *err, cudaStream_t st) {
  const uint32_t T = m.num_tris;
  if (T == 0) return cudaErrorInvalidValue;
  BuildTemp t;
  const size_t need = temp_layout(T, static_cast<char *>(temp), &t);
  if (need > temp_bytes) return cudaErrorMemoryAllocation;
  leaf_size = std::max(1, std::min(leaf_size, 16));
  m.leaf_size = leaf_size;
  cudaError_t e;
  k_init_bounds<<<1, 32, 0, st>>>(m.bounds);
  note_launch();
  k_prep<<<blocks_for(T), kThreads, 0, st>>>(m.verts, m.idx, m.num_verts, T, t.rec, t.lo, t.hi, m.bounds, err);
  note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (T == 1) {
    k_single<<<1, 1, 0, st>>>(t.lo, t.hi, m.nodes);
    note_launch();
    k_gather<<<1, kThreads, 0, st>>>(1, nullptr, t.rec, m.tris, m.leaf_order);
    note_launch();
    if (m.moments) {
      k_moments_single<<<1, 1, 0, st>>>(m.tris, m.moments);
      note_launch();
    }
    return cudaGetLastError();
  }
  k_morton<<<blocks_for(T), kThreads, 0, st>>>(t.lo, t.hi, T, m.bounds, t.keys, t.vals);
  note_launch();
  if ((e = radix_sort_pairs(t.keys, t.vals, t.keys_alt, t.vals_alt, T, 30, Scratch{t.scratch, t.scratch_bytes}, st)) !=
      cudaSuccess)
    return e;
  const int n = static_cast<int>(T);
  k_hierarchy<<<blocks_for(T - 1), kThreads, 0, st>>>(t.keys, n, t.child, t.range, t.iparent, t.lparent);
  note_launch();
  if ((e = cudaMemsetAsync(t.visits, 0, sizeof(int) * (T - 1), st)) != cudaSuccess) return e;
  k_refit<<<blocks_for(T), kThreads, 0, st>>>(n, t.vals, t.lo, t.hi, t.child, t.iparent, t.lparent, t.visits, t.ilo,
                                               t.ihi);
  note_launch();
  k_layout<<<blocks_for(T - 1), kThreads, 0, st>>>(n, leaf_size, t.vals, t.lo, t.hi, t.child, t.range, t.ilo, t.ihi,
                                                    m.nodes);
  note_launch();
  k_gather<<<blocks_for(T), kThreads, 0, st>>>(T, t.vals, t.rec, m.tris, m.leaf_order);
  note_launch();
  if (m.moments) {
    // the inner boxes are no longer needed: their space holds the node areas
    if ((e = cudaMemsetAsync(t.visits, 0, sizeof(int) * (T - 1), st)) != cudaSuccess) return e;
    k_moments<<<blocks_for(T), kThreads, 0, st>>>(n, m.tris, t.child, t.iparent, t.lparent, t.visits, m.moments,
                                                  reinterpret_cast<float *>(t.ilo));
    note_launch();
  }
  return cudaGetLastError();
}

}  // namespace sdfb
