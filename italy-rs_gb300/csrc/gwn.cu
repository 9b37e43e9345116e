// Generalized winding number sign for meshes that are not watertight (replaces the 5-ray parity
// vote of src/render/kernels/sdf_bake.cu:53-69, which assumes a closed mesh).
//
// w(q) = sum of triangle solid angles / 4 pi (Jacobson, Kavan & Sorkine-Hornung 2013); a cell is
// inside when |w| > 0.5. It is evaluated through an exact decomposition: the bake closes every
// boundary loop of the mesh with a small fan cap (caps.cu), so mesh + caps has no boundary
// and its winding number W(q) is an integer, namely the signed count of +z crossings above q
// (parity.cu stores each crossing's orientation). Then
//     w(q) = W(q) - w_caps(q),
// and only the caps -- small triangles hugging the holes -- need solid angles. A cap subtree far
// from q is replaced by its dipole term with a rigorous error bound (the far field of Barill et al.
// 2018, "Fast Winding Numbers for Soups and Clouds", with a Taylor bound of our own): a triangle
// of area a and unit normal n subtends the integral over it of f(x) = (x - q) . n / |x - q|^3,
// whose gradient is at most 2 / |x - q|^3 in length. For a cluster inside the ball of radius rho
// about c, at r = |c - q| > rho,
//     Omega = D . (c - q) / r^3  +/-  A * 2 rho / (r - rho)^3,    D = sum a_i n_i,  A = sum a_i,
// with (D, A) stored per node (lbvh.cu) and (c, rho) the child box's centre and half diagonal. A
// subtree is taken as its dipole when that bound is at most tau, and a cell is decided as soon as
// the summed bounds cannot move |w| across 0.5.
//
// Precision split:
//   pass 1 (FP32, every cell of every winding-number mesh, warp tiles of 4 x 4 x 8, four cells
//     of a column per lane): cells outside the band (|d| > band_voxels * voxel) whose interval
//     [c - e, c + e] lies on one side of |w| = 0.5 get their sign; the band and undecided cells
//     go to a refine list.
//   pass 2 (FP64 accumulation, exact cap solid angles in FP64 from the original FP32 vertices,
//     the same FP32 far field): signs of the refine list, first with coarse subtrees (kTau64),
//     then the cells that stay undecided again with fine ones (kTau64Fine); a cell still
//     undecided goes to
//   pass 3 (FP64 sum over every cap triangle of its mesh, one block per cell).
#include <algorithm>
#include <cstdint>

#include "api_internal.h"
#include "common.cuh"

using namespace sdfb;

namespace {

constexpr int kThreads = 256;
constexpr int kStack = 64;
constexpr double kInv4Pi = 0.07957747154594767;
// Largest far-field error bound (sr) taken for one cap subtree. A cell is decided once the summed
// bounds cannot move |w| across 0.5, and most cells have a margin near 0.5, so the FP32 pass takes
// coarse subtrees (500k-triangle soup at 512^3, sign stage: 4e-3 sr 256 ms, 2e-2 155 ms, 0.1
// 116 ms, 0.3 123 ms, with the same signs; 0.1 leaves 1.5% more cells to the FP64 pass). The FP64
// band pass runs twice: coarse subtrees first, then fine ones for the cells still undecided, and
// only cells neither decides go to the direct sum (one pass at 2e-2: sign stage 87 ms, ~950 cells
// summed directly; 0.1 then 5e-3: 74 ms, ~500; 0.3 then 1e-2: 71 ms, ~850; 5e-2 then 5e-4: 98 ms,
// ~120 -- the direct sum costs ~10 us a cell, the fine walk little, the coarse walk most).
constexpr float kTau32 = 1e-1f;
constexpr float kTau64 = 3e-1f;
constexpr float kTau64Fine = 1e-2f;

template <typename T> struct V3 {
  T x, y, z;
};

// Exact solid angle of triangle (a, b, c) seen from the origin (Van Oosterom & Strackee 1983).
template <typename T>
__device__ __forceinline__ T solid_angle(V3<T> a, V3<T> b, V3<T> c) {
  const T la = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  const T lb = sqrt(b.x * b.x + b.y * b.y + b.z * b.z);
  const T lc = sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
  const T det = a.x * (b.y * c.z - b.z * c.y) - a.y * (b.x * c.z - b.z * c.x) + a.z * (b.x * c.y - b.y * c.x);
  const T ab = a.x * b.x + a.y * b.y + a.z * b.z, bc = b.x * c.x + b.y * c.y + b.z * c.z,
          ca = c.x * a.x + c.y * a.y + c.z * a.z;
  const T den = la * lb * lc + ab * lc + bc * la + ca * lb;
  return T(2) * atan2(det, den);
}

struct GwnArgs {
  BatchDev batch;  // each GWN mesh record names its caps hierarchy
  const uint64_t *col_start;
  const float *col_z;
  const int8_t *col_s;
  float band_voxels;
  uint64_t *refine;  // pass 1 -> pass 2 (coarse); reused for pass 2 (fine) -> pass 3
  unsigned long long *refine_count;
  uint64_t *direct;  // pass 2 (coarse) -> pass 2 (fine)
  unsigned long long *direct_count;
  unsigned long long *final_count;  // cells for pass 3, listed in refine
  unsigned long long *tile_counter;
  uint32_t *err;
};

// Signed crossings of the column above height pz (the integer winding number of mesh + caps).
__device__ __forceinline__ int column_winding(const GwnArgs &a, const MeshRec &M, int vx, int vy, float pz) {
  const uint64_t col = M.col_base + uint64_t(vy) * M.g.nx + vx;
  const uint64_t s0 = __ldg(a.col_start + col), s1 = __ldg(a.col_start + col + 1);
  int w = 0;
  for (uint64_t k = s0; k < s1; ++k)
    if (__ldg(a.col_z + k) > pz) w += __ldg(a.col_s + k);
  return w;
}

// The same for V heights of one column, reading its crossings once.
template <int V>
__device__ __forceinline__ void column_windings(const GwnArgs &a, const MeshRec &M, int vx, int vy,
                                                const float (&pz)[V], int (&w)[V]) {
  const uint64_t col = M.col_base + uint64_t(vy) * M.g.nx + vx;
  const uint64_t s0 = __ldg(a.col_start + col), s1 = __ldg(a.col_start + col + 1);
#pragma unroll
  for (int v = 0; v < V; ++v) w[v] = 0;
  for (uint64_t k = s0; k < s1; ++k) {
    const float z = __ldg(a.col_z + k);
    const int s = __ldg(a.col_s + k);
#pragma unroll
    for (int v = 0; v < V; ++v) w[v] += z > pz[v] ? s : 0;
  }
}

// The far field of a cap cluster -- moment m = (D, A), inside the child box of centre c and half
// extent e (so inside the ball of radius |e| about c) -- seen from q: false when q is too close
// (r <= 2 |e|) or the error bound exceeds tau; else val = D . (c - q) / r^3 and err bounds
// |Omega - val|, widened for the rounding of T.
template <typename T>
__device__ __forceinline__ bool far_field(T qx, T qy, T qz, const float4 &n0, const float4 &n1, const float4 &n2,
                                          int which, const float4 &m, T tau, T &val, T &err) {
  const float cx = which ? n1.z : n0.x, cy = which ? n1.w : n0.y, cz = which ? n2.x : n0.z;
  const float ex = which ? n2.y : n0.w, ey = which ? n2.z : n1.x, ez = which ? n2.w : n1.y;
  const T dx = T(cx) - qx, dy = T(cy) - qy, dz = T(cz) - qz;
  const T r2 = dx * dx + dy * dy + dz * dz;
  const T rho = sqrt(T(ex) * T(ex) + T(ey) * T(ey) + T(ez) * T(ez));
  if (!(r2 > T(4) * rho * rho)) return false;
  const T r = sqrt(r2), g = r - rho;
  err = T(m.w) * T(2) * rho / (g * g * g);
  if (!(err <= tau)) return false;
  val = (T(m.x) * dx + T(m.y) * dy + T(m.z) * dz) / (r2 * r);
  constexpr T kRel = sizeof(T) == 4 ? T(1e-5) : T(1e-13);
  err = err * (T(1) + kRel) + kRel * fabs(val);
  return true;
}

// (D, A) of a leaf's cap triangles (D = half the sum of their edge cross products, A = half the
// sum of their lengths, which the records hold).
__device__ __forceinline__ float4 leaf_moment(const TriRec *tr, int count) {
  float4 m = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (int j = 0; j < count; ++j) {
    const float4 r3 = __ldg(&tr[j].r3);
    m.x += 0.5f * r3.x;
    m.y += 0.5f * r3.y;
    m.z += 0.5f * r3.z;
    m.w += 0.5f * r3.w;
  }
  return m;
}

// FP32 far field with one reciprocal square root per distance and one approximate reciprocal for
// the bound (each within 2 ulp, far inside the kRel margin the bound carries); the acceptance
// test err <= tau is taken as A 2 rho <= tau g^3 with a 1e-6 margin, without a division.
constexpr bool kFastFarField = true;
__device__ __forceinline__ bool far_field_fast(float qx, float qy, float qz, const float4 &n0, const float4 &n1,
                                               const float4 &n2, int which, const float4 &m, float tau, float &val,
                                               float &err) {
  const float cx = which ? n1.z : n0.x, cy = which ? n1.w : n0.y, cz = which ? n2.x : n0.z;
  const float ex = which ? n2.y : n0.w, ey = which ? n2.z : n1.x, ez = which ? n2.w : n1.y;
  const float dx = cx - qx, dy = cy - qy, dz = cz - qz;
  const float r2 = dx * dx + dy * dy + dz * dz;
  const float rho2 = ex * ex + ey * ey + ez * ez;
  if (!(r2 > 4.0f * rho2)) return false;
  const float ir = rsqrtf(r2);
  const float rho = rho2 > 0.0f ? rho2 * rsqrtf(rho2) : 0.0f;
  const float g = r2 * ir - rho;
  const float g3 = g * g * g;
  const float lim = m.w * 2.0f * rho;
  if (!(g3 > 1e-30f) || !(lim <= tau * (1.0f - 1e-6f) * g3)) return false;
  val = (m.x * dx + m.y * dy + m.z * dz) * (ir * ir * ir);
  constexpr float kRel = 1e-5f;
  err = __fdividef(lim, g3) * (1.0f + kRel) + kRel * fabsf(val);
  return true;
}

// Caps of one mesh seen from q, warp-uniform walk: a subtree every lane can take as its far field
// (error bound <= tau) adds its dipole term to wex and its bound to eps; otherwise the warp
// descends, and leaves give exact solid angles. T is the accumulation type. The far field is
// evaluated in FP32 either way (its error bound carries FP32's rounding); with EXACT64 the leaves'
// exact solid angles are FP64, from the original cap vertices, and everything is summed in FP64.
// q is a cell centre, an FP32 value; a lane walks for V cells of one column (heights qz[v]), and
// a subtree is taken as a far field only when it is one for every cell of the warp.
template <typename T, bool EXACT64, int V>
__device__ void caps_walk(const GwnArgs &a, const MeshRec &M, const bool (&active)[V], float qx, float qy,
                          const float (&qz)[V], float tau, T (&wex)[V], T (&eps)[V], bool &corrupt) {
  const int lane = threadIdx.x & 31;
  int cur = M.cap_root, sp = 0, stk0 = 0, stk1 = 0;
  const long long step_limit = 2ll * M.cap_nodes_n + 64;
  auto push = [&](int e) {
    if (sp < kStack) {
      if (sp < 32) {
        if (lane == sp) stk0 = e;
      } else if (lane == sp - 32) {
        stk1 = e;
      }
      ++sp;
    } else {
      corrupt = true;
    }
  };
  for (long long steps = 0;; ++steps) {
    if (cur < 0) {
      if (sp == 0) break;
      --sp;
      cur = __shfl_sync(kFull, sp < 32 ? stk0 : stk1, sp & 31);
    }
    if (steps > step_limit || cur >= M.cap_nodes_n) {
      corrupt = true;
      break;
    }
    const Node *np = M.cap_nodes + cur;
    const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
    const int4 n3 = __ldg(&np->n3);
    const int refs[2] = {n3.x, n3.y}, cnts[2] = {n3.z, n3.w};
    int next = -1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (cnts[k] < 0) continue;
      float4 mom;
      if (cnts[k] == 0) {
        if (refs[k] >= M.cap_inner_n) {
          corrupt = true;
          continue;
        }
        mom = __ldg(M.cap_moment + refs[k]);
      } else {
        if (refs[k] < 0 || cnts[k] > M.cap_recs_n - refs[k]) {
          corrupt = true;
          continue;
        }
        mom = leaf_moment(M.cap_trec + refs[k], cnts[k]);
      }
      float val[V], err[V];
      bool need = false;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        val[v] = 0.0f;
        err[v] = 0.0f;
        const bool far = kFastFarField ? far_field_fast(qx, qy, qz[v], n0, n1, n2, k, mom, tau, val[v], err[v])
                                       : far_field<float>(qx, qy, qz[v], n0, n1, n2, k, mom, tau, val[v], err[v]);
        need |= active[v] && !far;
      }
      if (!__any_sync(kFull, need)) {
#pragma unroll
        for (int v = 0; v < V; ++v)
          if (active[v]) {
            wex[v] += T(val[v]);
            eps[v] += T(err[v]);
          }
        continue;
      }
      if (cnts[k] == 0) {
        if (next < 0) next = refs[k];
        else push(refs[k]);
        continue;
      }
      for (int j = 0; j < cnts[k]; ++j) {
        if (EXACT64) {
          const uint32_t t = __ldg(M.cap_order + refs[k] + j);
          float c3[3][3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const uint32_t i = __ldg(M.cidx + 3ull * t + c);
            c3[c][0] = __ldg(M.cverts + 3ull * i);
            c3[c][1] = __ldg(M.cverts + 3ull * i + 1);
            c3[c][2] = __ldg(M.cverts + 3ull * i + 2);
          }
#pragma unroll
          for (int v = 0; v < V; ++v) {
            V3<T> p[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) p[c] = {T(c3[c][0]) - T(qx), T(c3[c][1]) - T(qy), T(c3[c][2]) - T(qz[v])};
            wex[v] += solid_angle<T>(p[0], p[1], p[2]);
          }
        } else {
          const TriRec *tr = M.cap_trec + refs[k] + j;
          const float4 r0 = __ldg(&tr->r0), r1 = __ldg(&tr->r1), r2 = __ldg(&tr->r2);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const V3<T> p{T(r0.x) - T(qx), T(r0.y) - T(qy), T(r0.z) - T(qz[v])};
            wex[v] += solid_angle<T>(p, {p.x + T(r1.x), p.y + T(r1.y), p.z + T(r1.z)},
                                     {p.x + T(r2.x), p.y + T(r2.y), p.z + T(r2.z)});
          }
        }
      }
    }
    cur = next;
  }
}

// Pass 1: FP32 over warp tiles of 4 x 4 x kGwnTileZ cells of the winding-number meshes, each lane
// walking for kGwnCellsPerLane cells of one column (the node loads, votes and stack are shared).
__global__ __launch_bounds__(kThreads) void k_gwn32(GwnArgs a) {
  constexpr int TX = 4, TY = 4, TZ = kGwnTileZ, V = kGwnCellsPerLane;
  const int lane = threadIdx.x & 31;
  const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
  const BatchDev &B = a.batch;
  bool corrupt = false;
  for (;;) {
    unsigned long long tile = 0;
    if (lane == 0) tile = atomicAdd(a.tile_counter, 1ull);
    tile = __shfl_sync(kFull, tile, 0);
    if (tile >= B.total_gwn_tiles) break;
    const int mesh = find_mesh(B.gwn_tile_starts, B.num_meshes, tile);
    const MeshRec &M = B.recs[mesh];
    const GridDev g = M.g;
    const unsigned long long local = tile - B.gwn_tile_starts[mesh];
    const int tiles_x = (g.nx + TX - 1) / TX, tiles_y = (g.ny + TY - 1) / TY;
    const int tx = static_cast<int>(local % tiles_x);
    const unsigned long long rest = local / tiles_x;
    const int ty = static_cast<int>(rest % tiles_y), tz = static_cast<int>(rest / tiles_y);
    const int vx = tx * TX + lx, vy = ty * TY + ly;
    bool active[V];
    float qz[V], wex[V], eps[V];
    bool any_active = false;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int vz = tz * TZ + lz + 2 * v;
      active[v] = vx < g.nx && vy < g.ny && vz < g.nz;
      any_active |= active[v];
      qz[v] = cell_center(g.oz, vz, g.voxel);
      wex[v] = 0.0f;
      eps[v] = 0.0f;
    }
    const float qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel);
    if (M.cap_root >= 0) caps_walk<float, false, V>(a, M, active, qx, qy, qz, kTau32, wex, eps, corrupt);
    if (!any_active) continue;
    int W[V];
    column_windings<V>(a, M, vx, vy, qz, W);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      if (!active[v]) continue;
      const int vz = tz * TZ + lz + 2 * v;
      const uint64_t cell = (uint64_t(vz) * g.ny + vy) * g.nx + vx;
      const float d = M.dist[cell];
      const float c = fabsf(float(W[v]) - wex[v] * float(kInv4Pi));
      const float e = eps[v] * float(kInv4Pi) + 1e-5f * (1.0f + fabsf(wex[v]));
      const bool band = d <= a.band_voxels * g.voxel;
      if (!band && c - e > 0.5f) {
        M.dist[cell] = -d;
      } else if (band || !(c + e < 0.5f)) {
        const unsigned long long at = atomicAdd(a.refine_count, 1ull);
        a.refine[at] = B.cell_starts[mesh] + cell;
      }
    }
  }
  if (corrupt) atomic_or_err(a.err, kErrCorruptTree);
}

__device__ __forceinline__ void cell_of(const BatchDev &B, uint64_t gcell, int &mesh, int &vx, int &vy, int &vz,
                                        uint64_t &cell) {
  mesh = find_mesh(B.cell_starts, B.num_meshes, gcell);
  const GridDev &g = B.recs[mesh].g;
  cell = gcell - B.cell_starts[mesh];
  vx = static_cast<int>(cell % uint64_t(g.nx));
  vy = static_cast<int>((cell / uint64_t(g.nx)) % uint64_t(g.ny));
  vz = static_cast<int>(cell / (uint64_t(g.nx) * g.ny));
}

// Pass 2: FP64, one listed cell per lane; a persistent grid that reads the list length on the
// device, so the whole pass needs no host round trip. Cells of `in` that the walk with subtree
// bound `tau` leaves undecided are appended to `out`.
__global__ __launch_bounds__(kThreads) void k_gwn64(GwnArgs a, const uint64_t *__restrict__ in,
                                                    const unsigned long long *in_count, float tau, uint64_t *out,
                                                    unsigned long long *out_count) {
  const unsigned long long n = *in_count;
  const int lane = threadIdx.x & 31;
  const BatchDev &B = a.batch;
  bool corrupt = false;
  const unsigned long long warps = (unsigned long long)gridDim.x * (kThreads / kWarp);
  for (unsigned long long base = (blockIdx.x * (kThreads / kWarp) + (threadIdx.x >> 5)) * 32ull; base < n;
       base += warps * 32ull) {
    const unsigned long long k = base + lane;
    const bool active = k < n;
    int mesh, vx, vy, vz;
    uint64_t cell;
    cell_of(B, active ? in[k] : in[base], mesh, vx, vy, vz, cell);
    const MeshRec &M = B.recs[mesh];
    const GridDev g = M.g;
    const float fz = cell_center(g.oz, vz, g.voxel);
    const float qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel);
    double wex[1] = {0.0}, eps[1] = {0.0};
    const float qzs[1] = {fz};
    // lanes of one warp may belong to different meshes: walk each distinct mesh in turn
    const int first_mesh = __shfl_sync(kFull, mesh, 0);
    const bool uniform = __all_sync(kFull, mesh == first_mesh);
    if (uniform) {
      const bool act[1] = {active};
      if (M.cap_root >= 0) caps_walk<double, true, 1>(a, M, act, qx, qy, qzs, tau, wex, eps, corrupt);
    } else {
      unsigned pending = __ballot_sync(kFull, true);
      while (pending) {
        const int leader = __ffs(pending) - 1;
        const int mm = __shfl_sync(kFull, mesh, leader);
        const bool mine = mesh == mm;
        const MeshRec &MM = B.recs[mm];
        const bool act[1] = {active && mine};
        if (MM.cap_root >= 0)
            caps_walk<double, true, 1>(a, MM, act, qx, qy, qzs, tau, wex, eps, corrupt);
        pending &= ~__ballot_sync(kFull, mine);
      }
    }
    if (!active) continue;
    const int W = column_winding(a, M, vx, vy, fz);
    const double c = fabs(double(W) - wex[0] * kInv4Pi);
    const double e = eps[0] * kInv4Pi + 1e-12 * (1.0 + fabs(wex[0]));
    if (c - e > 0.5) {
      M.dist[cell] = -fabsf(M.dist[cell]);
    } else if (!(c + e < 0.5)) {
      const unsigned long long at = atomicAdd(out_count, 1ull);
      out[at] = in[k];
    }
  }
  if (corrupt) atomic_or_err(a.err, kErrCorruptTree);
}

// Pass 3: one block per remaining cell, FP64 sum over every cap triangle of its mesh.
__global__ __launch_bounds__(kThreads) void k_gwn_direct(GwnArgs a) {
  __shared__ double part[kThreads / kWarp];
  const BatchDev &B = a.batch;
  const unsigned long long n = *a.final_count;
  for (unsigned long long k = blockIdx.x; k < n; k += gridDim.x) {
    int mesh, vx, vy, vz;
    uint64_t cell;
    cell_of(B, a.refine[k], mesh, vx, vy, vz, cell);
    const MeshRec &M = B.recs[mesh];
    const GridDev g = M.g;
    const float fz = cell_center(g.oz, vz, g.voxel);
    const double qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel), qz = fz;
    double w = 0.0;
    for (uint32_t t = threadIdx.x; t < M.cap_tris; t += kThreads) {
      V3<double> p[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const uint32_t i = __ldg(M.cidx + 3ull * t + j);
        p[j] = {double(__ldg(M.cverts + 3ull * i)) - qx, double(__ldg(M.cverts + 3ull * i + 1)) - qy,
                double(__ldg(M.cverts + 3ull * i + 2)) - qz};
      }
      w += solid_angle<double>(p[0], p[1], p[2]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(kFull, w, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int i = 0; i < kThreads / kWarp; ++i) s += part[i];
      const int W = column_winding(a, M, vx, vy, fz);
      if (fabs(double(W) - s * kInv4Pi) > 0.5) M.dist[cell] = -fabsf(M.dist[cell]);
    }
    __syncthreads();
  }
}

}  // namespace

size_t gwn_temp_bytes(uint64_t gwn_cells) { return 256 + 2 * ((gwn_cells * 8 + 255) & ~size_t(255)); }

cudaError_t gwn_enqueue(const GwnInput &in, void *temp, int num_sms, cudaStream_t st) {
  const BatchDev &B = in.batch;
  if (B.total_gwn_tiles == 0) return cudaSuccess;
  const size_t list_bytes = (in.gwn_cells * 8 + 255) & ~size_t(255);
  char *base = static_cast<char *>(temp);
  // [0] tiles, [1] pass 1's list, [2] coarse pass 2's, [3] fine pass 2's (the direct sum's cells)
  unsigned long long *counters = reinterpret_cast<unsigned long long *>(base);
  GwnArgs a;
  a.batch = B;
  a.col_start = in.col_start;
  a.col_z = in.col_z;
  a.col_s = in.col_s;
  a.band_voxels = in.band_voxels;
  a.refine = reinterpret_cast<uint64_t *>(base + 256);
  a.refine_count = counters + 1;
  a.direct = reinterpret_cast<uint64_t *>(base + 256 + list_bytes);
  a.direct_count = counters + 2;
  a.final_count = counters + 3;
  a.tile_counter = counters;
  a.err = in.err;
  cudaError_t e = cudaMemsetAsync(counters, 0, 64, st);
  if (e != cudaSuccess) return e;
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gwn32, kThreads, 0);
    per_sm = std::max(per_sm, 1);
  }
  long long blocks = static_cast<long long>(num_sms) * per_sm;
  blocks = std::min<long long>(blocks, static_cast<long long>((B.total_gwn_tiles + 7) / 8));
  k_gwn32<<<static_cast<unsigned>(std::max<long long>(blocks, 1)), kThreads, 0, st>>>(a);
  note_launch();
  k_gwn64<<<static_cast<unsigned>(num_sms * 8), kThreads, 0, st>>>(a, a.refine, a.refine_count, kTau64, a.direct,
                                                                   a.direct_count);
  note_launch();
  // the refine list has been read by now (stream order): it receives the fine pass's leftovers
  k_gwn64<<<static_cast<unsigned>(num_sms * 8), kThreads, 0, st>>>(a, a.direct, a.direct_count, kTau64Fine,
                                                                   a.refine, a.final_count);
  note_launch();
  k_gwn_direct<<<static_cast<unsigned>(num_sms * 4), kThreads, 0, st>>>(a);
  note_launch();
  return cudaGetLastError();
}

uint64_t *gwn_refine_counter(void *temp) { return reinterpret_cast<uint64_t *>(static_cast<char *>(temp)) + 1; }

uint64_t *gwn_direct_counter(void *temp) { return reinterpret_cast<uint64_t *>(static_cast<char *>(temp)) + 3; }
