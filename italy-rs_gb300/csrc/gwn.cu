// Generalized winding number sign for meshes that are not watertight (replaces the 5-ray parity
// vote of src/render/kernels/sdf_bake.cu:53-69, which assumes a closed mesh).
//
// w(q) = sum over triangles of the signed solid angle / 4 pi (Jacobson, Kavan & Sorkine-Hornung
// 2013); a cell is inside when |w| > 0.5. Solid angles are exact for near triangles
// (Van Oosterom & Strackee 1983) and far clusters use the dipole expansion of Barill et al. 2018
// kept to the second term: w_node = (N . r / d^3 + tr(M) / d^3 - 3 r^T M r / d^5) / (4 pi) with
// r = P - q, using the moments stored per inner node by lbvh.cu. A cluster counts as far when
// every cell of the warp's tile is more than beta * radius from P.
//
// Precision split:
//   pass 1 (FP32, every cell, warp tiles, beta = 2): cells farther than band_voxels from the
//     surface whose |w| is clear of 0.5 by more than the accumulated truncation estimate get their
//     sign; all others (the band and ambiguous cells) are appended to a refine list.
//   pass 2 (FP64 accumulation and arithmetic, beta = 3, exact triangles from the original FP32
//     vertices): signs of the refine list; a cell still within its FP64 estimate of 0.5 goes to
//   pass 3 (FP64 direct sum over every triangle, one block per cell).
#include <algorithm>
#include <cstdint>

#include "api_internal.h"
#include "common.cuh"

using namespace sdfb;

namespace {

constexpr int kThreads = 256;
constexpr int kStack = 64;
constexpr float kBeta32 = 2.0f;
constexpr double kBeta64 = 3.0;
constexpr double kInv4Pi = 0.07957747154594767;

template <typename T> struct V3 {
  T x, y, z;
};

// Exact solid angle of triangle (a, b, c) seen from q (Van Oosterom & Strackee).
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

// Second-order dipole expansion of one node at q; adds the truncation estimate A r^2 3/(4pi (d-r)^4).
template <typename T>
__device__ __forceinline__ T expand(const float4 &m0, const float4 &m1, const float4 &m2, const float4 &m3, T qx, T qy,
                                    T qz, T &err) {
  const T rx = T(m0.x) - qx, ry = T(m0.y) - qy, rz = T(m0.z) - qz;
  const T d2 = rx * rx + ry * ry + rz * rz;
  const T d = sqrt(d2);
  const T inv_d3 = T(1) / (d2 * d);
  const T M[9] = {T(m1.w), T(m2.x), T(m2.y), T(m2.z), T(m2.w), T(m3.x), T(m3.y), T(m3.z), T(m3.w)};
  const T nr = T(m1.x) * rx + T(m1.y) * ry + T(m1.z) * rz;
  const T tr = M[0] + M[4] + M[8];
  const T Mr0 = M[0] * rx + M[1] * ry + M[2] * rz, Mr1 = M[3] * rx + M[4] * ry + M[5] * rz,
          Mr2 = M[6] * rx + M[7] * ry + M[8] * rz;
  const T rMr = rx * Mr0 + ry * Mr1 + rz * Mr2;
  const T rad = T(m0.w);
  const T area = sqrt(T(m1.x) * T(m1.x) + T(m1.y) * T(m1.y) + T(m1.z) * T(m1.z));
  const T gap = d - rad;
  err += T(3) * area * rad * rad / (gap * gap * gap * gap);
  return (nr + tr) * inv_d3 - T(3) * rMr * inv_d3 / d2;
}

struct GwnArgs {
  const Node *nodes;
  const TriRec *tris;
  const float4 *mom;
  const uint32_t *leaf_order;
  const float *verts;
  const uint32_t *idx;
  int num_nodes, num_tris;
  GridDev g;
  float band;            // distance below which a cell is in the band
  float *dist;           // unsigned on entry, signed on exit
  uint32_t *refine;      // list of cells for the FP64 pass
  unsigned long long *refine_count;
  unsigned long long *tile_counter;
  uint32_t *err;
};

// Pass 1: FP32 over warp tiles of 4 x 4 x 2 cells.
__global__ __launch_bounds__(kThreads) void k_gwn32(GwnArgs a, long long num_tiles, int tiles_x, int tiles_y) {
  constexpr int TX = 4, TY = 4, TZ = 2;
  const int lane = threadIdx.x & 31;
  const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
  const GridDev g = a.g;
  bool corrupt = false;
  const long long step_limit = 2ll * a.num_nodes + 64;
  for (;;) {
    long long tile = 0;
    if (lane == 0) tile = static_cast<long long>(atomicAdd(a.tile_counter, 1ull));
    tile = __shfl_sync(kFull, tile, 0);
    if (tile >= num_tiles) break;
    const int tx = static_cast<int>(tile % tiles_x);
    const long long rest = tile / tiles_x;
    const int ty = static_cast<int>(rest % tiles_y), tz = static_cast<int>(rest / tiles_y);
    const int vx = tx * TX + lx, vy = ty * TY + ly, vz = tz * TZ + lz;
    const bool active = vx < g.nx && vy < g.ny && vz < g.nz;
    const float qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel),
                qz = cell_center(g.oz, vz, g.voxel);
    float w = 0.0f, err = 0.0f;
    int cur = 0, sp = 0, stk0 = 0, stk1 = 0;
    auto leaf = [&](int first, int count) {
      if (first < 0 || count > a.num_tris - first) {
        corrupt = true;
        return;
      }
      for (int k = 0; k < count; ++k) {
        const TriRec *tr = a.tris + first + k;
        const float4 r0 = __ldg(&tr->r0), r1 = __ldg(&tr->r1), r2 = __ldg(&tr->r2);
        const V3<float> p{r0.x - qx, r0.y - qy, r0.z - qz};
        w += solid_angle<float>(p, {p.x + r1.x, p.y + r1.y, p.z + r1.z}, {p.x + r2.x, p.y + r2.y, p.z + r2.z});
      }
    };
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
      if (steps > step_limit || cur >= a.num_nodes) {
        corrupt = true;
        break;
      }
      const int4 n3 = __ldg(&a.nodes[cur].n3);
      const int refs[2] = {n3.x, n3.y}, cnts[2] = {n3.z, n3.w};
      int next = -1;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (cnts[k] < 0) continue;
        if (cnts[k] > 0) {
          leaf(refs[k], cnts[k]);
          continue;
        }
        const float4 *mp = a.mom + 4ll * refs[k];
        const float4 m0 = __ldg(mp), m1 = __ldg(mp + 1);
        const float dx = m0.x - qx, dy = m0.y - qy, dz = m0.z - qz;
        const bool far = dx * dx + dy * dy + dz * dz > (kBeta32 * m0.w) * (kBeta32 * m0.w);
        if (__all_sync(kFull, far || !active)) {
          w += expand<float>(m0, m1, __ldg(mp + 2), __ldg(mp + 3), qx, qy, qz, err);
        } else if (next < 0) {
          next = refs[k];
        } else {
          push(refs[k]);
        }
      }
      cur = next;
    }
    if (!active) continue;
    const uint64_t cell = (uint64_t(vz) * g.ny + vy) * g.nx + vx;
    const float d = a.dist[cell];
    const float aw = fabsf(w * static_cast<float>(kInv4Pi));
    const float e = err * static_cast<float>(kInv4Pi) + 1e-4f + 1e-5f * fabsf(w);
    if (d <= a.band || fabsf(aw - 0.5f) <= e) {
      const unsigned long long at = atomicAdd(a.refine_count, 1ull);
      a.refine[at] = static_cast<uint32_t>(cell);
    } else if (aw > 0.5f) {
      a.dist[cell] = -d;
    }
  }
  if (corrupt) atomic_or_err(a.err, kErrCorruptTree);
}

// Pass 2: FP64, one cell per lane (cells from the refine list), exact triangles from the original
// vertices. Cells still ambiguous are appended to the direct-sum list.
__global__ __launch_bounds__(kThreads) void k_gwn64(GwnArgs a, unsigned long long n, uint32_t *direct,
                                                    unsigned long long *direct_count) {
  const int lane = threadIdx.x & 31;
  const GridDev g = a.g;
  bool corrupt = false;
  const long long step_limit = 2ll * a.num_nodes + 64;
  const unsigned long long warps = (unsigned long long)gridDim.x * (kThreads / kWarp);
  for (unsigned long long base = (blockIdx.x * (kThreads / kWarp) + (threadIdx.x >> 5)) * 32ull; base < n;
       base += warps * 32ull) {
    const unsigned long long k = base + lane;
    const bool active = k < n;
    const uint32_t cell = active ? a.refine[k] : 0u;
    const int vx = static_cast<int>(cell % uint32_t(g.nx)), vy = static_cast<int>((cell / uint32_t(g.nx)) % uint32_t(g.ny)),
              vz = static_cast<int>(cell / (uint32_t(g.nx) * uint32_t(g.ny)));
    const double qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel),
                 qz = cell_center(g.oz, vz, g.voxel);
    double w = 0.0, err = 0.0;
    int cur = 0, sp = 0, stk0 = 0, stk1 = 0;
    auto vert = [&](uint32_t i) -> V3<double> {
      return {double(__ldg(a.verts + 3ull * i)) - qx, double(__ldg(a.verts + 3ull * i + 1)) - qy,
              double(__ldg(a.verts + 3ull * i + 2)) - qz};
    };
    auto leaf = [&](int first, int count) {
      if (first < 0 || count > a.num_tris - first) {
        corrupt = true;
        return;
      }
      for (int j = 0; j < count; ++j) {
        const uint32_t t = __ldg(a.leaf_order + first + j);
        w += solid_angle<double>(vert(__ldg(a.idx + 3ull * t)), vert(__ldg(a.idx + 3ull * t + 1)),
                                 vert(__ldg(a.idx + 3ull * t + 2)));
      }
    };
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
      if (steps > step_limit || cur >= a.num_nodes) {
        corrupt = true;
        break;
      }
      const int4 n3 = __ldg(&a.nodes[cur].n3);
      const int refs[2] = {n3.x, n3.y}, cnts[2] = {n3.z, n3.w};
      int next = -1;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if (cnts[c] < 0) continue;
        if (cnts[c] > 0) {
          leaf(refs[c], cnts[c]);
          continue;
        }
        const float4 *mp = a.mom + 4ll * refs[c];
        const float4 m0 = __ldg(mp), m1 = __ldg(mp + 1);
        const double dx = double(m0.x) - qx, dy = double(m0.y) - qy, dz = double(m0.z) - qz;
        const double lim = kBeta64 * double(m0.w);
        const bool far = dx * dx + dy * dy + dz * dz > lim * lim;
        if (__all_sync(kFull, far || !active)) {
          w += expand<double>(m0, m1, __ldg(mp + 2), __ldg(mp + 3), qx, qy, qz, err);
        } else if (next < 0) {
          next = refs[c];
        } else {
          push(refs[c]);
        }
      }
      cur = next;
    }
    if (!active) continue;
    const double aw = fabs(w * kInv4Pi);
    const double e = err * kInv4Pi + 1e-9;
    if (fabs(aw - 0.5) <= e) {
      const unsigned long long at = atomicAdd(direct_count, 1ull);
      direct[at] = cell;
    } else if (aw > 0.5) {
      a.dist[cell] = -fabsf(a.dist[cell]);
    }
  }
  if (corrupt) atomic_or_err(a.err, kErrCorruptTree);
}

// Pass 3: one block per remaining cell, FP64 direct sum over every triangle.
__global__ __launch_bounds__(kThreads) void k_gwn_direct(GwnArgs a, const uint32_t *cells,
                                                         const unsigned long long *count) {
  __shared__ double part[kThreads / kWarp];
  const GridDev g = a.g;
  for (unsigned long long k = blockIdx.x; k < *count; k += gridDim.x) {
    const uint32_t cell = cells[k];
    const int vx = static_cast<int>(cell % uint32_t(g.nx)), vy = static_cast<int>((cell / uint32_t(g.nx)) % uint32_t(g.ny)),
              vz = static_cast<int>(cell / (uint32_t(g.nx) * uint32_t(g.ny)));
    const double qx = cell_center(g.ox, vx, g.voxel), qy = cell_center(g.oy, vy, g.voxel),
                 qz = cell_center(g.oz, vz, g.voxel);
    double w = 0.0;
    for (int t = threadIdx.x; t < a.num_tris; t += kThreads) {
      V3<double> p[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const uint32_t i = __ldg(a.idx + 3ull * t + j);
        p[j] = {double(__ldg(a.verts + 3ull * i)) - qx, double(__ldg(a.verts + 3ull * i + 1)) - qy,
                double(__ldg(a.verts + 3ull * i + 2)) - qz};
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
      if (fabs(s * kInv4Pi) > 0.5) a.dist[cell] = -fabsf(a.dist[cell]);
    }
    __syncthreads();
  }
}

}  // namespace

sdfb_status gwn_apply(sdfb_ctx *ctx, cudaStream_t st, const MeshDev &m, const BakeInput &in,
                      const sdfb_grid_desc &grid, const sdfb_opts &opts, float *d_dist, uint32_t *d_err) {
  if (!m.moments) return ctx_fail(ctx, SDFB_ERR_INTERNAL, "winding-number moments were not built");
  const uint64_t cells = uint64_t(grid.nx) * grid.ny * grid.nz;
  if (cells >= (1ull << 32))
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "winding-number sign supports grids below 2^32 cells");
  // refine list + direct list + counters
  const size_t need = cells * 4 + 256 + cells * 4 + 256;
  if (!ctx->gwn_tmp.ensure(need)) return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "winding-number workspace");
  char *base = static_cast<char *>(ctx->gwn_tmp.p);
  unsigned long long *counters = reinterpret_cast<unsigned long long *>(base);  // [0] tiles [1] refine [2] direct
  uint32_t *refine = reinterpret_cast<uint32_t *>(base + 256);
  uint32_t *direct = reinterpret_cast<uint32_t *>(base + 256 + ((cells * 4 + 255) & ~255ull));
  cudaError_t e = cudaMemsetAsync(counters, 0, 64, st);
  if (e != cudaSuccess) return ctx_cuda(ctx, e, "memset");
  GwnArgs a;
  a.nodes = m.nodes;
  a.tris = m.tris;
  a.mom = m.moments;
  a.leaf_order = m.leaf_order;
  a.verts = in.verts;
  a.idx = in.idx;
  a.num_nodes = static_cast<int>(std::max<uint32_t>(m.num_tris, 2) - 1);
  a.num_tris = static_cast<int>(m.num_tris);
  a.g = to_dev(grid);
  a.band = opts.band_voxels * grid.voxel_size;
  a.dist = d_dist;
  a.refine = refine;
  a.refine_count = counters + 1;
  a.tile_counter = counters;
  a.err = d_err;
  const int tiles_x = (grid.nx + 3) / 4, tiles_y = (grid.ny + 3) / 4, tiles_z = (grid.nz + 1) / 2;
  const long long num_tiles = static_cast<long long>(tiles_x) * tiles_y * tiles_z;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gwn32, kThreads, 0);
  long long blocks = static_cast<long long>(ctx->num_sms) * std::max(per_sm, 1);
  blocks = std::min<long long>(blocks, (num_tiles + 7) / 8);
  k_gwn32<<<static_cast<unsigned>(std::max<long long>(blocks, 1)), kThreads, 0, st>>>(a, num_tiles, tiles_x, tiles_y);
  note_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return ctx_cuda(ctx, e, "k_gwn32");
  // The refine count sizes pass 2's grid: read it back (the bake synchronises at its end anyway).
  unsigned long long n_refine = 0;
  if ((e = cudaMemcpyAsync(&n_refine, counters + 1, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return ctx_cuda(ctx, e, "refine count");
  if (n_refine) {
    const unsigned long long warps = (n_refine + 31) / 32;
    const unsigned g2 = static_cast<unsigned>(std::min<unsigned long long>((warps + 7) / 8, 65535ull * 8));
    k_gwn64<<<std::max(g2, 1u), kThreads, 0, st>>>(a, n_refine, direct, counters + 2);
    note_launch();
    k_gwn_direct<<<static_cast<unsigned>(ctx->num_sms * 4), kThreads, 0, st>>>(a, direct, counters + 2);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return ctx_cuda(ctx, e, "k_gwn64");
  }
  ctx->gwn_refined = n_refine;
  return SDFB_OK;
}
