// Nearest-triangle distance per cell with the sign fused in (replaces the 160-ray estimate of
// src/render/kernels/sdf_bake.cu:39-51 with the exact Euclidean distance).
//
// Work unit: a warp owns a tile of TX x TY x TZ cells (32 lanes, VPL cells per lane stacked in
// z) taken from a global counter, so long and short tiles balance across the persistent grid.
// The warp walks the BVH together: at each node every lane measures its cells against both child
// boxes, __any_sync decides whether any cell still needs a child, and the child with the smaller
// warp-minimum box distance (__reduce_min_sync) goes first. Leaves are tested right away by
// all lanes on the same triangle record (a broadcast 64-byte load), so lanes never diverge. The
// deferred child is pushed as (node, child) and its box is re-tested against the tightened
// bounds when popped. The stack lives in registers, one entry per lane, read with __shfl_sync.
//
// Sign: parity counts the column's crossing heights above each cell (the crossing list is
// built by parity.cu). Winding-number signs are applied afterwards by gwn.cu, which needs the
// unsigned distance to find the near-surface band.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

struct Shape {
  int tx, ty, tz;
};
constexpr Shape kShapes[] = {{4, 4, 2}, {8, 4, 1}, {4, 4, 4}, {8, 4, 2}, {4, 4, 8}, {8, 4, 4}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <int TX, int TY, int TZ, int STACK, bool COUNT>
__global__ __launch_bounds__(kThreads) void k_distance(DistanceArgs a) {
  constexpr int kLayer = TX * TY;
  constexpr int kLanesZ = kWarp / kLayer;
  constexpr int VPL = TZ / kLanesZ;
  static_assert(kLayer * kLanesZ == kWarp && VPL * kLanesZ == TZ, "tile must cover whole warps");
  static_assert(STACK == 32 || STACK == 64, "stack depth is one or two registers per lane");
  const int lane = threadIdx.x & 31;
  const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / kLayer;
  const BatchDev &B = a.batch;
  unsigned long long box_tests = 0, tri_tests = 0;
  bool overflow = false, corrupt = false;

  for (;;) {
    unsigned long long tile = 0;
    if (lane == 0) tile = atomicAdd(a.tile_counter, 1ull);
    tile = __shfl_sync(kFull, tile, 0);
    if (tile >= B.total_tiles) break;
    const int mesh = find_mesh(B.tile_starts, B.num_meshes, tile);
    const MeshRec &M = B.recs[mesh];
    const GridDev g = M.g;
    const Node *__restrict__ nodes = M.nodes;
    const TriRec *__restrict__ tris = M.tris;
    const int num_nodes = M.bvh_nodes, num_tris = M.bvh_tris;
    // A correct tree expands each inner node at most once per tile and pops at most once per
    // push; anything longer means a corrupt tree, and the walk stops with an error.
    const long long step_limit = 2ll * num_nodes + 64;
    const unsigned long long local = tile - B.tile_starts[mesh];
    const int tiles_x = (g.nx + TX - 1) / TX, tiles_y = (g.ny + TY - 1) / TY;
    const int tx = static_cast<int>(local % tiles_x);
    const unsigned long long rest = local / tiles_x;
    const int ty = static_cast<int>(rest % tiles_y);
    const int tz = static_cast<int>(rest / tiles_y);
    const int vx = tx * TX + lx, vy = ty * TY + ly;
    const float px = cell_center(g.ox, vx, g.voxel), py = cell_center(g.oy, vy, g.voxel);
    float pz[VPL], best[VPL];
    bool active[VPL];
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const int vz = tz * TZ + lz + v * kLanesZ;
      active[v] = vx < g.nx && vy < g.ny && vz < g.nz;
      pz[v] = cell_center(g.oz, vz, g.voxel);
      best[v] = active[v] ? __int_as_float(0x7f800000) : -1.0f;  // inactive cells never ask for work
    }

    auto test_leaf = [&](int first, int count) {
      if (first < 0 || count > num_tris - first) {
        corrupt = true;
        return;
      }
      for (int k = 0; k < count; ++k) {
        const TriRec *tr = tris + first + k;
        const float4 r0 = __ldg(&tr->r0), r1 = __ldg(&tr->r1), r2 = __ldg(&tr->r2), r3 = __ldg(&tr->r3);
#pragma unroll
        for (int v = 0; v < VPL; ++v) best[v] = fminf(best[v], point_tri_dist2(px, py, pz[v], r0, r1, r2, r3));
      }
      if (COUNT) tri_tests += static_cast<unsigned long long>(count) * kWarp * VPL;
    };

    int cur = M.root, sp = 0, stk0 = 0, stk1 = 0;
    for (long long steps = 0;; ++steps) {
      if (steps > step_limit || cur >= num_nodes) {
        corrupt = true;
        break;
      }
      if (cur < 0) {
        if (sp == 0) break;
        --sp;
        const int e = __shfl_sync(kFull, (STACK == 32 || sp < 32) ? stk0 : stk1, sp & 31);
        if ((e >> 1) >= num_nodes) {
          corrupt = true;
          break;
        }
        const Node *np = nodes + (e >> 1);
        const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
        const int4 n3 = __ldg(&np->n3);
        float lx0, ly0, lz0, hx0, hy0, hz0;
        int ref, cnt;
        if (e & 1) {
          lx0 = n1.z; ly0 = n1.w; lz0 = n2.x; hx0 = n2.y; hy0 = n2.z; hz0 = n2.w;
          ref = n3.y; cnt = n3.w;
        } else {
          lx0 = n0.x; ly0 = n0.y; lz0 = n0.z; hx0 = n0.w; hy0 = n1.x; hz0 = n1.y;
          ref = n3.x; cnt = n3.z;
        }
        bool want = false;
#pragma unroll
        for (int v = 0; v < VPL; ++v) want |= box_dist2(px, py, pz[v], lx0, ly0, lz0, hx0, hy0, hz0) < best[v];
        if (COUNT) box_tests += kWarp * VPL;
        if (!__any_sync(kFull, want)) continue;
        if (cnt > 0) test_leaf(ref, cnt);
        else cur = ref;
        continue;
      }
      const int node = cur;
      const Node *np = nodes + node;
      const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
      const int4 n3 = __ldg(&np->n3);
      float d0[VPL], d1[VPL];
      float m0 = __int_as_float(0x7f800000), m1 = m0;
      bool w0 = false, w1 = false;
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        d0[v] = box_dist2(px, py, pz[v], n0.x, n0.y, n0.z, n0.w, n1.x, n1.y);
        d1[v] = box_dist2(px, py, pz[v], n1.z, n1.w, n2.x, n2.y, n2.z, n2.w);
        w0 |= d0[v] < best[v];
        w1 |= d1[v] < best[v];
        if (active[v]) {
          m0 = fminf(m0, d0[v]);
          m1 = fminf(m1, d1[v]);
        }
      }
      if (COUNT) box_tests += 2 * kWarp * VPL;
      w0 = __any_sync(kFull, w0) && n3.z >= 0;
      w1 = __any_sync(kFull, w1) && n3.w >= 0;
      const bool second_first =
          __reduce_min_sync(kFull, __float_as_uint(m1)) < __reduce_min_sync(kFull, __float_as_uint(m0));
      const int near_ref = second_first ? n3.y : n3.x, near_cnt = second_first ? n3.w : n3.z;
      const int far_ref = second_first ? n3.x : n3.y, far_cnt = second_first ? n3.z : n3.w;
      bool near_w = second_first ? w1 : w0, far_w = second_first ? w0 : w1;
      cur = -1;
      if (near_w) {
        if (near_cnt > 0) {
          test_leaf(near_ref, near_cnt);
          if (far_w) {
            bool w = false;
#pragma unroll
            for (int v = 0; v < VPL; ++v) w |= (second_first ? d0[v] : d1[v]) < best[v];
            far_w = __any_sync(kFull, w);
          }
        } else {
          cur = near_ref;
        }
      }
      if (far_w) {
        if (cur >= 0) {
          if (sp < STACK) {
            const int e = (node << 1) | (second_first ? 0 : 1);
            if (STACK == 32 || sp < 32) {
              if (lane == sp) stk0 = e;
            } else if (lane == sp - 32) {
              stk1 = e;
            }
            ++sp;
          } else {
            overflow = true;
          }
        } else if (far_cnt > 0) {
          test_leaf(far_ref, far_cnt);
        } else {
          cur = far_ref;
        }
      }
    }

    // Sign and store.
    int inside[VPL];
#pragma unroll
    for (int v = 0; v < VPL; ++v) inside[v] = 0;
    if (M.sign == kSignParity && vx < g.nx && vy < g.ny) {
      const uint64_t col = M.col_base + uint64_t(vy) * g.nx + vx;
      const uint64_t s0 = __ldg(a.col_start + col), s1 = __ldg(a.col_start + col + 1);
      for (uint64_t k = s0; k < s1; ++k) {
        const float zc = __ldg(a.col_z + k);
#pragma unroll
        for (int v = 0; v < VPL; ++v) inside[v] ^= zc > pz[v] ? 1 : 0;
      }
    }
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      if (!active[v]) continue;
      const int vz = tz * TZ + lz + v * kLanesZ;
      const uint64_t cell = (uint64_t(vz) * g.ny + vy) * g.nx + vx;
      const float d = sqrtf(best[v]);
      M.dist[cell] = inside[v] ? -d : d;
    }
  }
  if (overflow) atomic_or_err(a.err, kErrStackOverflow);
  if (corrupt) atomic_or_err(a.err, kErrCorruptTree);
  if (COUNT && a.work_counters && lane == 0) {
    atomicAdd(a.work_counters, box_tests);
    atomicAdd(a.work_counters + 1, tri_tests);
  }
}

template <int I, int STACK, bool COUNT>
cudaError_t launch_shape(const DistanceArgs &a, int num_sms, cudaStream_t st) {
  constexpr Shape s = kShapes[I];
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_distance<s.tx, s.ty, s.tz, STACK, COUNT>, kThreads, 0);
    if (per_sm <= 0) per_sm = 1;
  }
  const unsigned long long warps_needed = a.batch.total_tiles;
  unsigned long long blocks = static_cast<unsigned long long>(num_sms) * per_sm;
  blocks = std::min<unsigned long long>(blocks, (warps_needed + (kThreads / kWarp) - 1) / (kThreads / kWarp));
  if (blocks < 1) blocks = 1;
  cudaError_t e = cudaMemsetAsync(a.tile_counter, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_distance<s.tx, s.ty, s.tz, STACK, COUNT><<<static_cast<unsigned>(blocks), kThreads, 0, st>>>(a);
  note_launch();
  return cudaGetLastError();
}

template <int STACK, bool COUNT>
cudaError_t launch_any(const DistanceArgs &a, int id, int num_sms, cudaStream_t st) {
  switch (id) {
    case 0: return launch_shape<0, STACK, COUNT>(a, num_sms, st);
    case 1: return launch_shape<1, STACK, COUNT>(a, num_sms, st);
    case 2: return launch_shape<2, STACK, COUNT>(a, num_sms, st);
    case 3: return launch_shape<3, STACK, COUNT>(a, num_sms, st);
    case 4: return launch_shape<4, STACK, COUNT>(a, num_sms, st);
    default: return launch_shape<5, STACK, COUNT>(a, num_sms, st);
  }
}

}  // namespace

int tile_shape_count() { return kNumShapes; }

void tile_shape(int id, int &tx, int &ty, int &tz) {
  const Shape s = kShapes[(id < 0 || id >= kNumShapes) ? 0 : id];
  tx = s.tx;
  ty = s.ty;
  tz = s.tz;
}

uint64_t tiles_for(const GridDev &g, int id) {
  int tx, ty, tz;
  tile_shape(id, tx, ty, tz);
  return uint64_t((g.nx + tx - 1) / tx) * uint64_t((g.ny + ty - 1) / ty) * uint64_t((g.nz + tz - 1) / tz);
}

cudaError_t distance_launch(const DistanceArgs &a, int tile_id, int stack_depth, int num_sms, cudaStream_t st) {
  if (a.batch.total_tiles == 0) return cudaSuccess;
  if (stack_depth <= 32) {
    if (a.work_counters) return launch_any<32, true>(a, tile_id, num_sms, st);
    return launch_any<32, false>(a, tile_id, num_sms, st);
  }
  if (a.work_counters) return launch_any<64, true>(a, tile_id, num_sms, st);
  return launch_any<64, false>(a, tile_id, num_sms, st);
}

}  // namespace sdfb
