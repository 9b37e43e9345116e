// Nearest-triangle distance per cell with the sign fused in (replaces the 160-ray estimate of
// src/render/kernels/sdf_bake.cu:39-51 with the exact Euclidean distance).
//
// Work unit: a warp owns a tile of TX x TY x TZ cells (32 lanes, VPL cells per lane stacked in
// z) taken from its block's chunk of neighbouring tiles, so long and short tiles balance across the
// persistent grid. The warp walks the BVH together: at each node every lane measures its cells
// against both child boxes, __any_sync decides whether any cell still needs a child, and the child
// whose box centre is nearer the tile's centre goes first. Leaves are tested right away by
// all lanes on the same triangle record (a broadcast 80-byte load), so lanes never diverge. The
// deferred child is pushed as (node, child) and its box is re-tested against the tightened
// bounds when popped. The stack lives in registers, one entry per lane, read with __shfl_sync.
//
// Two passes keep one expensive tile from holding the whole GPU. Cells far inside a closed surface
// are nearly equidistant to much of it, so their tiles walk a large part of the tree; a single
// such tile, taken late by one warp, used to run alone for a quarter of the kernel. In pass A a
// walk looks at the chunk counter every `step_budget` steps; once every chunk has been handed out
// (the tail, where a long walk would keep one SM busy while the rest idle) it stops, stores its
// cells' current bounds (squared distances, upper bounds of the answer) in the output and appends
// the tile to a deferred list. Pass B gives each deferred tile a whole block: the tree is cut into
// 2^kSplitBits subtrees below the root, the block's warps take subtrees from a shared counter,
// each walks its subtree for all the tile's cells starting from the stored bounds, and the warps
// publish their bounds to shared memory (atomicMin on the float bits, valid for non-negative
// values) after every subtree.
//
// Sign: parity counts the column's crossing heights above each cell (the crossing list is
// built by parity.cu). Winding-number signs are applied afterwards by gwn.cu, which needs the
// unsigned distance to find the near-surface band.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

// Pass A: a block takes chunks of consecutive tiles (a brick of neighbouring tiles) and its warps
// take tiles from the block's chunk, so the warps sharing an SM's L1 walk overlapping parts of the
// tree. Two blocks of 16 warps per SM: the walk waits on dependent node and record loads, and 32
// resident warps hide more of that latency than 20 warps without spills did (64-mesh batch
// 281 -> 259 ms; 24 warps at 80 registers: 267 ms). Pass B's block shares one tile: 16 warps over
// 64 subtrees, which also keeps a small grid (fewer tiles than the GPU holds warps) busy once its
// tiles are deferred.
constexpr int kThreadsA = 512;
constexpr int kMinBlocksA = 2;  // 32 warps per SM: 64 registers a thread, some of them spilled to L1
constexpr int kWarpsPerBlockA = kThreadsA / kWarp;
// Tile order within a mesh: bricks of kBrickX x kBrickY x kBrickZ tiles, x fastest inside a brick
// and across bricks. Tiles of a partial brick beyond the grid have no active cell.
constexpr int kBrickX = 4, kBrickY = 4, kBrickZ = 2, kBrickTiles = kBrickX * kBrickY * kBrickZ;
constexpr int kChunkMax = 32;  // tiles per chunk when there are plenty
constexpr unsigned long long kNoTile = ~0ull;
constexpr int kDispatchSpin = 1 << 22;  // bound on a warp's wait for its block's next chunk
constexpr int kThreads = 512;
constexpr int kSplitBits = 6;  // pass B: 64 subtrees per deferred tile
constexpr float kInf = __builtin_huge_valf();

struct Shape {
  int tx, ty, tz;
};
constexpr Shape kShapes[] = {{4, 4, 2}, {8, 4, 1}, {4, 4, 4}, {8, 4, 2}, {4, 4, 8}, {8, 4, 4}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

struct WalkStats {
  unsigned long long box_tests = 0, tri_tests = 0, plane_tests = 0, rect_tests = 0;
  bool overflow = false, corrupt = false;
};

// A tile's cells as one lane sees them.
template <int TX, int TY, int TZ>
struct TileCells {
  static constexpr int kLayer = TX * TY;
  static constexpr int kLanesZ = kWarp / kLayer;
  static constexpr int VPL = TZ / kLanesZ;
  static_assert(kLayer * kLanesZ == kWarp && VPL * kLanesZ == TZ, "tile must cover whole warps");
  const MeshRec *M;
  GridDev g;
  int vx, vy, vz0;  // this lane's column and first z; cell v is at z = vz0 + v * kLanesZ
  float px, py, pz[VPL];
  bool active[VPL];
  float cx, cy, cz;  // tile centre

  __device__ __forceinline__ void locate(const BatchDev &B, unsigned long long tile, int lane) {
    const int mesh = find_mesh(B.tile_starts, B.num_meshes, tile);
    M = &B.recs[mesh];
    g = M->g;
    const unsigned long long local = tile - B.tile_starts[mesh];
    const int tiles_x = (g.nx + TX - 1) / TX, tiles_y = (g.ny + TY - 1) / TY;
    const int bricks_x = (tiles_x + kBrickX - 1) / kBrickX, bricks_y = (tiles_y + kBrickY - 1) / kBrickY;
    const unsigned long long brick = local / kBrickTiles;
    const int w = static_cast<int>(local % kBrickTiles);
    const unsigned long long rest = brick / bricks_x;
    const int tx = static_cast<int>(brick % bricks_x) * kBrickX + w % kBrickX;
    const int ty = static_cast<int>(rest % bricks_y) * kBrickY + (w / kBrickX) % kBrickY;
    const int tz = static_cast<int>(rest / bricks_y) * kBrickZ + w / (kBrickX * kBrickY);
    cx = g.ox + (float(tx * TX) + 0.5f * TX) * g.voxel;
    cy = g.oy + (float(ty * TY) + 0.5f * TY) * g.voxel;
    cz = g.oz + (float(tz * TZ) + 0.5f * TZ) * g.voxel;
    vx = tx * TX + lane % TX;
    vy = ty * TY + (lane / TX) % TY;
    vz0 = tz * TZ + lane / kLayer;
    px = cell_center(g.ox, vx, g.voxel);
    py = cell_center(g.oy, vy, g.voxel);
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const int vz = vz0 + v * kLanesZ;
      active[v] = vx < g.nx && vy < g.ny && vz < g.nz;
      pz[v] = cell_center(g.oz, vz, g.voxel);
    }
  }

  __device__ __forceinline__ uint64_t cell(int v) const {
    return (uint64_t(vz0 + v * kLanesZ) * g.ny + vy) * g.nx + vx;
  }
};

template <int VPL, bool COUNT>
__device__ __forceinline__ void test_leaf(const DistTri *__restrict__ tris, int num_tris, int first, int count,
                                          float px, float py, const float (&pz)[VPL], float (&best)[VPL],
                                          WalkStats &ws) {
  if (first < 0 || count > num_tris - first) {
    ws.corrupt = true;
    return;
  }
  for (int k = 0; k < count; ++k) {
    const DistTri *tr = tris + first + k;
    const float4 q0 = __ldg(&tr->q0), q3 = __ldg(&tr->q3), q1 = __ldg(&tr->q1), q2 = __ldg(&tr->q2),
                 q4 = __ldg(&tr->q4);
    // The x and y parts of the frame coordinates are shared by the lane's cells.
    const float ax = px - q0.x, ay = py - q0.y;
    const float sh = fmaf(ay, q3.y, ax * q3.x);
    // The squared distance to the triangle's plane, h^2, bounds the squared distance to the
    // triangle from below: skip the triangle when no cell could improve.
    float az[VPL], h2[VPL];
    bool need = false;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      az[v] = pz[v] - q0.z;
      const float h = fmaf(az[v], q3.z, sh);
      h2[v] = h * h;
      need |= h2[v] < best[v];
    }
    if (COUNT) ws.plane_tests += kWarp * VPL;
    if (!__any_sync(kFull, need)) continue;
    // Then the distance to the triangle's bounding rectangle in its own plane, [0, b] x [0, c2],
    // with h^2: much tighter where a cell is near the triangle's plane but beside the triangle
    // (most cells that pass the plane bound). Its u part is edge AB's clamp in the full test.
    const float su = fmaf(ay, q1.y, ax * q1.x), sv = fmaf(ay, q2.y, ax * q2.x);
    // The in-plane coordinates are formed again by the full test (about one screen in eight
    // passes), so they need not stay live across the vote.
    need = false;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const float du = dist_to_range(fmaf(az[v], q1.z, su), q0.w);
      const float dw = dist_to_range(fmaf(az[v], q2.z, sv), q2.w);
      need |= fmaf(du, du, fmaf(dw, dw, h2[v])) < best[v];
    }
    if (COUNT) ws.rect_tests += kWarp * VPL;
    if (!__any_sync(kFull, need)) continue;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      const float u = fmaf(az[v], q1.z, su), w = fmaf(az[v], q2.z, sv);
      best[v] = fminf(best[v], h2[v] + inplane_dist2(u, w, dist_to_range(u, q0.w), q0.w, q1.w, q2.w, q3.w, q4));
    }
    if (COUNT) ws.tri_tests += kWarp * VPL;
  }
}

// When a walk may stop early: every `every` steps it reads the pass's tile counter, and it stops
// once every tile has been handed out (the pass is in its tail, where a long walk would run
// alone). every = 0: never.
struct TailCheck {
  const unsigned long long *counter;
  unsigned long long total;
  int every;
};

// Walks the subtree below inner node `start` for this lane's cells, tightening best[] (squared
// distances; inactive cells hold -1 and never ask for work). Returns false when the walk stopped
// early by the tail check with work left (best[] then holds upper bounds); a walk past the limit a
// correct tree allows stops with the corrupt flag.
// Bounds of one walk: the step limit (a correct tree expands each inner node at most once per walk
// and pops at most once per push) and the usable stack entries. The fault-injection bits shrink
// them so that the error paths behind them can be tested.
struct WalkLimits {
  int steps, stack;
};
template <int STACK>
__device__ __forceinline__ WalkLimits walk_limits(int num_nodes, int fault) {
  WalkLimits l;
  l.steps = num_nodes > (INT_MAX - 64) / 2 ? INT_MAX - 1 : 2 * num_nodes + 64;
  l.stack = STACK;
  if (fault) {
    if (fault & kFaultStepLimit) l.steps = 8;
    if ((fault & kFaultStackAll) || (STACK == 32 && (fault & kFaultShallowStack))) l.stack = 2;
  }
  return l;
}

template <int VPL, int STACK, bool COUNT>
__device__ __forceinline__ bool walk(const Node *__restrict__ nodes, const DistTri *__restrict__ tris, int num_nodes,
                                     int num_tris, int start, TailCheck tail, WalkLimits lim, int lane, float tcx,
                                     float tcy, float tcz, float px, float py, const float (&pz)[VPL],
                                     float (&best)[VPL], WalkStats &ws) {
  static_assert(STACK == 32 || STACK == 64, "stack depth is one or two registers per lane");
  const int step_limit = lim.steps;
  int next_check = tail.every > 0 ? tail.every : INT_MAX;
  int cur = start, sp = 0, stk0 = 0, stk1 = 0;
  for (int steps = 0;; ++steps) {
    if (steps > step_limit || cur >= num_nodes) {
      ws.corrupt = true;
      return true;
    }
    if (steps >= next_check) {
      unsigned long long handed = 0;
      if (lane == 0) handed = *reinterpret_cast<const volatile unsigned long long *>(tail.counter);
      handed = __shfl_sync(kFull, handed, 0);
      if (handed >= tail.total) return false;
      next_check = steps + tail.every;
    }
    if (cur < 0) {
      if (sp == 0) return true;
      --sp;
      const int e = __shfl_sync(kFull, (STACK == 32 || sp < 32) ? stk0 : stk1, sp & 31);
      if ((e >> 1) >= num_nodes) {
        ws.corrupt = true;
        return true;
      }
      const Node *np = nodes + (e >> 1);
      const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
      const int4 n3 = __ldg(&np->n3);
      float cx, cy, cz, ex, ey, ez;  // the popped child's box: centre and half extent
      int ref, cnt;
      if (e & 1) {
        cx = n1.z; cy = n1.w; cz = n2.x; ex = n2.y; ey = n2.z; ez = n2.w;
        ref = n3.y; cnt = n3.w;
      } else {
        cx = n0.x; cy = n0.y; cz = n0.z; ex = n0.w; ey = n1.x; ez = n1.y;
        ref = n3.x; cnt = n3.z;
      }
      bool want = false;
#pragma unroll
      for (int v = 0; v < VPL; ++v) want |= box_dist2(px, py, pz[v], cx, cy, cz, ex, ey, ez) < best[v];
      if (COUNT) ws.box_tests += kWarp * VPL;
      if (!__any_sync(kFull, want)) continue;
      if (cnt > 0) test_leaf<VPL, COUNT>(tris, num_tris, ref, cnt, px, py, pz, best, ws);
      else cur = ref;
      continue;
    }
    const int node = cur;
    const Node *np = nodes + node;
    const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
    const int4 n3 = __ldg(&np->n3);
    // Only the votes stay live: when the near child is a leaf, the far child's box is read again
    // (an L1 hit) and re-tested after it, which keeps the per-cell distances out of the registers
    // across the leaf test (fewer spills: 64-mesh batch 249 -> 244 ms).
    bool w0 = false, w1 = false;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      w0 |= box_dist2(px, py, pz[v], n0.x, n0.y, n0.z, n0.w, n1.x, n1.y) < best[v];
      w1 |= box_dist2(px, py, pz[v], n1.z, n1.w, n2.x, n2.y, n2.z, n2.w) < best[v];
    }
    if (COUNT) ws.box_tests += 2 * kWarp * VPL;
    w0 = __any_sync(kFull, w0) && n3.z >= 0;
    w1 = __any_sync(kFull, w1) && n3.w >= 0;
    // Near child first: the one whose box centre is nearer the tile's centre (the same on every
    // lane). The centres order the children where the tile lies inside both boxes, as near the
    // top of the tree; the box distances tie there (3-7% fewer tests than ordering by them).
    const float q0x = tcx - n0.x, q0y = tcy - n0.y, q0z = tcz - n0.z;
    const float q1x = tcx - n1.z, q1y = tcy - n1.w, q1z = tcz - n2.x;
    const bool second_first = q1x * q1x + q1y * q1y + q1z * q1z < q0x * q0x + q0y * q0y + q0z * q0z;
    const int near_ref = second_first ? n3.y : n3.x, near_cnt = second_first ? n3.w : n3.z;
    const int far_ref = second_first ? n3.x : n3.y, far_cnt = second_first ? n3.z : n3.w;
    bool near_w = second_first ? w1 : w0, far_w = second_first ? w0 : w1;
    cur = -1;
    if (near_w && near_cnt == 0) {
      cur = near_ref;
      if (far_w) {
        if (sp < lim.stack) {
          const int e = (node << 1) | (second_first ? 0 : 1);
          if (STACK == 32 || sp < 32) {
            if (lane == sp) stk0 = e;
          } else if (lane == sp - 32) {
            stk1 = e;
          }
          ++sp;
        } else {
          ws.overflow = true;
        }
      }
      continue;
    }
    if (near_w) {
      test_leaf<VPL, COUNT>(tris, num_tris, near_ref, near_cnt, px, py, pz, best, ws);
      if (far_w) {
        bool w = false;
        const Node *fp = nodes + node;
        const float4 f0 = __ldg(&fp->n0), f1 = __ldg(&fp->n1), f2 = __ldg(&fp->n2);
#pragma unroll
        for (int v = 0; v < VPL; ++v)
          w |= (second_first ? box_dist2(px, py, pz[v], f0.x, f0.y, f0.z, f0.w, f1.x, f1.y)
                             : box_dist2(px, py, pz[v], f1.z, f1.w, f2.x, f2.y, f2.z, f2.w)) < best[v];
        far_w = __any_sync(kFull, w);
      }
    }
    if (far_w) {
      if (far_cnt > 0) test_leaf<VPL, COUNT>(tris, num_tris, far_ref, far_cnt, px, py, pz, best, ws);
      else cur = far_ref;
    }
  }
}

// Signs (parity) and writes a tile's distances.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void store_cells(const DistanceArgs &a, const TileCells<TX, TY, TZ> &c,
                                            const float (&best)[TileCells<TX, TY, TZ>::VPL]) {
  constexpr int VPL = TileCells<TX, TY, TZ>::VPL;
  const MeshRec &M = *c.M;
  int inside[VPL];
#pragma unroll
  for (int v = 0; v < VPL; ++v) inside[v] = 0;
  if (M.sign == kSignParity && c.vx < c.g.nx && c.vy < c.g.ny) {
    const uint64_t col = M.col_base + uint64_t(c.vy) * c.g.nx + c.vx;
    const uint64_t s0 = __ldg(a.col_start + col), s1 = __ldg(a.col_start + col + 1);
    for (uint64_t k = s0; k < s1; ++k) {
      const float zc = __ldg(a.col_z + k);
#pragma unroll
      for (int v = 0; v < VPL; ++v) inside[v] ^= zc > c.pz[v] ? 1 : 0;
    }
  }
#pragma unroll
  for (int v = 0; v < VPL; ++v) {
    if (!c.active[v]) continue;
    const float d = sqrtf(best[v]);
    M.dist[c.cell(v)] = inside[v] ? -d : d;
  }
}

template <bool COUNT>
__device__ __forceinline__ void flush_stats(const DistanceArgs &a, const WalkStats &ws, int lane) {
  if (ws.overflow) atomic_or_err(a.err, kErrStackOverflow);
  if (ws.corrupt) atomic_or_err(a.err, kErrCorruptTree);
  if (COUNT && a.work_counters && lane == 0) {
    atomicAdd(a.work_counters, ws.box_tests);
    atomicAdd(a.work_counters + 1, ws.tri_tests);
    atomicAdd(a.work_counters + 3, ws.plane_tests);
    atomicAdd(a.work_counters + 4, ws.rect_tests);
  }
}

// Hands lane 0 of a warp its next tile. *state packs the block's current chunk (high 32 bits)
// and the next index within it (low 32 bits); chunks come from the global counter. The warp that
// draws index == per_chunk moves the block to a new chunk; warps drawing past it wait for that
// (bounded: past the limit the dispatch error is raised and the warp stops). Returns kNoTile when
// every chunk has been handed out.
__device__ unsigned long long next_tile(unsigned long long *state, unsigned long long *chunks,
                                        unsigned long long per_chunk, unsigned long long total_chunks,
                                        unsigned long long total_tiles, uint32_t *err, int fault) {
  // Fault injection: nobody moves the block on, and the waits are short.
  const bool stuck = fault & kFaultDispatch;
  const int spin_limit = stuck ? (1 << 12) : kDispatchSpin;
  for (;;) {
    const unsigned long long old = atomicAdd(state, 1ull);
    const unsigned long long chunk = old >> 32, idx = old & 0xffffffffull;
    if (chunk >= total_chunks) return kNoTile;
    if (idx < per_chunk) {
      const unsigned long long t = chunk * per_chunk + idx;
      if (t < total_tiles) return t;
      continue;  // past the end of the last chunk: draw on until the block moves on
    }
    if (idx == per_chunk && !stuck) {
      atomicExch(state, atomicAdd(chunks, 1ull) << 32);
      continue;
    }
    const volatile unsigned long long *vs = state;
    int spin = 0;
    while ((*vs >> 32) == chunk && spin < spin_limit) ++spin;
    if (spin == spin_limit) {
      atomic_or_err(err, kErrDispatch);
      return kNoTile;
    }
  }
}

// Pass A: warps take tiles from their block's chunk, blocks take chunks from a global counter; a
// tile still walking in the pass's tail (every chunk handed out) is deferred to pass B.
template <int TX, int TY, int TZ, int STACK, bool COUNT>
__global__ __launch_bounds__(kThreadsA, kMinBlocksA) void k_distance(DistanceArgs a) {
  using Cells = TileCells<TX, TY, TZ>;
  constexpr int VPL = Cells::VPL;
  const int lane = threadIdx.x & 31;
  const BatchDev &B = a.batch;
  WalkStats ws;
  const unsigned long long total_chunks = (B.total_tiles + a.chunk_tiles - 1) / a.chunk_tiles;
  TailCheck tail{a.tile_counter, total_chunks,
                 (a.defer_list && a.step_budget > 0) ? static_cast<int>(min(a.step_budget, 1ll << 30)) : 0};
  const TailCheck never{nullptr, 0, 0};
  __shared__ unsigned long long s_state;
  if (threadIdx.x == 0) s_state = atomicAdd(a.tile_counter, 1ull) << 32;
  __syncthreads();

  for (;;) {
    unsigned long long tile = 0;
    if (lane == 0)
      tile = next_tile(&s_state, a.tile_counter, a.chunk_tiles, total_chunks, B.total_tiles, a.err, a.fault);
    tile = __shfl_sync(kFull, tile, 0);
    if (tile == kNoTile) break;
    // Only what the walk reads stays live across it; the tile's cell indices, activity and output
    // pointer are located again afterwards.
    float best[VPL], px, py, pz[VPL], tcx, tcy, tcz;
    const Node *nodes;
    const DistTri *tris;
    int bvh_nodes, bvh_tris, root;
    {
      Cells c0;
      c0.locate(B, tile, lane);
#pragma unroll
      for (int v = 0; v < VPL; ++v) {
        best[v] = c0.active[v] ? kInf : -1.0f;
        pz[v] = c0.pz[v];
      }
      px = c0.px;
      py = c0.py;
      tcx = c0.cx;
      tcy = c0.cy;
      tcz = c0.cz;
      nodes = c0.M->nodes;
      tris = c0.M->tris;
      bvh_nodes = c0.M->bvh_nodes;
      bvh_tris = c0.M->bvh_tris;
      root = c0.M->root;
    }
    const WalkLimits lim = walk_limits<STACK>(bvh_nodes, a.fault);
    bool done = walk<VPL, STACK, COUNT>(nodes, tris, bvh_nodes, bvh_tris, root, tail, lim, lane, tcx, tcy, tcz, px, py,
                                        pz, best, ws);
    Cells c;
    c.locate(B, tile, lane);
    const MeshRec &M = *c.M;
    if (!done) {
      unsigned long long slot = 0;
      if (lane == 0) slot = atomicAdd(a.defer_counters, 1ull);
      slot = __shfl_sync(kFull, slot, 0);
      if (slot < a.defer_capacity) {
        if (lane == 0) a.defer_list[slot] = tile;
#pragma unroll
        for (int v = 0; v < VPL; ++v)
          if (c.active[v]) M.dist[c.cell(v)] = best[v];  // the bounds pass B starts from
        continue;
      }
      // The list is full: finish the tile here, from the bounds found so far.
      walk<VPL, STACK, COUNT>(M.nodes, M.tris, M.bvh_nodes, M.bvh_tris, M.root, never, lim, lane, c.cx, c.cy, c.cz,
                              c.px, c.py, c.pz, best, ws);
    }
    store_cells<TX, TY, TZ>(a, c, best);
  }
  flush_stats<COUNT>(a, ws, lane);
}

// Pass B: one block per deferred tile; its warps share the tile's subtrees and bounds.
template <int TX, int TY, int TZ, int STACK, bool COUNT>
__global__ __launch_bounds__(kThreads) void k_distance_deferred(DistanceArgs a) {
  using Cells = TileCells<TX, TY, TZ>;
  constexpr int VPL = Cells::VPL;
  constexpr int kItems = 1 << kSplitBits;
  __shared__ unsigned long long s_tile;
  __shared__ int s_item;
  __shared__ uint32_t s_best[VPL * kWarp];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const BatchDev &B = a.batch;
  WalkStats ws;
  const unsigned long long count = a.defer_counters[0];
  const unsigned long long total = count < a.defer_capacity ? count : a.defer_capacity;

  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long k = atomicAdd(a.defer_counters + 1, 1ull);
      s_tile = k < total ? a.defer_list[k] : ~0ull;
      s_item = 0;
    }
    __syncthreads();
    const unsigned long long tile = s_tile;
    if (tile == ~0ull) break;
    Cells c;
    c.locate(B, tile, lane);
    const MeshRec &M = *c.M;
    float best[VPL];
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      best[v] = c.active[v] ? M.dist[c.cell(v)] : -1.0f;
      if (warp == 0) s_best[v * kWarp + lane] = __float_as_uint(c.active[v] ? best[v] : 0.0f);
    }
    __syncthreads();
    for (;;) {
      int item = 0;
      if (lane == 0) item = atomicAdd(&s_item, 1);
      item = __shfl_sync(kFull, item, 0);
      if (item >= kItems) break;
#pragma unroll
      for (int v = 0; v < VPL; ++v)
        if (c.active[v]) best[v] = fminf(best[v], __uint_as_float(s_best[v * kWarp + lane]));
      // Descend to this item's subtree: each node with two children consumes one bit of the item
      // (most significant first); a leaf reached early is tested by the item whose remaining bits
      // are all zero.
      int cur = M.root, bits = kSplitBits;
      bool walk_it = false;
      for (int guard = 0; guard < 64; ++guard) {
        if (bits == 0) {
          walk_it = true;
          break;
        }
        if (cur < 0 || cur >= M.bvh_nodes) {
          ws.corrupt = true;
          break;
        }
        const Node *np = M.nodes + cur;
        const float4 n0 = __ldg(&np->n0), n1 = __ldg(&np->n1), n2 = __ldg(&np->n2);
        const int4 n3 = __ldg(&np->n3);
        const bool e0 = n3.z < 0, e1 = n3.w < 0;
        if (e0 && e1) break;
        int which;
        if (!e0 && !e1) {
          --bits;
          which = (item >> bits) & 1;
        } else {
          which = e0 ? 1 : 0;
        }
        bool want = false;
#pragma unroll
        for (int v = 0; v < VPL; ++v) {
          const float d = which ? box_dist2(c.px, c.py, c.pz[v], n1.z, n1.w, n2.x, n2.y, n2.z, n2.w)
                                : box_dist2(c.px, c.py, c.pz[v], n0.x, n0.y, n0.z, n0.w, n1.x, n1.y);
          want |= d < best[v];
        }
        if (COUNT) ws.box_tests += kWarp * VPL;
        if (!__any_sync(kFull, want)) break;
        const int ref = which ? n3.y : n3.x, cnt = which ? n3.w : n3.z;
        if (cnt > 0) {
          if ((item & ((1 << bits) - 1)) == 0)
            test_leaf<VPL, COUNT>(M.tris, M.bvh_tris, ref, cnt, c.px, c.py, c.pz, best, ws);
          break;
        }
        cur = ref;
      }
      if (walk_it)
        walk<VPL, STACK, COUNT>(M.nodes, M.tris, M.bvh_nodes, M.bvh_tris, cur, TailCheck{nullptr, 0, 0},
                                walk_limits<STACK>(M.bvh_nodes, a.fault), lane, c.cx, c.cy, c.cz, c.px, c.py, c.pz,
                                best, ws);
#pragma unroll
      for (int v = 0; v < VPL; ++v)
        if (c.active[v]) atomicMin(&s_best[v * kWarp + lane], __float_as_uint(best[v]));
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
      for (int v = 0; v < VPL; ++v) best[v] = c.active[v] ? __uint_as_float(s_best[v * kWarp + lane]) : -1.0f;
      store_cells<TX, TY, TZ>(a, c, best);
    }
    __syncthreads();
  }
  flush_stats<COUNT>(a, ws, lane);
}

template <typename K>
int blocks_per_sm(K kernel, int threads) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  return per_sm > 0 ? per_sm : 1;
}

template <int I, int STACK, bool COUNT>
cudaError_t launch_shape(const DistanceArgs &a, int num_sms, cudaStream_t st) {
  constexpr Shape s = kShapes[I];
  static const int per_sm = blocks_per_sm(k_distance<s.tx, s.ty, s.tz, STACK, COUNT>, kThreadsA);
  static const int per_sm_b = blocks_per_sm(k_distance_deferred<s.tx, s.ty, s.tz, STACK, COUNT>, kThreads);
  const unsigned long long warps_needed = a.batch.total_tiles;
  unsigned long long blocks = static_cast<unsigned long long>(num_sms) * per_sm;
  blocks = std::min<unsigned long long>(blocks, (warps_needed + kWarpsPerBlockA - 1) / kWarpsPerBlockA);
  if (blocks < 1) blocks = 1;
  // kChunkMax tiles per chunk when there are plenty, fewer when the tiles would not reach every
  // warp several times over. Pass A uses no shared memory to speak of: all of it goes to L1.
  static const bool carveout = cudaFuncSetAttribute(k_distance<s.tx, s.ty, s.tz, STACK, COUNT>,
                                                    cudaFuncAttributePreferredSharedMemoryCarveout,
                                                    cudaSharedmemCarveoutMaxL1) == cudaSuccess;
  (void)carveout;
  DistanceArgs ca = a;
  ca.chunk_tiles = std::max<unsigned long long>(
      1, std::min<unsigned long long>(kChunkMax, a.batch.total_tiles / (blocks * kWarpsPerBlockA * 4)));
  cudaError_t e = cudaMemsetAsync(a.tile_counter, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess && a.defer_list) e = cudaMemsetAsync(a.defer_counters, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_distance<s.tx, s.ty, s.tz, STACK, COUNT><<<static_cast<unsigned>(blocks), kThreadsA, 0, st>>>(ca);
  note_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess || !a.defer_list || a.step_budget <= 0) return e;
  // Pass B: a persistent grid; the number of deferred tiles is read on the device.
  const unsigned long long blocks_b =
      std::min<unsigned long long>(static_cast<unsigned long long>(num_sms) * per_sm_b, a.defer_capacity);
  k_distance_deferred<s.tx, s.ty, s.tz, STACK, COUNT>
      <<<static_cast<unsigned>(std::max<unsigned long long>(blocks_b, 1)), kThreads, 0, st>>>(a);
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

double distance_work_flops(int tile_id, const unsigned long long *w) {
  int tx, ty, tz;
  tile_shape(tile_id, tx, ty, tz);
  const int vpl = tz / (kWarp / (tx * ty));
  return distance_flops(vpl, double(w[0]), double(w[3]), double(w[4]), double(w[1]));
}

void tile_shape(int id, int &tx, int &ty, int &tz) {
  const Shape s = kShapes[(id < 0 || id >= kNumShapes) ? 0 : id];
  tx = s.tx;
  ty = s.ty;
  tz = s.tz;
}

uint64_t tiles_for(const GridDev &g, int id) {
  int tx, ty, tz;
  tile_shape(id, tx, ty, tz);
  const uint64_t bx = ((g.nx + tx - 1) / tx + kBrickX - 1) / kBrickX;
  const uint64_t by = ((g.ny + ty - 1) / ty + kBrickY - 1) / kBrickY;
  const uint64_t bz = ((g.nz + tz - 1) / tz + kBrickZ - 1) / kBrickZ;
  return bx * by * bz * kBrickTiles;
}

uint64_t defer_capacity_for(uint64_t total_tiles) {
  return std::min<uint64_t>(total_tiles, std::max<uint64_t>(4096, total_tiles / 8));
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
