// Exact +z ray parity for watertight meshes (the reference's first parity ray is +z,
// src/render/kernels/sdf_bake.cu:53-69; there it is stepped with a 1e-4 epsilon and voted over 5
// rays, here it is one exact ray per column).
//
// Every cell of a column (x, y) shares the line through the column's FP32 centre, so the bake
// finds, once per column, the heights at which that line crosses the mesh; a cell is inside when
// an odd number of crossings lie above its centre. Whether the line crosses a triangle is decided
// with exact orientation predicates and simulation of simplicity (common.cuh), so a line through
// a shared edge or vertex is counted exactly once and the parity is exact for every column.
//
//   k_col_items   candidate columns per triangle (centres inside its xy bounds, with slack)
//   scan          item starts
//   k_col_hits<0> exact test per (triangle, column) item; counts crossings per column (atomics)
//   scan          column starts
//   k_col_hits<1> same test; writes each crossing height into its column's slot range
// The order of heights inside a column is irrelevant: the distance kernel only counts those
// above each cell.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "expand.cuh"
#include "kernels.h"

namespace sdfb {
namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct TriCols {
  f3 a, b, c;
  int x0, x1, y0, y1;
  int mesh;
};

__device__ __forceinline__ f3 vload(const float *v, uint32_t i) {
  return {__ldg(v + 3ull * i), __ldg(v + 3ull * i + 1), __ldg(v + 3ull * i + 2)};
}

// Column index range [lo, hi] whose centres o + (i + 0.5) v may fall inside [mn, mx], widened by
// a margin far above the FP32 error of the index arithmetic.
__device__ __forceinline__ void col_range(float mn, float mx, float o, float v, int n, int &lo, int &hi) {
  const float a = (mn - o) / v - 0.5f, b = (mx - o) / v - 0.5f;
  const float eps = 0.01f + 2e-6f * fmaxf(fabsf(a), fabsf(b));
  const float fa = ceilf(a - eps), fb = floorf(b + eps);
  lo = fa < 0.0f ? 0 : (fa > float(n - 1) ? n : static_cast<int>(fa));
  hi = fb < 0.0f ? -1 : (fb > float(n - 1) ? n - 1 : static_cast<int>(fb));
}

// Parity triangle t (global over the parity meshes) and its candidate columns.
__device__ __forceinline__ TriCols tri_cols(const BatchDev &B, uint64_t t) {
  TriCols r;
  r.mesh = find_mesh(B.ptri_starts, B.num_meshes, t);
  const MeshRec &M = B.recs[r.mesh];
  const uint64_t lt = t - B.ptri_starts[r.mesh];
  const uint32_t V = M.pnum_verts;
  const uint32_t i0 = __ldg(M.pidx + 3 * lt), i1 = __ldg(M.pidx + 3 * lt + 1), i2 = __ldg(M.pidx + 3 * lt + 2);
  r.a = vload(M.pverts, i0 < V ? i0 : 0);
  r.b = vload(M.pverts, i1 < V ? i1 : 0);
  r.c = vload(M.pverts, i2 < V ? i2 : 0);
  const bool ok = isfinite(r.a.x + r.a.y + r.b.x + r.b.y + r.c.x + r.c.y + r.a.z + r.b.z + r.c.z);
  const GridDev &g = M.g;
  col_range(fminf(fminf(r.a.x, r.b.x), r.c.x), fmaxf(fmaxf(r.a.x, r.b.x), r.c.x), g.ox, g.voxel, g.nx, r.x0, r.x1);
  col_range(fminf(fminf(r.a.y, r.b.y), r.c.y), fmaxf(fmaxf(r.a.y, r.b.y), r.c.y), g.oy, g.voxel, g.ny, r.y0, r.y1);
  if (!ok || r.x1 < r.x0 || r.y1 < r.y0) {
    r.x0 = r.y0 = 0;
    r.x1 = r.y1 = -1;
  }
  return r;
}

// Candidate columns per triangle, as 64-bit counts (a triangle across a wide, flat grid can cover
// more than 2^32 columns).
__global__ __launch_bounds__(kThreads) void k_col_items(BatchDev B, uint64_t *__restrict__ items) {
  const uint64_t t = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
  if (t >= B.total_ptris) return;
  const TriCols tc = tri_cols(B, t);
  items[t] = tc.x1 < tc.x0 ? 0ull : uint64_t(tc.x1 - tc.x0 + 1) * uint64_t(tc.y1 - tc.y0 + 1);
}

template <bool FILL>
__global__ __launch_bounds__(kThreads) void k_col_hits(BatchDev B, const uint64_t *__restrict__ starts,
                                                       uint32_t *__restrict__ col_count,
                                                       const uint64_t *__restrict__ col_start,
                                                       float *__restrict__ col_z, int8_t *__restrict__ col_s,
                                                       uint64_t capacity, uint32_t *__restrict__ err) {
  const uint64_t T = B.total_ptris;
  const uint64_t total = starts[T];
  const uint64_t stride = uint64_t(gridDim.x) * kThreads * kExpandChunk;
  for (uint64_t w0 = (uint64_t(blockIdx.x) * kThreads + threadIdx.x) * kExpandChunk; w0 < total; w0 += stride) {
    uint64_t t = item_owner(starts, static_cast<uint32_t>(T), w0);
    TriCols tc = tri_cols(B, t);
    uint64_t tstart = starts[t], tend = starts[t + 1];
    const uint64_t wend = min(w0 + kExpandChunk, total);
    for (uint64_t w = w0; w < wend; ++w) {
      while (w >= tend) {
        ++t;
        tstart = tend;
        tend = starts[t + 1];
        if (tend > tstart) tc = tri_cols(B, t);
      }
      const MeshRec &M = B.recs[tc.mesh];
      const GridDev &g = M.g;
      const uint64_t k = w - tstart;
      const uint32_t sx = tc.x1 - tc.x0 + 1;
      const int x = tc.x0 + static_cast<int>(k % sx);
      const int y = tc.y0 + static_cast<int>(k / sx);
      const float px = cell_center(g.ox, x, g.voxel), py = cell_center(g.oy, y, g.voxel);
      float z;
      int sgn;
      if (!column_crossing(tc.a, tc.b, tc.c, px, py, z, sgn)) continue;
      const uint64_t col = M.col_base + uint64_t(y) * g.nx + x;
      const uint32_t slot = atomicAdd(col_count + col, 1u);
      if (FILL) {
        const uint64_t at = col_start[col] + slot;
        if (at < capacity) {
          col_z[at] = z;
          col_s[at] = static_cast<int8_t>(sgn);
        } else {
          atomic_or_err(err, kErrCrossingOverflow);
        }
      }
    }
  }
}

struct ParTemp {
  uint64_t *items;
  uint64_t *starts;
  uint32_t *col_count;
  void *scratch;
  size_t scratch_bytes;
};

size_t par_layout(uint64_t T, uint64_t ncols, char *base, ParTemp *o) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  ParTemp x;
  x.items = reinterpret_cast<uint64_t *>(take(size_t(T) * 8 + 8));
  x.starts = reinterpret_cast<uint64_t *>(take((size_t(T) + 1) * 8));
  x.col_count = reinterpret_cast<uint32_t *>(take(ncols * 4 + 4));
  x.scratch_bytes = std::max(scan_scratch_bytes(T), scan_scratch_bytes(ncols));
  x.scratch = take(x.scratch_bytes);
  if (o) *o = x;
  return off;
}

}  // namespace

size_t parity_temp_bytes(uint64_t total_ptris, uint64_t total_cols) {
  return par_layout(total_ptris, total_cols, nullptr, nullptr);
}

cudaError_t parity_columns(const BatchDev &B, uint64_t *col_start, float *col_z, int8_t *col_s, uint64_t capacity,
                           void *temp, size_t temp_bytes, uint32_t *err, int num_sms, cudaStream_t st) {
  const uint64_t T = B.total_ptris, ncols = B.total_cols;
  ParTemp o;
  if (par_layout(T, ncols, static_cast<char *>(temp), &o) > temp_bytes) return cudaErrorMemoryAllocation;
  cudaError_t e;
  if ((e = cudaMemsetAsync(o.col_count, 0, ncols * 4, st)) != cudaSuccess) return e;
  if (T == 0) return cudaMemsetAsync(col_start, 0, (ncols + 1) * 8, st);
  const Scratch sc{o.scratch, o.scratch_bytes};
  k_col_items<<<static_cast<unsigned>((T + kThreads - 1) / kThreads), kThreads, 0, st>>>(B, o.items);
  note_launch();
  if ((e = exclusive_scan_u64(o.items, o.starts, T, sc, st)) != cudaSuccess) return e;
  const unsigned grid = num_sms * 8;
  k_col_hits<false><<<grid, kThreads, 0, st>>>(B, o.starts, o.col_count, nullptr, nullptr, nullptr, 0, err);
  note_launch();
  if ((e = exclusive_scan_u32(o.col_count, col_start, ncols, sc, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(o.col_count, 0, ncols * 4, st)) != cudaSuccess) return e;
  k_col_hits<true><<<grid, kThreads, 0, st>>>(B, o.starts, o.col_count, col_start, col_z, col_s, capacity, err);
  note_launch();
  return cudaGetLastError();
}

}  // namespace sdfb
