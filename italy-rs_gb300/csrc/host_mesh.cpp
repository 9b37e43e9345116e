// Host mesh utilities: the reference's weld and watertight gate, used to pick the sign mode.
//
// weld_positions follows weldPositions (src/io/mesh_weld.cpp:26-48): lattice cell
// max(|extent| * 1e-5, 1e-6) in FP32 (|extent| as glm::length, ((x*x + y*y) + z*z)), keys
// lround(p / cell) per axis, indices numbered by first occurrence. watertight follows
// isWatertight (src/io/mesh_validate.cpp:21-59): degenerate welded triangles are skipped, an edge
// used once is a boundary edge, more than twice non-manifold. Both use open-addressing hash
// tables, so they run in O(n).
#include "host_mesh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

namespace sdfb {
namespace {

inline uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

size_t table_size(size_t n) {
  size_t cap = 16;
  while (cap < 2 * n + 16) cap <<= 1;
  return cap;
}

}  // namespace

float weld_cell(const float bmin[3], const float bmax[3]) {
  const float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  const float diag = std::sqrt(ex * ex + ey * ey + ez * ez);
  const float cell = diag * 1e-5f;
  return cell < 1e-6f ? 1e-6f : cell;
}

uint32_t weld_positions(const float *pos, size_t n, const float bmin[3], const float bmax[3], uint32_t *welded) {
  const float cell = weld_cell(bmin, bmax);
  const size_t cap = table_size(n);
  std::vector<int64_t> keys(cap * 3);
  std::vector<uint32_t> vals(cap, 0xffffffffu);
  uint32_t next = 0;
  for (size_t i = 0; i < n; ++i) {
    const int64_t k[3] = {static_cast<int64_t>(std::lround(pos[3 * i] / cell)),
                          static_cast<int64_t>(std::lround(pos[3 * i + 1] / cell)),
                          static_cast<int64_t>(std::lround(pos[3 * i + 2] / cell))};
    uint64_t h = mix64(mix64(mix64(static_cast<uint64_t>(k[0])) ^ static_cast<uint64_t>(k[1])) ^
                       static_cast<uint64_t>(k[2]));
    size_t s = h & (cap - 1);
    for (;;) {
      if (vals[s] == 0xffffffffu) {
        keys[3 * s] = k[0];
        keys[3 * s + 1] = k[1];
        keys[3 * s + 2] = k[2];
        vals[s] = next++;
        break;
      }
      if (keys[3 * s] == k[0] && keys[3 * s + 1] == k[1] && keys[3 * s + 2] == k[2]) break;
      s = (s + 1) & (cap - 1);
    }
    welded[i] = vals[s];
  }
  return next;
}

int watertight_flag(const uint32_t *tri, size_t ntris, uint64_t *boundary, uint64_t *nonmanifold) {
  *boundary = 0;
  *nonmanifold = 0;
  if (ntris == 0) return -1;
  const size_t cap = table_size(3 * ntris);
  std::vector<uint64_t> keys(cap, ~0ull);
  std::vector<uint32_t> count(cap, 0);
  for (size_t t = 0; t < ntris; ++t) {
    const uint32_t a = tri[3 * t], b = tri[3 * t + 1], c = tri[3 * t + 2];
    if (a == b || b == c || c == a) continue;
    const uint32_t e[3][2] = {{a, b}, {b, c}, {c, a}};
    for (int k = 0; k < 3; ++k) {
      const uint32_t u = e[k][0] < e[k][1] ? e[k][0] : e[k][1];
      const uint32_t v = e[k][0] < e[k][1] ? e[k][1] : e[k][0];
      const uint64_t key = (static_cast<uint64_t>(u) << 32) | v;
      size_t s = mix64(key) & (cap - 1);
      while (keys[s] != ~0ull && keys[s] != key) s = (s + 1) & (cap - 1);
      keys[s] = key;
      count[s]++;
    }
  }
  for (size_t s = 0; s < cap; ++s) {
    if (keys[s] == ~0ull) continue;
    if (count[s] == 1) ++*boundary;
    else if (count[s] > 2) ++*nonmanifold;
  }
  return (*boundary == 0 && *nonmanifold == 0) ? 1 : 0;
}

int indexed_mesh_watertight(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T) {
  if (T == 0 || V == 0) return -1;
  float bmin[3] = {verts[0], verts[1], verts[2]}, bmax[3] = {verts[0], verts[1], verts[2]};
  for (uint32_t i = 1; i < V; ++i)
    for (int a = 0; a < 3; ++a) {
      const float v = verts[3 * size_t(i) + a];
      bmin[a] = v < bmin[a] ? v : bmin[a];
      bmax[a] = v > bmax[a] ? v : bmax[a];
    }
  std::vector<uint32_t> w(V);
  weld_positions(verts, V, bmin, bmax, w.data());
  std::vector<uint32_t> tri(3 * size_t(T));
  for (size_t k = 0; k < 3 * size_t(T); ++k) {
    const uint32_t i = idx[k];
    if (i >= V) return -2;
    tri[k] = w[i];
  }
  uint64_t b, m;
  return watertight_flag(tri.data(), T, &b, &m);
}

void srgb_to_linear_table(float out[256]) {
  for (int b = 0; b < 256; ++b) {
    const float c = static_cast<float>(b) / 255.0f;
    out[b] = c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f);
  }
}

}  // namespace sdfb
