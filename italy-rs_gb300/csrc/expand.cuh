// Load-balanced expansion of per-triangle work: triangle t owns the items
// [starts[t], starts[t + 1]) of an exclusive scan of its item counts. Threads take chunks of
// consecutive items, find the owner of the first by binary search and walk forward.
#pragma once

#include <cstdint>

namespace sdfb {

constexpr int kExpandChunk = 4;

// Largest t in [0, n) with starts[t] <= w (starts[0] = 0).
__device__ __forceinline__ uint32_t item_owner(const uint64_t *__restrict__ starts, uint32_t n, uint64_t w) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(starts + mid) <= w) lo = mid;
    else hi = mid;
  }
  return lo;
}

}  // namespace sdfb
