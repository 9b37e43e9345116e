// Host mesh utilities (weld, watertight gate); see host_mesh.cpp.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace sdfb {

float weld_cell(const float bmin[3], const float bmax[3]);
// Returns the number of unique positions; welded receives one index per position.
uint32_t weld_positions(const float *pos, size_t n, const float bmin[3], const float bmax[3], uint32_t *welded);
// 1 watertight, 0 not, -1 empty. tri holds 3 welded indices per triangle.
int watertight_flag(const uint32_t *tri, size_t ntris, uint64_t *boundary, uint64_t *nonmanifold);
// Watertight gate of an indexed mesh (weld of its vertices, then the edge test over the welded
// triangles, equivalent to the reference's test on the de-indexed soup). -2: index out of range.
int indexed_mesh_watertight(const float *verts, uint32_t V, const uint32_t *idx, uint32_t T);

// srgbToLinear (src/convert/sdf_baker.cpp:42, voxelize.cpp:12) of every 8-bit channel value
// b / 255.0f, evaluated on the host as the reference does (so the device reads the same bits).
void srgb_to_linear_table(float out[256]);

}  // namespace sdfb
