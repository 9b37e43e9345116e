// Test infrastructure only. A thin C driver around the reference's own CPU code for the bake
// path, compiled from the reference's sources (see oracle/build_oracle.py) into
// oracle/_ref/libitaly_ref.so. It exists so the oracle's restatement and the golden fixtures can
// be checked against the reference itself:
//   * ref_occupancy_dense restates the candidate-cell loop of bakePerCellMaterial
//     (src/convert/sdf_baker.cpp:89-118; that function sits in the OptiX translation unit, which
//     cannot be built here) around the reference's own italy::triBoxOverlap
//     (src/convert/tri_box_overlap.h:72-114). Occupancy = count > 0 (sdf_baker.cpp:115,121-122).
//   * ref_grid_from_bounds restates the grid sizing of bakeSdf (sdf_baker.cpp:138-148) in the
//     same glm operation order.
//   * ref_voxelize calls italy::voxelizeMesh (src/convert/voxelize.cpp:52-107) unchanged;
//     ref_voxelize_colors does too and also returns its per-cell colours (textures, uvs and
//     per-triangle materials included).
//   * ref_materials_dense restates the material averaging of bakePerCellMaterial
//     (sdf_baker.cpp:76-128) with its triangleMaterial / sampleColorNearest / srgbToLinear
//     (sdf_baker.cpp:42-74), in the reference's glm operation order.
//   * ref_weld / ref_is_watertight call italy::weldPositions (src/io/mesh_weld.cpp:26-48) and
//     italy::isWatertight (src/io/mesh_validate.cpp:21-59) unchanged.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "convert/tri_box_overlap.h"
#include "convert/voxelize.h"
#include "io/mesh_validate.h"
#include "io/mesh_weld.h"

namespace {

std::vector<glm::vec3> toVec3(const float *xyz, int64_t n) {
  std::vector<glm::vec3> out(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i)
    out[static_cast<size_t>(i)] = glm::vec3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  return out;
}

italy::MeshAsset soupMesh(const float *soup, int64_t tris, const float *bmin, const float *bmax) {
  italy::MeshAsset mesh;
  mesh.positions = toVec3(soup, 3 * tris);
  mesh.boundsMin = glm::vec3(bmin[0], bmin[1], bmin[2]);
  mesh.boundsMax = glm::vec3(bmax[0], bmax[1], bmax[2]);
  mesh.materials.push_back(italy::MaterialAsset{});
  return mesh;
}

// The material inputs in flat arrays: 5 floats per material (base colour r, g, b, metallic,
// roughness) and its base colour texture; per-triangle material indices; 2 floats per uv; every
// texture's RGBA8 texels concatenated, with offsets, sizes and sRGB flags.
struct FlatMaterials {
  const float *mat_f;
  const int32_t *mat_tex;
  int64_t nmat;
  const uint32_t *tri_mat;
  int64_t ntri_mat;
  const float *uvs;
  int64_t nuv;
  const uint8_t *pixels;
  const int64_t *tex_off;
  const int32_t *tex_w, *tex_h, *tex_srgb;
  int64_t ntex;
};

void addMaterials(italy::MeshAsset &mesh, const FlatMaterials &f) {
  mesh.materials.clear();
  for (int64_t i = 0; i < f.nmat; ++i) {
    italy::MaterialAsset m;
    m.baseColorFactor = glm::vec3(f.mat_f[5 * i], f.mat_f[5 * i + 1], f.mat_f[5 * i + 2]);
    m.metallic = f.mat_f[5 * i + 3];
    m.roughness = f.mat_f[5 * i + 4];
    m.baseColorTexture = f.mat_tex[i];
    mesh.materials.push_back(m);
  }
  mesh.triangleMaterial.assign(f.tri_mat, f.tri_mat + f.ntri_mat);
  mesh.uvs.resize(static_cast<size_t>(f.nuv));
  for (int64_t i = 0; i < f.nuv; ++i) mesh.uvs[static_cast<size_t>(i)] = glm::vec2(f.uvs[2 * i], f.uvs[2 * i + 1]);
  for (int64_t k = 0; k < f.ntex; ++k) {
    italy::TextureAsset t;
    t.width = f.tex_w[k];
    t.height = f.tex_h[k];
    t.srgb = f.tex_srgb[k] != 0;
    const size_t bytes = static_cast<size_t>(t.width) * static_cast<size_t>(t.height) * 4;
    t.pixelsRGBA.assign(f.pixels + f.tex_off[k], f.pixels + f.tex_off[k] + bytes);
    mesh.textures.push_back(std::move(t));
  }
}

// sdf_baker.cpp:42-74, restated (that translation unit needs OptiX).
float srgbToLinearR(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }

glm::vec3 sampleColorNearestR(const italy::TextureAsset &tex, glm::vec2 uv) {
  auto wrap = [](float x) { return x - std::floor(x); };
  const int px = std::clamp(static_cast<int>(wrap(uv.x) * tex.width), 0, tex.width - 1);
  const int py = std::clamp(static_cast<int>(wrap(uv.y) * tex.height), 0, tex.height - 1);
  const size_t idx = (static_cast<size_t>(py) * tex.width + px) * 4;
  const glm::vec3 raw(tex.pixelsRGBA[idx] / 255.0f, tex.pixelsRGBA[idx + 1] / 255.0f,
                      tex.pixelsRGBA[idx + 2] / 255.0f);
  if (!tex.srgb) return raw;
  return glm::vec3(srgbToLinearR(raw.r), srgbToLinearR(raw.g), srgbToLinearR(raw.b));
}

struct CellMaterialR {
  glm::vec3 baseColor;
  float metallic;
  float roughness;
};

CellMaterialR triangleMaterialR(const italy::MeshAsset &mesh, size_t triangle) {
  const italy::MaterialAsset &mat = mesh.materialForTriangle(triangle);
  glm::vec3 color = mat.baseColorFactor;
  const size_t base = triangle * 3;
  if (mat.baseColorTexture >= 0 && mat.baseColorTexture < static_cast<int>(mesh.textures.size()) &&
      base + 2 < mesh.uvs.size()) {
    const italy::TextureAsset &tex = mesh.textures[mat.baseColorTexture];
    if (tex.width > 0 && tex.height > 0) {
      const glm::vec2 uv = (mesh.uvs[base] + mesh.uvs[base + 1] + mesh.uvs[base + 2]) / 3.0f;
      color = sampleColorNearestR(tex, uv) * mat.baseColorFactor;
    }
  }
  return CellMaterialR{color, mat.metallic, mat.roughness};
}

} // namespace

extern "C" {

void ref_grid_from_bounds(const float *bmin, const float *bmax, int32_t resolution, float *origin_out,
                          float *voxel_out, int32_t *n_out) {
  const glm::vec3 lo(bmin[0], bmin[1], bmin[2]), hi(bmax[0], bmax[1], bmax[2]);
  const glm::vec3 extent = hi - lo;
  const float longestAxis = std::max({extent.x, extent.y, extent.z, 1e-6f});
  const float voxel = longestAxis / static_cast<float>(std::max(resolution, 1));
  constexpr int kPad = 2;
  const glm::vec3 origin = lo - glm::vec3(voxel * kPad);
  const glm::vec3 padded = extent + glm::vec3(voxel * kPad * 2.0f);
  origin_out[0] = origin.x;
  origin_out[1] = origin.y;
  origin_out[2] = origin.z;
  *voxel_out = voxel;
  n_out[0] = static_cast<int>(std::ceil(padded.x / voxel)) + 1;
  n_out[1] = static_cast<int>(std::ceil(padded.y / voxel)) + 1;
  n_out[2] = static_cast<int>(std::ceil(padded.z / voxel)) + 1;
}

// Dense occupancy over an explicit grid; `soup` holds 9 floats per triangle.
void ref_occupancy_dense(const float *soup, int64_t tris, const float *origin3, float voxel, int32_t nx, int32_t ny,
                         int32_t nz, uint8_t *occ) {
  const size_t cells = static_cast<size_t>(nx) * ny * nz;
  std::memset(occ, 0, cells);
  const glm::vec3 origin(origin3[0], origin3[1], origin3[2]);
  for (int64_t t = 0; t < tris; ++t) {
    const float *s = soup + 9 * t;
    const glm::vec3 p0(s[0], s[1], s[2]), p1(s[3], s[4], s[5]), p2(s[6], s[7], s[8]);
    const glm::vec3 triMin = glm::min(glm::min(p0, p1), p2);
    const glm::vec3 triMax = glm::max(glm::max(p0, p1), p2);
    const glm::ivec3 res(nx - 1, ny - 1, nz - 1);
    const glm::ivec3 cellMin = glm::clamp(glm::ivec3(glm::floor((triMin - origin) / voxel)), glm::ivec3(0), res);
    const glm::ivec3 cellMax = glm::clamp(glm::ivec3(glm::floor((triMax - origin) / voxel)), glm::ivec3(0), res);
    for (int z = cellMin.z; z <= cellMax.z; ++z)
      for (int y = cellMin.y; y <= cellMax.y; ++y)
        for (int x = cellMin.x; x <= cellMax.x; ++x) {
          const glm::vec3 center = origin + (glm::vec3(x, y, z) + 0.5f) * voxel;
          const glm::vec3 half(voxel * 0.5f);
          if (italy::triBoxOverlap(center, half, p0, p1, p2))
            occ[(static_cast<size_t>(z) * ny + y) * nx + x] = 1;
        }
  }
}

// Sparse voxelization through the reference's own voxelizeMesh. Returns the number of cells; at
// most `cap` cells (ivec3, in the reference's insertion order) are written to `cells_out`.
int64_t ref_voxelize(const float *soup, int64_t tris, const float *bmin, const float *bmax, int32_t resolution,
                     int32_t *cells_out, int64_t cap, float *origin_out, float *voxel_out) {
  const italy::MeshAsset mesh = soupMesh(soup, tris, bmin, bmax);
  const italy::VoxelGrid grid = italy::voxelizeMesh(mesh, resolution);
  const int64_t n = static_cast<int64_t>(grid.cells.size());
  for (int64_t i = 0; i < n && i < cap; ++i) {
    cells_out[3 * i] = grid.cells[i].x;
    cells_out[3 * i + 1] = grid.cells[i].y;
    cells_out[3 * i + 2] = grid.cells[i].z;
  }
  origin_out[0] = grid.origin.x;
  origin_out[1] = grid.origin.y;
  origin_out[2] = grid.origin.z;
  *voxel_out = grid.voxelSize;
  return n;
}

// Returns the number of unique welded vertices; welded_out receives one index per position.
int64_t ref_weld(const float *positions, int64_t n, const float *bmin, const float *bmax, uint32_t *welded_out) {
  const std::vector<glm::vec3> pos = toVec3(positions, n);
  const std::vector<uint32_t> w =
      italy::weldPositions(pos, glm::vec3(bmin[0], bmin[1], bmin[2]), glm::vec3(bmax[0], bmax[1], bmax[2]));
  std::copy(w.begin(), w.end(), welded_out);
  return static_cast<int64_t>(italy::weldedIndexCount(w));
}

// 1 = watertight, 0 = not; the reference's message is copied into err (NUL-terminated).
int32_t ref_is_watertight(const float *soup, int64_t tris, const float *bmin, const float *bmax, char *err,
                          int32_t err_cap) {
  const italy::MeshAsset mesh = soupMesh(soup, tris, bmin, bmax);
  std::string msg;
  const bool ok = italy::isWatertight(mesh, msg);
  if (err && err_cap > 0) {
    const size_t n = std::min(msg.size(), static_cast<size_t>(err_cap - 1));
    std::memcpy(err, msg.data(), n);
    err[n] = '\0';
  }
  return ok ? 1 : 0;
}

} // extern "C"

extern "C" {

// voxelizeMesh with materials: returns the cell count; writes min(count, cap) cells and colours.
int64_t ref_voxelize_colors(const float *soup, int64_t tris, const float *bmin, const float *bmax, int32_t resolution,
                            const float *mat_f, const int32_t *mat_tex, int64_t nmat, const uint32_t *tri_mat,
                            int64_t ntri_mat, const float *uvs, int64_t nuv, const uint8_t *pixels,
                            const int64_t *tex_off, const int32_t *tex_w, const int32_t *tex_h,
                            const int32_t *tex_srgb, int64_t ntex, int32_t *cells_out, float *colors_out,
                            int64_t cap) {
  italy::MeshAsset mesh = soupMesh(soup, tris, bmin, bmax);
  addMaterials(mesh, FlatMaterials{mat_f, mat_tex, nmat, tri_mat, ntri_mat, uvs, nuv, pixels, tex_off, tex_w, tex_h,
                                   tex_srgb, ntex});
  const italy::VoxelGrid grid = italy::voxelizeMesh(mesh, resolution);
  const int64_t n = static_cast<int64_t>(grid.cells.size());
  for (int64_t i = 0; i < n && i < cap; ++i) {
    cells_out[3 * i] = grid.cells[i].x;
    cells_out[3 * i + 1] = grid.cells[i].y;
    cells_out[3 * i + 2] = grid.cells[i].z;
    colors_out[3 * i] = grid.colors[i].x;
    colors_out[3 * i + 1] = grid.colors[i].y;
    colors_out[3 * i + 2] = grid.colors[i].z;
  }
  return n;
}

// bakePerCellMaterial (sdf_baker.cpp:76-128) over an explicit grid; color_out holds 3 floats per cell.
void ref_materials_dense(const float *soup, int64_t tris, const float *origin3, float voxel, int32_t nx, int32_t ny,
                         int32_t nz, const float *mat_f, const int32_t *mat_tex, int64_t nmat,
                         const uint32_t *tri_mat, int64_t ntri_mat, const float *uvs, int64_t nuv,
                         const uint8_t *pixels, const int64_t *tex_off, const int32_t *tex_w, const int32_t *tex_h,
                         const int32_t *tex_srgb, int64_t ntex, float *color_out, float *metal_out,
                         float *rough_out) {
  const float zero[3] = {0.0f, 0.0f, 0.0f};
  italy::MeshAsset mesh = soupMesh(soup, tris, zero, zero);
  addMaterials(mesh, FlatMaterials{mat_f, mat_tex, nmat, tri_mat, ntri_mat, uvs, nuv, pixels, tex_off, tex_w, tex_h,
                                   tex_srgb, ntex});
  const size_t numCells = static_cast<size_t>(nx) * ny * nz;
  const glm::vec3 origin(origin3[0], origin3[1], origin3[2]);
  std::vector<glm::vec3> colorSum(numCells, glm::vec3(0.0f));
  std::vector<float> metallicSum(numCells, 0.0f), roughnessSum(numCells, 0.0f);
  std::vector<int> count(numCells, 0);
  for (int64_t t = 0; t < tris; ++t) {
    const size_t base = static_cast<size_t>(t) * 3;
    const glm::vec3 &p0 = mesh.positions[base];
    const glm::vec3 &p1 = mesh.positions[base + 1];
    const glm::vec3 &p2 = mesh.positions[base + 2];
    const glm::vec3 triMin = glm::min(glm::min(p0, p1), p2);
    const glm::vec3 triMax = glm::max(glm::max(p0, p1), p2);
    const glm::ivec3 res(nx - 1, ny - 1, nz - 1);
    const glm::ivec3 cellMin = glm::clamp(glm::ivec3(glm::floor((triMin - origin) / voxel)), glm::ivec3(0), res);
    const glm::ivec3 cellMax = glm::clamp(glm::ivec3(glm::floor((triMax - origin) / voxel)), glm::ivec3(0), res);
    const CellMaterialR mat = triangleMaterialR(mesh, static_cast<size_t>(t));
    for (int z = cellMin.z; z <= cellMax.z; ++z)
      for (int y = cellMin.y; y <= cellMax.y; ++y)
        for (int x = cellMin.x; x <= cellMax.x; ++x) {
          const glm::vec3 center = origin + (glm::vec3(x, y, z) + 0.5f) * voxel;
          const glm::vec3 half(voxel * 0.5f);
          if (!italy::triBoxOverlap(center, half, p0, p1, p2)) continue;
          const size_t idx = (static_cast<size_t>(z) * ny + y) * nx + x;
          colorSum[idx] += mat.baseColor;
          metallicSum[idx] += mat.metallic;
          roughnessSum[idx] += mat.roughness;
          count[idx] += 1;
        }
  }
  for (size_t i = 0; i < numCells; ++i) {
    glm::vec3 c(1.0f);
    float m = 0.0f, r = 1.0f;
    if (count[i] != 0) {
      c = colorSum[i] / static_cast<float>(count[i]);
      m = metallicSum[i] / static_cast<float>(count[i]);
      r = roughnessSum[i] / static_cast<float>(count[i]);
    }
    color_out[3 * i] = c.x;
    color_out[3 * i + 1] = c.y;
    color_out[3 * i + 2] = c.z;
    metal_out[i] = m;
    rough_out[i] = r;
  }
}

}  // extern "C"
