/*
 * sdfb.h -- C ABI of the GB300 mesh -> signed-distance-field bake.
 *
 * This is the drop-in boundary for the reference's bake path. Every entry point takes plain
 * pointers and sizes, returns an sdfb_status, and never throws across the ABI. The reference
 * interface each one replaces is cited beside it (paths inside the reference project).
 *
 * Conventions
 *   - Grids are dense, x-fastest: cell (x, y, z) is at (z * ny + y) * nx + x
 *     (src/convert/sdf_grid.h:35). The sample point of a cell is its FP32 centre
 *     origin + (float(i) + 0.5f) * voxel_size per axis (src/render/kernels/sdf_bake.cu:34-37,
 *     src/convert/sdf_baker.cpp:107).
 *   - Distances are FP32, negative inside (sdf_bake.cu:69-72). Occupancy is uint8 0/1: a cell is
 *     occupied when a triangle whose clamped cell range contains it passes the triangle/box
 *     separating-axis test (sdf_baker.cpp:89-118, tri_box_overlap.h:72-114).
 *   - Meshes are indexed: verts is V x 3 FP32, idx is T x 3 uint32. The soup entry point takes the
 *     reference's MeshAsset layout (3 positions per triangle, src/io/mesh_asset.h:33-46).
 *   - A context owns one device, its streams, device memory and the resident mesh cache. Use one
 *     context from one host thread at a time; separate contexts are independent.
 *   - On an error the entry point returns a non-zero status and sdfb_last_error(ctx) describes it
 *     (the reference throws std::runtime_error from OPTIX_CHECK / CUDA_CHECK,
 *     src/render/optix_check.h:13-52).
 */
#ifndef SDFB_H
#define SDFB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDFB_ABI_VERSION 1

typedef enum sdfb_status {
  SDFB_OK = 0,
  SDFB_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad grid */
  SDFB_ERR_OUT_OF_MEMORY = 2,    /* device or pinned host allocation failed, or over a budget */
  SDFB_ERR_CUDA = 3,             /* a CUDA runtime call failed (message in sdfb_last_error) */
  SDFB_ERR_BAD_MESH = 4,         /* triangle index >= V, or a non-finite vertex */
  SDFB_ERR_OVERFLOW = 5,         /* a bounded device structure overflowed (traversal stack) */
  SDFB_ERR_BUSY = 6,             /* serving: no slot or memory free right now */
  SDFB_ERR_TIMEOUT = 7,          /* serving: a wait ran out */
  SDFB_ERR_NOT_FOUND = 8,        /* serving: unknown mesh or request id */
  SDFB_ERR_NO_DEVICE = 9,        /* no CUDA device, or the device is not sm_103 */
  SDFB_ERR_INTERNAL = 10
} sdfb_status;

/* Sign modes. AUTO welds the mesh (src/io/mesh_weld.cpp:26-48) and runs the watertight test
 * (src/io/mesh_validate.cpp:21-59): watertight meshes use PARITY, others GWN. */
typedef enum sdfb_sign_mode {
  SDFB_SIGN_AUTO = 0,
  SDFB_SIGN_PARITY = 1, /* exact +z ray parity, robust predicates */
  SDFB_SIGN_GWN = 2,    /* generalized winding number, |w| > 0.5 is inside */
  SDFB_SIGN_NONE = 3    /* unsigned distance */
} sdfb_sign_mode;

typedef struct sdfb_ctx sdfb_ctx;

/* Dense grid description (the reference's SdfGrid origin / voxelSize / nx, ny, nz,
 * src/convert/sdf_grid.h:21-26). */
typedef struct sdfb_grid_desc {
  float origin[3];
  float voxel_size;
  int32_t nx, ny, nz;
} sdfb_grid_desc;

/* Bake options. Zero-initialise and set struct_size = sizeof(sdfb_opts); zero fields take the
 * defaults named beside them. */
typedef struct sdfb_opts {
  uint32_t struct_size;
  int32_t sign_mode;      /* sdfb_sign_mode, default AUTO */
  float band_voxels;      /* GWN: width in voxels of the FP64 band around the surface, default 1 */
  int32_t leaf_size;      /* BVH leaf size 1..16, default: autotuned table */
  int32_t tile;           /* distance tile shape 1..6 (4x4x2, 8x4x1, 4x4x4, 8x4x2, 4x4x8, 8x4x4
                             cells per warp), 0: autotuned table */
  int32_t no_occupancy;   /* 1: skip occupancy (occ_out may be NULL) */
  int32_t no_distance;    /* 1: occupancy only (dist_out may be NULL) */
  int32_t count_work;     /* 1: count traversal work into stats (a slower, instrumented kernel) */
  int32_t stack_depth;    /* traversal stack entries, 32 or 64, 0: autotuned table */
  int32_t step_budget;    /* a distance tile's walk checks every this many steps whether all tiles
                             are handed out, and if so leaves its tile to a second pass where a
                             whole block finishes it; 0: autotuned table, -1: never */
  int32_t fault_inject;   /* testing only, 0 in normal use: SDFB_FAULT_* bits that make a bounded
                             device wait or limit run out on purpose (the bake then fails with the
                             status that limit maps to, and the context stays usable) */
  int32_t alloc_cap_kib;  /* testing only, 0 = none: a workspace allocation above this many KiB
                             fails as if the device were out of memory (SDFB_ERR_OUT_OF_MEMORY) */
  int32_t reserved[4];
} sdfb_opts;

/* sdfb_opts.fault_inject bits. None of them faults the GPU: each makes a wait or a limit that the
 * kernels already bound run out early, so the error path behind it can be tested. */
#define SDFB_FAULT_DISPATCH 1      /* no warp hands its block a new chunk of distance tiles: the
                                      other warps' bounded wait for one runs out -> INTERNAL */
#define SDFB_FAULT_STEP_LIMIT 2    /* a traversal walk may take only 8 steps -> INTERNAL */
#define SDFB_FAULT_SHALLOW_STACK 4 /* a 32-entry traversal stack holds 2 entries: the walk
                                      overflows and the bake reruns with 64 entries */
#define SDFB_FAULT_STACK_ALL 8     /* every traversal stack holds 2 entries -> OVERFLOW */

/* Per-call statistics, filled when the pointer is non-null. Times are CUDA-event times on the
 * bake stream (ms); counts are exact. */
typedef struct sdfb_stats {
  uint32_t struct_size;
  int32_t sign_mode_used;
  int32_t watertight;      /* 1, 0, or -1 when not evaluated */
  int32_t leaf_size_used;
  int32_t tile_used;
  int32_t stack_used;
  double ms_total;         /* first to last event on the device */
  double ms_prepare;       /* upload of the batch tables and counter reset */
  double ms_build;         /* triangle records, Morton codes, sort, hierarchy, refit, layout */
  double ms_occupancy;
  double ms_sign;          /* parity crossings or winding-number band */
  double ms_distance;      /* nearest-triangle traversal (+ fused sign) */
  uint64_t voxels;
  uint64_t triangles;
  uint64_t sat_tests;      /* triangle/box tests run by the occupancy kernel */
  uint64_t crossings;      /* parity crossings found */
  uint64_t box_tests;      /* count_work: point-box tests, one per cell */
  uint64_t tri_tests;      /* count_work: full point-triangle tests, one per cell */
  double flops_distance;   /* count_work: FP32 flops of the distance tests as executed, terms a lane
                              shares between its cells counted once (FMA = 2) */
  uint64_t kernel_launches; /* kernels this call launched */
  uint64_t gwn_fp64_cells;  /* GWN: cells whose winding number was evaluated in FP64 (band + ambiguous) */
  uint64_t graph_replayed;  /* 1 when the launch sequence was replayed from a CUDA graph */
  uint64_t tiles_deferred;  /* distance tiles that exceeded the step budget and were finished by a
                               whole block in the second distance pass */
  uint64_t plane_tests;     /* count_work: cell-plane lower-bound tests that screen triangles, per cell */
  uint64_t rect_tests;      /* count_work: in-plane bounding-rectangle tests after the plane screen,
                               per cell */
  uint64_t gwn_direct_cells; /* GWN: cells whose sign needed the direct FP64 sum over every cap */
} sdfb_stats;

/* ---- context ---------------------------------------------------------------------------- */

/* Creates a context on CUDA device `device` (sm_103 required). */
sdfb_status sdfb_ctx_create(int32_t device, sdfb_ctx **out);
void sdfb_ctx_destroy(sdfb_ctx *ctx);
/* Last error text of the context (empty when none); valid until the next call on ctx. */
const char *sdfb_last_error(const sdfb_ctx *ctx);
/* Library ABI version (SDFB_ABI_VERSION). */
int32_t sdfb_abi_version(void);
/* Releases cached device memory that no live object uses. */
sdfb_status sdfb_ctx_trim(sdfb_ctx *ctx);
/* Bytes of device memory the context holds (cached buffers and resident meshes). */
uint64_t sdfb_ctx_device_bytes(const sdfb_ctx *ctx);

/* ---- grids (bakeSdf sizing, src/convert/sdf_baker.cpp:138-148) -------------------------- */

/* voxel = max(extent, 1e-6) / max(res, 1); origin = bmin - 2 voxel;
 * n_axis = ceil((extent_axis + 4 voxel) / voxel) + 1, all in FP32 as the reference does. */
sdfb_status sdfb_grid_from_bounds_res(const float bmin[3], const float bmax[3], int32_t resolution,
                                      sdfb_grid_desc *out);

/* ---- plain bake (replaces italy::bakeSdf, src/convert/sdf_baker.h:8) --------------------- */

/* Synchronous bake from host buffers. dist_out holds nx*ny*nz floats, occ_out nx*ny*nz bytes;
 * either may be NULL to skip that output. opts and stats may be NULL. */
sdfb_status sdfb_bake(sdfb_ctx *ctx, const float *verts, uint32_t num_verts, const uint32_t *idx,
                      uint32_t num_tris, const sdfb_grid_desc *grid, const sdfb_opts *opts, float *dist_out,
                      uint8_t *occ_out, sdfb_stats *stats);

/* Same bake with every buffer already in device memory of the context's device. Work is
 * enqueued on `stream` (a cudaStream_t, NULL = the context's stream); the call returns after the
 * work completes and its error flags are read. */
sdfb_status sdfb_bake_device(sdfb_ctx *ctx, const float *d_verts, uint32_t num_verts, const uint32_t *d_idx,
                             uint32_t num_tris, const sdfb_grid_desc *grid, const sdfb_opts *opts,
                             float *d_dist_out, uint8_t *d_occ_out, void *stream, sdfb_stats *stats);

/* MeshAsset-layout bake (src/convert/sdf_baker.cpp:137-310): `positions` holds 9 floats per
 * triangle; the grid is sized from bounds and resolution exactly as bakeSdf does and written to
 * grid_out. Call once with dist_out = occ_out = NULL to learn the grid, then again with buffers
 * of grid_out->nx * ny * nz elements. */
sdfb_status sdfb_bake_soup(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                           const float bounds_max[3], int32_t resolution, const sdfb_opts *opts,
                           sdfb_grid_desc *grid_out, float *dist_out, uint8_t *occ_out, sdfb_stats *stats);

/* ---- sparse voxelization (replaces italy::voxelizeMesh, src/convert/voxelize.h:8) -------- */

/* `positions` holds 9 floats per triangle. origin = bounds_min, voxel = longest / res, cells in
 * the reference's insertion order (voxelize.cpp:52-107). Writes min(count, cap) cells (3 int32
 * each) and returns the full count in *count. */
sdfb_status sdfb_voxelize_sparse(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const float bounds_min[3],
                                 const float bounds_max[3], int32_t resolution, int32_t *cells_out, uint64_t cap,
                                 uint64_t *count, float origin_out[3], float *voxel_out);

/* ---- per-cell materials (src/convert/sdf_baker.cpp:42-128, src/convert/voxelize.cpp:12-107) */

/* One RGBA8 texture (TextureAsset, src/io/mesh_asset.h:10-15). */
typedef struct sdfb_texture {
  const uint8_t *rgba; /* width * height * 4 bytes, rows of texels */
  int32_t width;
  int32_t height;
  int32_t srgb;        /* nonzero: the texels are sRGB-encoded and are decoded to linear */
  int32_t reserved;
} sdfb_texture;

/* The MaterialAsset fields the bake reads (src/io/mesh_asset.h:17-31). */
typedef struct sdfb_material {
  float base_color[3];
  float metallic;
  float roughness;
  int32_t base_color_texture; /* index into the texture list; out of range = no texture */
} sdfb_material;

/* A MeshAsset's materials: per triangle t the material triangle_material[t] (material 0 past the
 * end of the list or of the material table), its base colour modulated by the texture texel
 * nearest the mean of the triangle's three uvs (uvs[3t..3t+2], wrapped to [0, 1)) when the
 * material names a texture and the triangle has uvs. */
typedef struct sdfb_materials {
  uint32_t struct_size;      /* sizeof(sdfb_materials) */
  uint32_t num_materials;    /* >= 1 */
  const sdfb_material *materials;
  const uint32_t *triangle_material; /* may be NULL */
  uint64_t num_triangle_material;
  const float *uvs;          /* 2 floats per soup vertex (3 per triangle); may be NULL */
  uint64_t num_uvs;          /* uv pairs */
  const sdfb_texture *textures;
  uint32_t num_textures;
  uint32_t reserved;
} sdfb_materials;

/* Per-cell material of the SDF grid (bakePerCellMaterial, src/convert/sdf_baker.cpp:76-128):
 * every triangle of the soup (9 floats each) that overlaps a cell by the occupancy rule adds its
 * material to the cell in triangle order; a cell's base colour, metallic and roughness are the
 * means, and a cell without a triangle keeps (1, 1, 1), 0 and 1. The grid is the bake's (e.g. from
 * sdfb_grid_from_bounds_res or sdfb_bake_soup). Outputs are host buffers of nx * ny * nz cells,
 * x fastest; base_color_out holds 3 floats per cell. Any output may be NULL. */
sdfb_status sdfb_bake_materials(sdfb_ctx *ctx, const float *positions, uint32_t num_tris, const sdfb_grid_desc *grid,
                                const sdfb_materials *materials, float *base_color_out, float *metallic_out,
                                float *roughness_out);

/* sdfb_voxelize_sparse plus VoxelGrid::colors (src/convert/voxelize.cpp:78-104): colors_out gets
 * 3 floats per written cell, the mean base colour of the triangles overlapping it. */
sdfb_status sdfb_voxelize_sparse_colors(sdfb_ctx *ctx, const float *positions, uint32_t num_tris,
                                        const float bounds_min[3], const float bounds_max[3], int32_t resolution,
                                        const sdfb_materials *materials, int32_t *cells_out, float *colors_out,
                                        uint64_t cap, uint64_t *count, float origin_out[3], float *voxel_out);

/* ---- consumer check (src/render/kernels/pathtracer.cu:587-613, 684-702, 740-787) --------- */

/* The renderer's trilinear sample of a baked grid (sampleSdf, pathtracer.cu:684-702) at
 * num_points points (3 floats each). `dist` is the grid's host distance buffer (nx*ny*nz, x
 * fastest); every axis needs at least 2 cells. */
sdfb_status sdfb_sample_sdf(sdfb_ctx *ctx, const sdfb_grid_desc *grid, const float *dist, const float *points,
                            uint64_t num_points, float *out);

/* The renderer's sphere-traced intersection with a baked grid (__intersection__sdf,
 * pathtracer.cu:740-787): per ray (origin, direction: 6 floats) the hit distance it reports within
 * [tmin, tmax], or -1 when it reports none. */
sdfb_status sdfb_trace_sdf(sdfb_ctx *ctx, const sdfb_grid_desc *grid, const float *dist, const float *rays,
                           uint64_t num_rays, float tmin, float tmax, float *t_out);

/* ---- mesh utilities (src/io/mesh_weld.cpp:26-48, src/io/mesh_validate.cpp:21-59) -------- */

/* Welds positions on the max(|extent| * 1e-5, 1e-6) lattice; welded_out gets one index per
 * position (first-occurrence numbering), *num_unique the number of distinct vertices. */
sdfb_status sdfb_weld(sdfb_ctx *ctx, const float *positions, uint32_t num_positions, const float bounds_min[3],
                      const float bounds_max[3], uint32_t *welded_out, uint32_t *num_unique);
/* Watertight test over a welded index buffer (3 per triangle): *watertight = 1 when no edge is
 * used once (boundary) or more than twice (non-manifold); degenerate triangles are skipped. */
sdfb_status sdfb_is_watertight(sdfb_ctx *ctx, const uint32_t *welded_idx, uint32_t num_tris, int32_t *watertight,
                               uint64_t *boundary_edges, uint64_t *nonmanifold_edges);

/* The same two on the device, for soups already in device memory (d_positions: 3 floats per
 * position; d_welded_out / d_welded_idx: device uint32). Work runs on `stream` (NULL = the
 * context's stream); the calls return after it completes. Same numbering and verdicts as above;
 * a mesh without triangles is not watertight (mesh_validate.cpp:23-26). */
sdfb_status sdfb_weld_device(sdfb_ctx *ctx, const float *d_positions, uint32_t num_positions,
                             const float bounds_min[3], const float bounds_max[3], uint32_t *d_welded_out,
                             uint32_t *num_unique, void *stream);
sdfb_status sdfb_is_watertight_device(sdfb_ctx *ctx, const uint32_t *d_welded_idx, uint32_t num_tris,
                                      int32_t *watertight, uint64_t *boundary_edges, uint64_t *nonmanifold_edges,
                                      void *stream);

/* ---- batched bake -------------------------------------------------------------------------- */

typedef struct sdfb_mesh_desc {
  const float *verts;    /* V x 3 */
  const uint32_t *idx;   /* T x 3 */
  uint32_t num_verts;
  uint32_t num_tris;
} sdfb_mesh_desc;

/* Bakes `count` meshes, each onto its own grid, in one persistent launch per stage replayed from
 * a CUDA graph. Buffers are host memory; dist_outs[i] / occ_outs[i] have grid i's cell count
 * (either array, or any entry, may be NULL). stats (optional) receives the aggregate. */
sdfb_status sdfb_bake_batch(sdfb_ctx *ctx, uint32_t count, const sdfb_mesh_desc *meshes,
                            const sdfb_grid_desc *grids, const sdfb_opts *opts, float *const *dist_outs,
                            uint8_t *const *occ_outs, sdfb_stats *stats);

/* Device-buffer form of the batched bake: every pointer in meshes/dist_outs/occ_outs is device
 * memory. Returns after completion. */
sdfb_status sdfb_bake_batch_device(sdfb_ctx *ctx, uint32_t count, const sdfb_mesh_desc *meshes,
                                   const sdfb_grid_desc *grids, const sdfb_opts *opts, float *const *dist_outs,
                                   uint8_t *const *occ_outs, void *stream, sdfb_stats *stats);

/* ---- serving ------------------------------------------------------------------------------- */

typedef struct sdfb_server sdfb_server;

typedef struct sdfb_server_opts {
  uint32_t struct_size;
  uint64_t hbm_budget_bytes; /* admission budget for resident meshes + in-flight jobs */
  int32_t max_inflight;      /* jobs on the device at once, default 128 */
  int32_t wave_voxels_log2;  /* most work per wave (log2 voxels), default 28; a wave takes what is queued */
  int32_t reserved[8];
} sdfb_server_opts;

typedef struct sdfb_request_info {
  uint32_t struct_size;
  int32_t status;        /* sdfb_status of the finished request */
  double t_submit_ms;    /* host monotonic clock */
  double t_admit_ms;
  double t_done_ms;
  uint64_t voxels;
  int32_t mesh_was_resident;
  int32_t pad;
} sdfb_request_info;

/* Starts the serving loop (one admission/scheduling thread) on ctx's device. */
sdfb_status sdfb_server_create(sdfb_ctx *ctx, const sdfb_server_opts *opts, sdfb_server **out);
/* Drains in-flight work and stops the loop. */
void sdfb_server_destroy(sdfb_server *srv);
/* Uploads a mesh and builds its hierarchy on the device; *mesh_id identifies it from then on.
 * Registering identical contents again returns the resident id (content hash). */
sdfb_status sdfb_mesh_register(sdfb_server *srv, const float *verts, uint32_t num_verts, const uint32_t *idx,
                               uint32_t num_tris, uint64_t *mesh_id);
/* Queues a bake of a registered mesh. Output buffers are host memory owned by the caller and
 * must stay valid until sdfb_poll reports the request done. */
sdfb_status sdfb_submit(sdfb_server *srv, uint64_t mesh_id, const sdfb_grid_desc *grid, const sdfb_opts *opts,
                        float *dist_out, uint8_t *occ_out, uint64_t *request_id);
/* Waits up to timeout_ms (0 = just look, < 0 = forever) for a request. *done = 1 when finished,
 * with its outcome in info (optional). A finished request is forgotten after it is reported. */
sdfb_status sdfb_poll(sdfb_server *srv, uint64_t request_id, int32_t timeout_ms, int32_t *done,
                      sdfb_request_info *info);
/* Text of the server's last error (valid in the calling thread until its next call here). */
const char *sdfb_server_last_error(const sdfb_server *srv);

/* ---- occupancy without allocation (no counterpart in the reference) ---------------------- */

/* Dense occupancy -- the same SAT rule and result as sdfb_bake's occ_out -- for callers that may
 * not allocate device memory: plugins whose host application owns every device allocation,
 * processes held to a fixed device-memory quota, and latency-bound loops that must avoid the
 * allocator and cudaFree's device-wide synchronisation. All buffers are device memory supplied by
 * the caller;
 * work is enqueued on `stream` (a cudaStream_t, NULL = the legacy default stream) and not waited
 * for. Working memory is one fixed device array inside the library (about 16 MiB, held on every
 * device that loads the library until the process exits), so:
 *   - meshes above 1,048,576 triangles are rejected with SDFB_ERR_INVALID_ARGUMENT;
 *   - the first call on each device sets up the array's address and must come before any stream
 *     capture on that device;
 *   - calls whose work overlaps on the GPU share the array and race; order them on one stream;
 *   - launch failures are read with cudaGetLastError, which also clears an error left pending by
 *     the caller's own earlier work on this host thread: check your own errors first. */
sdfb_status sdfb_occupancy_noalloc(const float *d_verts, uint32_t num_verts, const uint32_t *d_idx,
                                   uint32_t num_tris, const sdfb_grid_desc *grid, uint8_t *d_occ_out,
                                   void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SDFB_H */
