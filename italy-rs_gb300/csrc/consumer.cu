// The consumer side of a baked grid, without a renderer: the path tracer's trilinear SDF sample
// (src/render/kernels/pathtracer.cu:684-702) and its sphere-traced SDF intersection
// (pathtracer.cu:740-787, with the slab test of :587-613) as CUDA kernels over the grid in device
// memory. They let a bake be checked the way the renderer consumes it: where rays meet the zero
// level set of the interpolated grid, against exact ray/mesh intersections.
//
// Every FP32 operation is one IEEE operation (_rn intrinsics, no contraction), so the CPU oracle's
// C restatement reproduces the results bit for bit. One thread per point or ray.
#include <algorithm>
#include <cstdarg>

#include "api_internal.h"
#include "common.cuh"
#include "kernels.h"

using namespace sdfb;

namespace {

constexpr int kThreads = 256;

struct SdfView {
  const float *dist;
  float ox, oy, oz, voxel;
  int nx, ny, nz;
};

__device__ __forceinline__ float at(const SdfView &g, int x, int y, int z) {
  return __ldg(g.dist + (int64_t(z) * g.ny + y) * g.nx + x);
}

__device__ __forceinline__ float lerp_ref(float a, float b, float f) {
  return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, f)), __fmul_rn(b, f));  // a * (1 - f) + b * f
}

// sampleSdf (pathtracer.cu:684-702).
__device__ float sample_sdf(const SdfView &g, float px, float py, float pz) {
  const float lx = __fsub_rn(__fdiv_rn(__fsub_rn(px, g.ox), g.voxel), 0.5f);
  const float ly = __fsub_rn(__fdiv_rn(__fsub_rn(py, g.oy), g.voxel), 0.5f);
  const float lz = __fsub_rn(__fdiv_rn(__fsub_rn(pz, g.oz), g.voxel), 0.5f);
  const int x0 = max(0, min(g.nx - 2, f2i_sat(floorf(lx))));
  const int y0 = max(0, min(g.ny - 2, f2i_sat(floorf(ly))));
  const int z0 = max(0, min(g.nz - 2, f2i_sat(floorf(lz))));
  const float fx = fminf(fmaxf(__fsub_rn(lx, static_cast<float>(x0)), 0.0f), 1.0f);
  const float fy = fminf(fmaxf(__fsub_rn(ly, static_cast<float>(y0)), 0.0f), 1.0f);
  const float fz = fminf(fmaxf(__fsub_rn(lz, static_cast<float>(z0)), 0.0f), 1.0f);
  const float c00 = lerp_ref(at(g, x0, y0, z0), at(g, x0 + 1, y0, z0), fx);
  const float c10 = lerp_ref(at(g, x0, y0 + 1, z0), at(g, x0 + 1, y0 + 1, z0), fx);
  const float c01 = lerp_ref(at(g, x0, y0, z0 + 1), at(g, x0 + 1, y0, z0 + 1), fx);
  const float c11 = lerp_ref(at(g, x0, y0 + 1, z0 + 1), at(g, x0 + 1, y0 + 1, z0 + 1), fx);
  const float c0 = lerp_ref(c00, c10, fy);
  const float c1 = lerp_ref(c01, c11, fy);
  return lerp_ref(c0, c1, fz);
}

__device__ __forceinline__ float sample_at(const SdfView &g, const float o[3], const float d[3], float t) {
  return sample_sdf(g, __fadd_rn(o[0], __fmul_rn(t, d[0])), __fadd_rn(o[1], __fmul_rn(t, d[1])),
                    __fadd_rn(o[2], __fmul_rn(t, d[2])));
}

// slabTest (pathtracer.cu:587-613) without the entry face, which the SDF program does not use.
__device__ bool slab(const float o[3], const float d[3], const float lo[3], const float hi[3], float &t0, float &t1) {
  for (int a = 0; a < 3; ++a) {
    const float inv = __fdiv_rn(1.0f, d[a]);
    float tn = __fmul_rn(__fsub_rn(lo[a], o[a]), inv);
    float tf = __fmul_rn(__fsub_rn(hi[a], o[a]), inv);
    if (tn > tf) {
      const float tmp = tn;
      tn = tf;
      tf = tmp;
    }
    if (tn > t0) t0 = tn;
    if (tf < t1) t1 = tf;
    if (t0 > t1) return false;
  }
  return true;
}

// __intersection__sdf (pathtracer.cu:740-787): the reported hit distance, or -1 when the program
// reports none.
__device__ float trace_sdf(const SdfView &g, const float o[3], const float d[3], float tmin, float tmax) {
  const float lo[3] = {g.ox, g.oy, g.oz};
  const float hi[3] = {__fadd_rn(g.ox, __fmul_rn(static_cast<float>(g.nx), g.voxel)),
                       __fadd_rn(g.oy, __fmul_rn(static_cast<float>(g.ny), g.voxel)),
                       __fadd_rn(g.oz, __fmul_rn(static_cast<float>(g.nz), g.voxel))};
  float t0 = tmin, t1 = tmax;
  if (!slab(o, d, lo, hi, t0, t1)) return -1.0f;
  const float eps = __fmul_rn(g.voxel, 0.02f);
  const float min_step = __fmul_rn(g.voxel, 0.05f);
  const float min_adv = __fmul_rn(g.voxel, 0.3f);
  float t = t0, prev_t = t0;
  float prev = sample_at(g, o, d, t0);
  t = __fadd_rn(t, fmaxf(fabsf(prev), min_step));
  for (int i = 1; i < 512 && t <= t1; ++i) {
    const float dist = sample_at(g, o, d, t);
    const bool crossed = (prev > 0.0f) != (dist > 0.0f);
    if ((crossed || fabsf(dist) < eps) && __fsub_rn(t, t0) > min_adv) {
      float hit = t;
      if (crossed) {
        float a = prev_t, b = t, fa = prev, fb = dist;
        for (int k = 0; k < 8; ++k) {
          const float m = __fmul_rn(0.5f, __fadd_rn(a, b));
          const float fm = sample_at(g, o, d, m);
          if ((fa > 0.0f) != (fm > 0.0f)) {
            b = m;
            fb = fm;
          } else {
            a = m;
            fa = fm;
          }
        }
        const float denom = __fsub_rn(fa, fb);
        hit = fabsf(denom) > 1e-9f ? __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), __fdiv_rn(fa, denom)))
                                   : __fmul_rn(0.5f, __fadd_rn(a, b));
      }
      return fmaxf(hit, t0);
    }
    prev_t = t;
    prev = dist;
    t = __fadd_rn(t, fmaxf(__fmul_rn(fabsf(dist), 0.85f), min_step));
  }
  return -1.0f;
}

__global__ __launch_bounds__(kThreads) void k_sample(SdfView g, const float *__restrict__ pts, uint64_t n,
                                                     float *__restrict__ out) {
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads)
    out[i] = sample_sdf(g, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
}

__global__ __launch_bounds__(kThreads) void k_trace(SdfView g, const float *__restrict__ rays, uint64_t n, float tmin,
                                                    float tmax, float *__restrict__ out) {
  for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < n; i += uint64_t(gridDim.x) * kThreads) {
    const float o[3] = {rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]};
    const float d[3] = {rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]};
    out[i] = trace_sdf(g, o, d, tmin, tmax);
  }
}

#define CK(call)                                            \
  do {                                                      \
    const cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return ctx_cuda(ctx, e_, #call); \
  } while (0)

#define ENSURE(buf, bytes)                                                                       \
  do {                                                                                           \
    if (!(buf).ensure(bytes))                                                                    \
      return ctx_fail(ctx, SDFB_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of device memory", \
                      static_cast<size_t>(bytes));                                               \
  } while (0)

// Uploads the grid and `in_floats` floats of queries; returns the view and the device buffers.
sdfb_status stage(sdfb_ctx *ctx, const sdfb_grid_desc *grid, const float *dist, const float *in, uint64_t in_floats,
                  uint64_t n_out, SdfView &v, float *&d_in, float *&d_out) {
  if (!grid_ok(grid) || grid->nx < 2 || grid->ny < 2 || grid->nz < 2)
    return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "the grid needs at least 2 cells along each axis");
  if (!dist || (n_out && !in)) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "null argument");
  cudaSetDevice(ctx->device);
  const cudaStream_t st = ctx->stream;
  const uint64_t cells = uint64_t(grid->nx) * grid->ny * grid->nz;
  ENSURE(ctx->cons_grid, cells * 4);
  ENSURE(ctx->cons_io, (((in_floats + 63) & ~uint64_t(63)) + n_out) * 4 + 256);  // queries, then results
  CK(cudaMemcpyAsync(ctx->cons_grid.p, dist, cells * 4, cudaMemcpyHostToDevice, st));
  d_in = static_cast<float *>(ctx->cons_io.p);
  d_out = d_in + ((in_floats + 63) & ~uint64_t(63));
  if (in_floats) CK(cudaMemcpyAsync(d_in, in, in_floats * 4, cudaMemcpyHostToDevice, st));
  v.dist = static_cast<const float *>(ctx->cons_grid.p);
  v.ox = grid->origin[0];
  v.oy = grid->origin[1];
  v.oz = grid->origin[2];
  v.voxel = grid->voxel_size;
  v.nx = grid->nx;
  v.ny = grid->ny;
  v.nz = grid->nz;
  return SDFB_OK;
}

unsigned blocks_for(sdfb_ctx *ctx, uint64_t n) {
  return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + kThreads - 1) / kThreads,
                                                                         uint64_t(ctx->num_sms) * 16)));
}

}  // namespace

extern "C" sdfb_status sdfb_sample_sdf(sdfb_ctx *ctx, const sdfb_grid_desc *grid, const float *dist,
                                       const float *points, uint64_t num_points, float *out) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (num_points && !out) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "out is NULL");
  SdfView v;
  float *d_in = nullptr, *d_out = nullptr;
  const sdfb_status s = stage(ctx, grid, dist, points, num_points * 3, num_points, v, d_in, d_out);
  if (s != SDFB_OK) return s;
  if (num_points == 0) return SDFB_OK;
  const cudaStream_t st = ctx->stream;
  k_sample<<<blocks_for(ctx, num_points), kThreads, 0, st>>>(v, d_in, num_points, d_out);
  note_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, d_out, num_points * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}

extern "C" sdfb_status sdfb_trace_sdf(sdfb_ctx *ctx, const sdfb_grid_desc *grid, const float *dist, const float *rays,
                                      uint64_t num_rays, float tmin, float tmax, float *t_out) {
  if (!ctx) return SDFB_ERR_INVALID_ARGUMENT;
  ctx->err.clear();
  if (num_rays && !t_out) return ctx_fail(ctx, SDFB_ERR_INVALID_ARGUMENT, "t_out is NULL");
  SdfView v;
  float *d_in = nullptr, *d_out = nullptr;
  const sdfb_status s = stage(ctx, grid, dist, rays, num_rays * 6, num_rays, v, d_in, d_out);
  if (s != SDFB_OK) return s;
  if (num_rays == 0) return SDFB_OK;
  const cudaStream_t st = ctx->stream;
  k_trace<<<blocks_for(ctx, num_rays), kThreads, 0, st>>>(v, d_in, num_rays, tmin, tmax, d_out);
  note_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(t_out, d_out, num_rays * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SDFB_OK;
}
