// sdfb_occupancy_noalloc: dense occupancy (the reference's SAT voxelization rule) for callers that
// may not allocate device memory.
//
// Some callers cannot call cudaMalloc: a plugin running inside a host application that owns every
// device allocation and hands the plugin only its input and output buffers; a process held to a
// fixed device-memory quota, where a late allocation can fail; a latency-bound render or
// simulation loop that must not hit cudaFree's implicit device-wide synchronisation or the
// allocator's unbounded time. This entry point serves them: it runs the same occupancy kernels
// as the context-based bake, but its working memory -- per-triangle candidate counts, their scan and
// the one-mesh batch record -- lives in a fixed file-scope device array, so a call allocates
// nothing. The caller passes device inputs and the device output grid. The one-mesh record is
// written into the array by a one-thread kernel that receives it as a launch argument, so no
// host memory is read after the call returns.
//
// Limits and rules:
//   * at most kNoAllocMaxTris triangles; larger meshes are rejected with
//     SDFB_ERR_INVALID_ARGUMENT before anything is launched;
//   * the array is set aside once per device that loads the library and stays there until the
//     process exits;
//   * the first call on each device looks up the array's device address (cudaGetSymbolAddress)
//     with that device current; make that first call before any stream capture;
//   * every call shares the one array: calls whose work overlaps on the GPU (different streams,
//     or different host threads without ordering) race on it. Nothing in it has to start at zero:
//     each call writes the counts and records it reads, and the occupancy grid is cleared by the
//     call itself;
//   * launch failures are read with cudaGetLastError, which also clears an error that the
//     caller's own earlier work left pending on this host thread.
#include <cstring>
#include <mutex>

#include "api_internal.h"
#include "common.cuh"
#include "kernels.h"

using namespace sdfb;

namespace {

constexpr uint32_t kNoAllocMaxTris = 1u << 20;  // 1,048,576 triangles
constexpr size_t kRecordBytes = 4096;           // one MeshRec and its prefix tables
// Candidate counts (8 B per triangle), their exclusive scan (8 B per triangle + 1), the scan's
// block sums, plus alignment slack: about 16 MiB in all.
constexpr size_t kScratchBytes = kRecordBytes + size_t(kNoAllocMaxTris) * 16 + (size_t(1) << 16);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

// The one-mesh batch record and its prefix tables.
struct Records {
  MeshRec rec;
  alignas(8) uint64_t tris[2];
  alignas(8) uint64_t cells[2];
  alignas(8) uint64_t zero[2];
};
static_assert(sizeof(Records) <= kRecordBytes, "records fit their slot");
static_assert(sizeof(Records) <= 4000, "records pass as one kernel argument");

// Writes the records into the array; the argument is copied when the launch is enqueued.
__global__ void k_put_records(Records *dst, Records src) { *dst = src; }

}  // namespace

extern "C" sdfb_status sdfb_occupancy_noalloc(const float *d_verts, uint32_t num_verts, const uint32_t *d_idx,
                                              uint32_t num_tris, const sdfb_grid_desc *grid, uint8_t *d_occ_out,
                                              void *stream) {
  if (!d_verts || !d_idx || !d_occ_out || !grid_ok(grid) || num_verts == 0) return SDFB_ERR_INVALID_ARGUMENT;
  if (num_tris == 0 || num_tris > kNoAllocMaxTris) return SDFB_ERR_INVALID_ARGUMENT;
  if (occupancy_temp_bytes(num_tris) + kRecordBytes > kScratchBytes) return SDFB_ERR_INVALID_ARGUMENT;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return SDFB_ERR_NO_DEVICE;
  }
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      // Set-up, once per device, with that device current: the array's device address.
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return SDFB_ERR_CUDA;
      }
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t cells = uint64_t(grid->nx) * grid->ny * grid->nz;
  Records h;
  std::memset(&h, 0, sizeof h);
  h.rec.verts = d_verts;
  h.rec.idx = d_idx;
  h.rec.num_verts = num_verts;
  h.rec.num_tris = num_tris;
  h.rec.occ = d_occ_out;
  h.rec.g = to_dev(*grid);
  h.rec.leaf_size = 1;
  h.tris[1] = num_tris;
  h.cells[1] = cells;
  char *d = static_cast<char *>(scratch);
  k_put_records<<<1, 1, 0, st>>>(reinterpret_cast<Records *>(d), h);
  if (cudaGetLastError() != cudaSuccess) return SDFB_ERR_CUDA;
  const Records *dr = reinterpret_cast<const Records *>(d);
  BatchDev B;
  B.num_meshes = 1;
  B.recs = &dr->rec;
  B.tri_starts = dr->tris;
  B.cell_starts = dr->cells;
  B.ptri_starts = B.tile_starts = B.gwn_tile_starts = dr->zero;
  B.total_tris = num_tris;
  B.total_cells = cells;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const cudaError_t e = occupancy_batch(B, nullptr, d + kRecordBytes, kScratchBytes - kRecordBytes, nullptr,
                                        sms > 0 ? sms : 1, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SDFB_ERR_CUDA;
  }
  return SDFB_OK;
}
