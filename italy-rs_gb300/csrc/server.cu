// Serving loop: continuous batching of bake requests over device-resident meshes.
//
// The reference bakes one mesh per call, rebuilding its acceleration structure and pipeline every
// time (src/convert/sdf_baker.cpp:150-305). Here a server keeps meshes and their hierarchies
// resident and runs requests in waves:
//
//   * sdfb_mesh_register uploads a mesh, decides its sign mode (the weld + watertight gate, on the
//     device), caps it for the winding number when needed, and builds its hierarchy in one of a
//     few registration slots (each its own stream and workspace), so registrations from several
//     threads overlap. Meshes are keyed by a hash of their contents, so a repeat registration is
//     a cache hit; a thread registering a mesh another thread is building waits for that build.
//     Resident bytes count against the HBM budget; unreferenced meshes are evicted least
//     recently used first when a new one needs room.
//   * sdfb_submit queues a request; the scheduler thread admits queued requests into the next
//     wave while a wave slot is free and the budget holds (resident meshes + every in-flight
//     wave's outputs). A wave is one batched launch sequence (orchestrate.cu) over all its
//     requests; waves run on separate streams, so a wave admitted while others are on the GPU
//     overlaps with them. Each cell is computed as in a single bake with the wave's launch
//     parameters (those of its largest grid), so a result is the same alone and in any mix up to
//     rounding where two triangles nearly tie (bit for bit under the same parameters).
//   * Outputs go straight to the caller's buffers when they are pinned (a pinned distance grid is
//     written in place by the distance kernel, occupancy by cudaMemcpyAsync), else through the
//     wave's pinned staging buffer and a host copy when the wave retires.
//   * sdfb_poll waits (bounded) on a condition variable for a request's completion.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "host_mesh.h"
#include "kernels.h"

using namespace sdfb;

namespace {

constexpr int kRegSlots = 4;  // meshes registered (uploaded, gated, built) at the same time
// While a registration is in progress, waves may launch their persistent kernels on kReserveSms
// fewer SMs and run one after another (kSerialWaves), so that a registration's steps (gate, caps,
// hierarchy, separated by host reads) are not queued behind the waves in flight. Off: on the
// serving stream (Poisson 200 requests/s, 70% new meshes) 8 reserved SMs with serial waves halved
// register()'s own latency but lowered capacity 974 -> 933 M voxels/s and doubled the requests'
// p50 (0.37 -> 0.73-1.9 s); registration streams keep the highest priority instead.
constexpr int kReserveSms = 0;
constexpr bool kSerialWaves = false;

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Two independent 64-bit content hashes of a byte range, in one pass over 8-byte words: h.a
// multiplies by the FNV prime and folds high bits down, h.b adds each word to a golden-ratio
// multiply-rotate chain; both end in an avalanche. A mesh's id is its a-hash; the b-hash and the
// vertex and triangle counts are compared on every cache hit, so two meshes whose ids collide are
// never taken for each other.
struct Hash2 {
  uint64_t a = 0xcbf29ce484222325ull, b = 0x6a09e667f3bcc909ull;
};

inline uint64_t avalanche(uint64_t h) {
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdull;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ull;
  h ^= h >> 33;
  return h;
}

void content_hash(const void *p, size_t n, Hash2 &h) {
  const uint8_t *bytes = static_cast<const uint8_t *>(p);
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, bytes + i, 8);
    h.a = (h.a ^ w) * 0x100000001b3ull;
    h.a ^= h.a >> 29;
    h.b = (h.b + w) * 0x9e3779b97f4a7c15ull;
    h.b = (h.b << 31) | (h.b >> 33);
  }
  for (; i < n; ++i) {
    h.a = (h.a ^ bytes[i]) * 0x100000001b3ull;
    h.b = (h.b + bytes[i]) * 0x9e3779b97f4a7c15ull;
  }
}

// Stream-ordered device allocation (no device-wide synchronisation when freed).
struct AsyncBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Resident {
  uint64_t id = 0;
  uint64_t check = 0;  // the second content hash, compared with V and T on a cache hit
  AsyncBuf verts, idx, pverts, pidx, cidx, bvh, caps;
  ResidentBvh tree, cap_tree;
  uint32_t V = 0, T = 0, pV = 0, pT = 0, cT = 0;
  int sign = kSignParity, watertight = -1;
  uint64_t bytes = 0;
  uint64_t last_use = 0;
  int refs = 0;  // in-flight requests
};

struct Request {
  uint64_t id = 0, mesh = 0;
  sdfb_grid_desc grid{};
  sdfb_opts opts{};
  float *dist_out = nullptr;
  uint8_t *occ_out = nullptr;
  bool dist_pinned = false, occ_pinned = false;
  float *dist_direct = nullptr;  // device address of a pinned distance output the wave writes in place
  double t_submit = 0, t_admit = 0, t_done = 0;
  int status = -1;  // -1 pending, else sdfb_status
  uint64_t voxels = 0;
  int was_resident = 0;
  bool done = false;
  void *res = nullptr;  // the Resident mesh, pinned by a reference while the request lives
};

struct Wave {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Workspace ws;
  DevBuf out_dist, out_occ;
  PinBuf stage_dist, stage_occ;
  std::vector<Request *> reqs;
  std::vector<uint64_t> offs;  // cell offset of each request in the wave buffers
  std::vector<PlanMesh> plan;
  BatchState state;
  sdfb_opts opts{};
  uint64_t bytes = 0;  // budget charge of this wave
  bool busy = false;
  bool lean = false;  // launched while a registration was in progress
};

bool is_pinned(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged;
}

// The device address of page-locked host memory, or null (the distance kernel then writes the
// request's grid in place over NVLink-C2C).
float *mapped_host(float *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<float *>(a.devicePointer) : nullptr;
}

}  // namespace

struct sdfb_server {
  int device = 0;
  std::unique_ptr<sdfb_ctx> sched;  // the scheduler's private context (error text, tuned tables)
  // Registration slots: private contexts (stream, workspace) that build meshes concurrently.
  std::vector<std::unique_ptr<sdfb_ctx>> regs;
  std::vector<char> reg_busy;
  std::unordered_set<uint64_t> building;  // meshes being registered (their first registrant builds)
  std::condition_variable cv_reg;
  std::vector<std::unique_ptr<Wave>> waves;
  std::thread thread;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::unordered_map<uint64_t, std::unique_ptr<Resident>> meshes;
  std::deque<Request *> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_req = 1, tick = 0;
  uint64_t budget = 0, resident_bytes_used = 0, inflight_bytes = 0;
  int max_inflight = 128, inflight = 0;
  uint64_t wave_cells = 1ull << 27;
  cudaEvent_t last_wave_done = nullptr;  // the last launched wave's completion (serial waves)
  int all_sms = 0;
  std::string err;
  cudaMemPool_t pool = nullptr;

  sdfb_status fail(sdfb_status s, const std::string &m) {
    std::lock_guard<std::mutex> g(err_mu);
    err = m;
    return s;
  }
  std::mutex err_mu;

  void run();
  bool launch_wave(Wave &w);
  void retire_wave(Wave &w);
  void free_resident(Resident &r, cudaStream_t st);
  bool make_room(uint64_t need);
};

namespace {

// high_priority: the stream's pending blocks are scheduled before those of default-priority
// streams (the waves') as SMs free up.
std::unique_ptr<sdfb_ctx> make_private_ctx(int device, int num_sms, const sdfb_ctx *tuned, bool high_priority = false) {
  auto c = std::make_unique<sdfb_ctx>();
  c->device = device;
  c->num_sms = num_sms;
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
    cudaGetLastError();
    greatest = least = 0;
  }
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, high_priority ? greatest : least) != cudaSuccess)
    return nullptr;
  if (!c->ws.init()) return nullptr;
  std::memcpy(c->tuned_leaf, tuned->tuned_leaf, sizeof c->tuned_leaf);
  std::memcpy(c->tuned_tile, tuned->tuned_tile, sizeof c->tuned_tile);
  std::memcpy(c->tuned_stack, tuned->tuned_stack, sizeof c->tuned_stack);
  std::memcpy(c->tuned_budget, tuned->tuned_budget, sizeof c->tuned_budget);
  c->batch_tile = tuned->batch_tile;
  c->batch_stack = tuned->batch_stack;
  c->batch_budget = tuned->batch_budget;
  return c;
}

bool async_alloc(AsyncBuf &b, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return true;
  if (cudaMallocAsync(&b.p, bytes, st) != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return false;
  }
  b.bytes = bytes;
  return true;
}

void async_free(AsyncBuf &b, cudaStream_t st) {
  if (b.p) cudaFreeAsync(b.p, st);
  b.p = nullptr;
  b.bytes = 0;
}

}  // namespace

void sdfb_server::free_resident(Resident &r, cudaStream_t st) {
  AsyncBuf *bs[] = {&r.verts, &r.idx, &r.pverts, &r.pidx, &r.cidx, &r.bvh, &r.caps};
  for (AsyncBuf *b : bs) async_free(*b, st);
}

// Evicts unreferenced meshes, least recently used first, until `need` more bytes fit. mu held.
bool sdfb_server::make_room(uint64_t need) {
  while (resident_bytes_used + inflight_bytes + need > budget) {
    Resident *victim = nullptr;
    for (auto &kv : meshes)
      if (kv.second->refs == 0 && (!victim || kv.second->last_use < victim->last_use)) victim = kv.second.get();
    if (!victim) return false;
    resident_bytes_used -= victim->bytes;
    free_resident(*victim, sched->stream);
    meshes.erase(victim->id);
  }
  return true;
}

void enqueue_readback(Wave &w);

bool sdfb_server::launch_wave(Wave &w) {
  // runs unlocked: every request holds a reference on its mesh, so r->res cannot go away
  std::vector<PlanMesh> &plan = w.plan;
  plan.clear();
  w.offs.clear();
  uint64_t cells = 0;
  for (Request *r : w.reqs) {
    w.offs.push_back(cells);
    cells += uint64_t(r->grid.nx) * r->grid.ny * r->grid.nz;
  }
  const bool any_dist = std::any_of(w.reqs.begin(), w.reqs.end(), [](Request *r) { return r->dist_out != nullptr; });
  const bool any_occ = std::any_of(w.reqs.begin(), w.reqs.end(), [](Request *r) { return r->occ_out != nullptr; });
  if ((any_dist && !w.out_dist.ensure(cells * 4)) || (any_occ && !w.out_occ.ensure(cells))) return false;
  const bool stage_d = std::any_of(w.reqs.begin(), w.reqs.end(), [](Request *r) { return r->dist_out && !r->dist_pinned; });
  const bool stage_o = std::any_of(w.reqs.begin(), w.reqs.end(), [](Request *r) { return r->occ_out && !r->occ_pinned; });
  if ((stage_d && !w.stage_dist.ensure(cells * 4)) || (stage_o && !w.stage_occ.ensure(cells))) return false;
  for (size_t k = 0; k < w.reqs.size(); ++k) {
    Request *r = w.reqs[k];
    Resident *m = static_cast<Resident *>(r->res);
    PlanMesh p;
    p.verts = static_cast<const float *>(m->verts.p);
    p.idx = static_cast<const uint32_t *>(m->idx.p);
    p.V = m->V;
    p.T = m->T;
    const int forced = r->opts.sign_mode;
    p.sign = forced == SDFB_SIGN_NONE ? kSignNone : m->sign;
    p.watertight = m->watertight;
    if (m->sign == kSignGwn) {
      p.pverts = static_cast<const float *>(m->pverts.p);
      p.pidx = static_cast<const uint32_t *>(m->pidx.p);
      p.pV = m->pV;
      p.pT = m->pT;
      p.cverts = p.pverts;
      p.cidx = static_cast<const uint32_t *>(m->cidx.p);
      p.cT = m->cT;
      p.caps = m->cT ? &m->cap_tree : nullptr;
    }
    p.bvh = &m->tree;
    p.grid = r->grid;
    // A pinned distance output is written in place, except for winding-number meshes, whose band
    // pass reads the distances back.
    r->dist_direct = (r->dist_pinned && m->sign != kSignGwn) ? mapped_host(r->dist_out) : nullptr;
    p.dist = r->dist_out ? (r->dist_direct ? r->dist_direct : static_cast<float *>(w.out_dist.p) + w.offs[k])
                         : nullptr;
    p.occ = r->occ_out ? static_cast<uint8_t *>(w.out_occ.p) + w.offs[k] : nullptr;
    plan.push_back(p);
  }
  w.opts = w.reqs[0]->opts;
  w.opts.sign_mode = SDFB_SIGN_AUTO;  // per-mesh signs are already resolved in the plan
  sched->num_sms = w.lean ? std::max(1, all_sms - kReserveSms) : all_sms;
  if (kSerialWaves && w.lean && last_wave_done) cudaStreamWaitEvent(w.stream, last_wave_done, 0);
  sdfb_status s = enqueue_batch(sched.get(), w.ws, w.stream, plan, w.opts, false, w.state);
  if (s != SDFB_OK) {
    for (Request *r : w.reqs) r->status = s;
    return true;
  }
  enqueue_readback(w);
  cudaEventRecord(w.done, w.stream);
  last_wave_done = w.done;
  return true;
}

// Copies each request's grids out of the wave buffers: straight into pinned caller buffers,
// through the wave's pinned staging buffer otherwise (finished by retire_wave on the host).
// Distances already written in place need no copy.
void enqueue_readback(Wave &w) {
  for (size_t k = 0; k < w.reqs.size(); ++k) {
    Request *r = w.reqs[k];
    const uint64_t n = uint64_t(r->grid.nx) * r->grid.ny * r->grid.nz;
    if (r->dist_out && !r->dist_direct) {
      const float *src = static_cast<const float *>(w.out_dist.p) + w.offs[k];
      void *dst = r->dist_pinned ? static_cast<void *>(r->dist_out)
                                 : static_cast<void *>(static_cast<float *>(w.stage_dist.p) + w.offs[k]);
      cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToHost, w.stream);
    }
    if (r->occ_out) {
      const uint8_t *src = static_cast<const uint8_t *>(w.out_occ.p) + w.offs[k];
      void *dst = r->occ_pinned ? static_cast<void *>(r->occ_out)
                                : static_cast<void *>(static_cast<uint8_t *>(w.stage_occ.p) + w.offs[k]);
      cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, w.stream);
    }
  }
}

void sdfb_server::retire_wave(Wave &w) {
  sdfb_status s = SDFB_OK;
  bool failed_early = false;
  for (Request *r : w.reqs)
    if (r->status >= 0) failed_early = true;
  if (!failed_early) {
    s = finish_batch(sched.get(), w.ws, w.stream, w.state, w.plan, nullptr);
    for (int attempt = 0; attempt < 3 && s == SDFB_ERR_BUSY; ++attempt) {  // crossing list resized: run again
      s = enqueue_batch(sched.get(), w.ws, w.stream, w.plan, w.opts, false, w.state);
      if (s == SDFB_OK) {
        enqueue_readback(w);
        s = finish_batch(sched.get(), w.ws, w.stream, w.state, w.plan, nullptr);
      }
    }
    if (s == SDFB_OK)
      for (size_t k = 0; k < w.reqs.size(); ++k) {
        Request *r = w.reqs[k];
        const uint64_t n = uint64_t(r->grid.nx) * r->grid.ny * r->grid.nz;
        if (r->dist_out && !r->dist_pinned)
          std::memcpy(r->dist_out, static_cast<float *>(w.stage_dist.p) + w.offs[k], n * 4);
        if (r->occ_out && !r->occ_pinned)
          std::memcpy(r->occ_out, static_cast<uint8_t *>(w.stage_occ.p) + w.offs[k], n);
      }
  }
  const double t = now_ms();
  std::lock_guard<std::mutex> g(mu);
  for (Request *r : w.reqs) {
    if (r->status < 0) r->status = s;
    r->t_done = t;
    r->done = true;
    static_cast<Resident *>(r->res)->refs--;
  }
  inflight -= static_cast<int>(w.reqs.size());
  inflight_bytes -= w.bytes;
  w.bytes = 0;
  w.reqs.clear();
  w.busy = false;
  cv_done.notify_all();
}

void sdfb_server::run() {
  cudaSetDevice(device);
  for (;;) {
    // retire finished waves (their event has completed)
    for (auto &wp : waves) {
      Wave &w = *wp;
      if (!w.busy) continue;
      const cudaError_t q = cudaEventQuery(w.done);
      if (q == cudaSuccess) {
        retire_wave(w);
      } else if (q != cudaErrorNotReady) {
        // the context has failed: complete the wave's requests with an error, do not wait
        cudaGetLastError();
        {
          std::lock_guard<std::mutex> g(mu);
          for (Request *r : w.reqs)
            if (r->status < 0) r->status = SDFB_ERR_CUDA;
        }
        retire_wave(w);
      }
    }
    Wave *free_slot = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (stop && pending.empty() && inflight == 0) break;
      for (auto &wp : waves)
        if (!wp->busy) {
          free_slot = wp.get();
          break;
        }
      if (free_slot && !pending.empty()) {
        // admit queued requests in arrival order while the wave and the budget hold
        uint64_t cells = 0;
        while (!pending.empty() && inflight < max_inflight) {
          Request *r = pending.front();
          const uint64_t n = uint64_t(r->grid.nx) * r->grid.ny * r->grid.nz;
          const uint64_t bytes = n * ((r->dist_out ? 4 : 0) + (r->occ_out ? 1 : 0)) + n / 4;
          if (!free_slot->reqs.empty() && (cells + n > wave_cells)) break;
          // Room for the outputs: evict unreferenced meshes if needed. When nothing is in flight
          // the request is admitted even over the budget, so the queue always makes progress.
          if (resident_bytes_used + inflight_bytes + bytes > budget && !make_room(bytes) && inflight > 0) break;
          pending.pop_front();
          r->t_admit = now_ms();
          free_slot->reqs.push_back(r);
          free_slot->bytes += bytes;
          inflight_bytes += bytes;
          inflight++;
          cells += n;
        }
        if (!free_slot->reqs.empty()) {
          free_slot->busy = true;
          free_slot->lean = std::any_of(reg_busy.begin(), reg_busy.end(), [](char b) { return b != 0; });
        } else {
          free_slot = nullptr;
        }
      } else {
        free_slot = nullptr;
      }
      if (!free_slot) {
        const bool any_busy = std::any_of(waves.begin(), waves.end(), [](const std::unique_ptr<Wave> &w) { return w->busy; });
        if (!any_busy) {
          cv_work.wait_for(lk, std::chrono::milliseconds(2));
          continue;
        }
      }
    }
    if (free_slot) {
      if (!launch_wave(*free_slot)) {
        std::lock_guard<std::mutex> g(mu);
        for (Request *r : free_slot->reqs) r->status = SDFB_ERR_OUT_OF_MEMORY;
      }
      continue;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

extern "C" {

sdfb_status sdfb_server_create(sdfb_ctx *ctx, const sdfb_server_opts *opts, sdfb_server **out) {
  if (!ctx || !out) return SDFB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  auto srv = std::make_unique<sdfb_server>();
  srv->device = ctx->device;
  sdfb_server_opts o;
  std::memset(&o, 0, sizeof o);
  if (opts) std::memcpy(&o, opts, std::min<size_t>(sizeof o, opts->struct_size ? opts->struct_size : sizeof o));
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  srv->budget = o.hbm_budget_bytes ? o.hbm_budget_bytes : uint64_t(free_b) * 3 / 4;
  // Defaults measured on GB300 with every mesh resident, closed loop: 64 jobs in flight and waves
  // of 2^27 voxels 973 M voxels/s; 128 and 2^28 1042 M (fuller waves, fewer tails).
  srv->max_inflight = o.max_inflight > 0 ? o.max_inflight : 128;
  srv->wave_cells = 1ull << (o.wave_voxels_log2 > 10 && o.wave_voxels_log2 < 36 ? o.wave_voxels_log2 : 28);
  srv->all_sms = ctx->num_sms;
  srv->sched = make_private_ctx(ctx->device, ctx->num_sms, ctx);
  if (!srv->sched) return SDFB_ERR_CUDA;
  for (int k = 0; k < kRegSlots; ++k) {
    srv->regs.push_back(make_private_ctx(ctx->device, ctx->num_sms, ctx, true));
    if (!srv->regs.back()) return SDFB_ERR_CUDA;
  }
  srv->reg_busy.assign(kRegSlots, 0);
  // keep freed device memory in the stream-ordered pool for reuse
  if (cudaDeviceGetDefaultMemPool(&srv->pool, ctx->device) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  const int slots = 3;
  for (int i = 0; i < slots; ++i) {
    auto w = std::make_unique<Wave>();
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->done, cudaEventDisableTiming) != cudaSuccess || !w->ws.init())
      return SDFB_ERR_CUDA;
    srv->waves.push_back(std::move(w));
  }
  sdfb_server *raw = srv.release();
  raw->thread = std::thread([raw] { raw->run(); });
  *out = raw;
  return SDFB_OK;
}

void sdfb_server_destroy(sdfb_server *srv) {
  if (!srv) return;
  {
    // requests not yet admitted are cancelled; waves in flight finish
    std::lock_guard<std::mutex> g(srv->mu);
    srv->stop = true;
    const double t = now_ms();
    for (Request *r : srv->pending) {
      r->status = SDFB_ERR_BUSY;
      r->t_done = t;
      r->done = true;
      static_cast<Resident *>(r->res)->refs--;
    }
    srv->pending.clear();
  }
  srv->cv_done.notify_all();
  srv->cv_work.notify_all();
  if (srv->thread.joinable()) srv->thread.join();
  cudaSetDevice(srv->device);
  for (auto &kv : srv->meshes) srv->free_resident(*kv.second, srv->sched->stream);
  cudaStreamSynchronize(srv->sched->stream);
  for (auto &w : srv->waves) {
    cudaStreamSynchronize(w->stream);
    if (w->done) cudaEventDestroy(w->done);
    if (w->stream) cudaStreamDestroy(w->stream);
  }
  delete srv;
}

const char *sdfb_server_last_error(const sdfb_server *srv) {
  if (!srv) return "null server";
  // a copy per calling thread: other threads may set a new error meanwhile
  thread_local std::string copy;
  {
    std::lock_guard<std::mutex> g(const_cast<sdfb_server *>(srv)->err_mu);
    copy = srv->err;
  }
  return copy.c_str();
}

sdfb_status sdfb_mesh_register(sdfb_server *srv, const float *verts, uint32_t num_verts, const uint32_t *idx,
                               uint32_t num_tris, uint64_t *mesh_id) {
  if (!srv || !verts || !idx || !mesh_id) return SDFB_ERR_INVALID_ARGUMENT;
  if (num_tris == 0 || num_verts == 0) return srv->fail(SDFB_ERR_BAD_MESH, "mesh has no triangles");
  for (size_t k = 0; k < size_t(num_tris) * 3; ++k)
    if (idx[k] >= num_verts) return srv->fail(SDFB_ERR_BAD_MESH, "triangle index out of range");
  Hash2 hh;
  const uint32_t counts[2] = {num_verts, num_tris};
  content_hash(counts, sizeof counts, hh);
  content_hash(verts, size_t(num_verts) * 12, hh);
  content_hash(idx, size_t(num_tris) * 12, hh);
  uint64_t h = avalanche(hh.a);
  const uint64_t check = avalanche(hh.b);
  // A cache hit (same id, second hash and counts) returns at once. An id held by other contents
  // moves this mesh on to the next id in a fixed probe sequence. Otherwise this thread takes a free
  // registration slot and builds the mesh, unless another thread is already building under the
  // same id: then it waits for that build and looks again (a second build would replace a
  // Resident that queued requests may point to).
  int slot = -1;
  {
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
      auto it = srv->meshes.find(h);
      if (it != srv->meshes.end()) {
        const Resident &m = *it->second;
        if (m.check == check && m.V == num_verts && m.T == num_tris) {
          it->second->last_use = ++srv->tick;
          *mesh_id = h;
          return SDFB_OK;
        }
        h = avalanche(h + 0x9e3779b97f4a7c15ull);  // another mesh holds this id
        continue;
      }
      if (!srv->building.count(h)) {
        for (size_t k = 0; k < srv->reg_busy.size(); ++k)
          if (!srv->reg_busy[k]) {
            slot = static_cast<int>(k);
            break;
          }
        if (slot >= 0) break;
      }
      srv->cv_reg.wait(lk);
    }
    srv->reg_busy[slot] = 1;
    srv->building.insert(h);
  }
  struct SlotRelease {
    sdfb_server *s;
    int slot;
    uint64_t h;
    ~SlotRelease() {
      {
        std::lock_guard<std::mutex> g(s->mu);
        s->reg_busy[slot] = 0;
        s->building.erase(h);
      }
      s->cv_reg.notify_all();
    }
  } release{srv, slot, h};
  sdfb_ctx *rc = srv->regs[slot].get();
  cudaSetDevice(srv->device);
  auto r = std::make_unique<Resident>();
  r->id = h;
  r->check = check;
  *mesh_id = h;
  r->V = num_verts;
  r->T = num_tris;
  const size_t bvh_bytes = resident_bytes(num_tris, false);
  r->bytes = size_t(num_verts) * 12 + size_t(num_tris) * 12 + bvh_bytes;
  {
    std::lock_guard<std::mutex> g(srv->mu);
    if (!srv->make_room(r->bytes))
      return srv->fail(SDFB_ERR_OUT_OF_MEMORY, "mesh does not fit the HBM budget next to in-flight work");
    srv->resident_bytes_used += r->bytes;  // reserved now, released on failure
  }
  cudaStream_t st = rc->stream;
  auto undo = [&](sdfb_status s, const std::string &m) {
    srv->free_resident(*r, st);
    cudaStreamSynchronize(st);
    std::lock_guard<std::mutex> g(srv->mu);
    srv->resident_bytes_used -= r->bytes;
    return srv->fail(s, m);
  };
  if (!async_alloc(r->verts, size_t(num_verts) * 12, st) || !async_alloc(r->idx, size_t(num_tris) * 12, st) ||
      !async_alloc(r->bvh, bvh_bytes, st))
    return undo(SDFB_ERR_OUT_OF_MEMORY, "device allocation failed");
  cudaMemcpyAsync(r->verts.p, verts, size_t(num_verts) * 12, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(r->idx.p, idx, size_t(num_tris) * 12, cudaMemcpyHostToDevice, st);
  // the weld + watertight gate on the device decides the sign mode
  sdfb_opts auto_opts;
  std::memset(&auto_opts, 0, sizeof auto_opts);
  auto_opts.sign_mode = SDFB_SIGN_AUTO;
  int sign = kSignParity, watertight = -1;
  const sdfb_status gs = device_sign(rc, auto_opts, static_cast<const float *>(r->verts.p), num_verts,
                                     static_cast<const uint32_t *>(r->idx.p), num_tris, st, &sign, &watertight);
  if (gs != SDFB_OK) return undo(gs, rc->err);
  r->sign = sign;
  r->watertight = watertight;
  size_t cap_bytes = 0;
  if (r->sign == kSignGwn) {
    // caps built on the device in the registration slot's buffers, then copied to exact-size
    // resident buffers
    std::vector<PlanMesh> cm(1);
    cm[0].verts = static_cast<const float *>(r->verts.p);
    cm[0].idx = static_cast<const uint32_t *>(r->idx.p);
    cm[0].V = num_verts;
    cm[0].T = num_tris;
    cm[0].sign = kSignGwn;
    const sdfb_status cs = device_caps(rc, st, cm, true);
    if (cs != SDFB_OK) return undo(cs, rc->err);
    r->pV = cm[0].pV;
    r->pT = cm[0].pT;
    r->cT = cm[0].cT;
    cap_bytes = r->cT ? resident_bytes(r->cT, true) : 0;
    const uint64_t extra = cap_bytes + uint64_t(r->pV) * 12 + uint64_t(r->pT) * 12 + uint64_t(r->cT) * 12;
    {
      std::lock_guard<std::mutex> g(srv->mu);
      if (!srv->make_room(extra)) {
        srv->free_resident(*r, st);
        cudaStreamSynchronize(st);
        srv->resident_bytes_used -= r->bytes;
        return srv->fail(SDFB_ERR_OUT_OF_MEMORY, "mesh does not fit the HBM budget next to in-flight work");
      }
      srv->resident_bytes_used += extra;
      r->bytes += extra;
    }
    if (!async_alloc(r->pverts, size_t(r->pV) * 12, st) || !async_alloc(r->pidx, size_t(r->pT) * 12, st) ||
        !async_alloc(r->cidx, std::max<size_t>(r->cT, 1) * 12, st) || (cap_bytes && !async_alloc(r->caps, cap_bytes, st)))
      return undo(SDFB_ERR_OUT_OF_MEMORY, "device allocation failed");
    cudaMemcpyAsync(r->pverts.p, cm[0].pverts, size_t(r->pV) * 12, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(r->pidx.p, cm[0].pidx, size_t(r->pT) * 12, cudaMemcpyDeviceToDevice, st);
    if (r->cT) cudaMemcpyAsync(r->cidx.p, cm[0].cidx, size_t(r->cT) * 12, cudaMemcpyDeviceToDevice, st);
  }
  PlanMesh p;
  p.verts = static_cast<const float *>(r->verts.p);
  p.idx = static_cast<const uint32_t *>(r->idx.p);
  p.V = num_verts;
  p.T = num_tris;
  p.cverts = static_cast<const float *>(r->pverts.p);
  p.cidx = static_cast<const uint32_t *>(r->cidx.p);
  p.pV = r->pV;
  p.cT = r->cT;
  p.grid.nx = p.grid.ny = p.grid.nz = 256;  // leaf size is tuned for a typical grid
  const sdfb_status s = build_resident(rc, rc->ws, st, p, r->bvh.p, r->tree, r->caps.p, r->cap_tree);
  if (s != SDFB_OK) return undo(s, rc->err);
  std::lock_guard<std::mutex> g(srv->mu);
  r->last_use = ++srv->tick;
  srv->meshes.emplace(h, std::move(r));  // h was in `building`, so no other thread inserted it
  return SDFB_OK;
}

sdfb_status sdfb_submit(sdfb_server *srv, uint64_t mesh_id, const sdfb_grid_desc *grid, const sdfb_opts *opts,
                        float *dist_out, uint8_t *occ_out, uint64_t *request_id) {
  if (!srv || !request_id || !grid_ok(grid)) return SDFB_ERR_INVALID_ARGUMENT;
  if (!dist_out && !occ_out) return srv->fail(SDFB_ERR_INVALID_ARGUMENT, "no output requested");
  auto r = std::make_unique<Request>();
  r->mesh = mesh_id;
  r->grid = *grid;
  r->opts = opts_or_default(opts);
  r->dist_out = r->opts.no_distance ? nullptr : dist_out;
  r->occ_out = r->opts.no_occupancy ? nullptr : occ_out;
  r->dist_pinned = is_pinned(r->dist_out);
  r->occ_pinned = is_pinned(r->occ_out);
  r->t_submit = now_ms();
  r->voxels = uint64_t(grid->nx) * grid->ny * grid->nz;
  {
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->meshes.find(mesh_id);
    if (it == srv->meshes.end()) return srv->fail(SDFB_ERR_NOT_FOUND, "mesh is not registered (or was evicted)");
    it->second->refs++;
    it->second->last_use = ++srv->tick;
    r->res = it->second.get();
    r->was_resident = 1;
    r->id = srv->next_req++;
    *request_id = r->id;
    srv->pending.push_back(r.get());
    srv->reqs[r->id] = std::move(r);
  }
  srv->cv_work.notify_one();
  return SDFB_OK;
}

sdfb_status sdfb_poll(sdfb_server *srv, uint64_t request_id, int32_t timeout_ms, int32_t *done,
                      sdfb_request_info *info) {
  if (!srv || !done) return SDFB_ERR_INVALID_ARGUMENT;
  *done = 0;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->reqs.find(request_id);
  if (it == srv->reqs.end()) return SDFB_ERR_NOT_FOUND;
  Request *r = it->second.get();
  if (!r->done) {
    if (timeout_ms < 0) {
      srv->cv_done.wait(lk, [&] { return r->done; });
    } else if (timeout_ms > 0) {
      srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; });
    }
  }
  if (!r->done) return SDFB_OK;
  *done = 1;
  if (info) {
    sdfb_request_info x;
    std::memset(&x, 0, sizeof x);
    x.struct_size = sizeof x;
    x.status = r->status;
    x.t_submit_ms = r->t_submit;
    x.t_admit_ms = r->t_admit;
    x.t_done_ms = r->t_done;
    x.voxels = r->voxels;
    x.mesh_was_resident = r->was_resident;
    std::memcpy(info, &x, std::min<size_t>(info->struct_size ? info->struct_size : sizeof x, sizeof x));
  }
  const sdfb_status st = static_cast<sdfb_status>(r->status);
  srv->reqs.erase(it);
  return st == SDFB_OK ? SDFB_OK : st;
}

}  // extern "C"
