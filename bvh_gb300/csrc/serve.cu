// serve.cu -- continuously batched build+trace serving (no reference counterpart).
//
// Requests (a host mesh, host rays, host hit buffers) are queued by bvh_serve_submit.  A
// scheduler thread admits the oldest waiting request as soon as a slot is free and its device
// memory estimate fits the HBM budget next to everything in flight; each slot owns a CUDA
// stream and a device workspace, so admitted requests overlap on the GPU.  A request runs:
// upload mesh + rays, LBVH build (bvh_gb300/csrc/lbvh.cu), closest-hit traversal
// (bvh_gb300/csrc/trace.cu), download hits; completion is detected with an event and the
// request's memory returns to the budget.  Results do not depend on what else is in flight:
// every request uses only its slot's buffers and the kernels are deterministic.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/bvh_gb300.h"
#include "lbvh.cuh"
#include "trace.cuh"

using namespace bvhgb;

namespace {

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Pending {
  bvh_serve_request req;
  uint64_t t_submit;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Workspace ws;
  float* mesh = nullptr;  // 9 SoA arrays, stride mesh_stride
  size_t mesh_stride = 0;
  float* rays = nullptr;  // 6 arrays, stride ray_stride
  size_t ray_stride = 0;
  void* hits = nullptr;   // t, prim, visited, aabb, tri (stride ray_stride)
  uint32_t* h_status = nullptr;  // pinned: the build's device status word, read at completion
  bool busy = false;
  Pending cur;
  uint64_t t_admit = 0, t_launch = 0, bytes = 0;
};

}  // namespace

struct bvh_server {
  bvh_serve_config cfg;
  std::vector<Slot> slots;
  std::deque<Pending> queue;
  std::deque<bvh_serve_result> done;
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool stop = false;
  uint64_t in_flight_bytes = 0;
  bvh_serve_stats stats{};
  bvh_status fatal = BVH_OK;
};

static uint64_t request_bytes(const bvh_serve_request& r) {
  const uint64_t n = r.mesh.n, nr = r.rays.n;
  // mesh copy + workspace (keys x2, values x2, boxes, nodes, slots, deltas) + rays + hits
  return 36 * n + n * (16 + 8 + 32 + 96 + 8 + 1) + 24 * nr + 20 * nr + (4u << 20);
}

static cudaError_t grow(Slot& s, uint32_t n, uint32_t nr) {
  cudaError_t e = cudaSuccess;
  const size_t ms = ((size_t)n + 3) & ~size_t(3);
  if (ms > s.mesh_stride) {
    cudaFree(s.mesh);
    s.mesh = nullptr;
    s.mesh_stride = 0;
    if ((e = cudaMalloc(&s.mesh, ms * 9 * 4)) != cudaSuccess) return e;
    s.mesh_stride = ms;
  }
  const size_t rs = ((size_t)nr + 3) & ~size_t(3);
  if (rs > s.ray_stride) {
    cudaFree(s.rays);
    cudaFree(s.hits);
    s.rays = nullptr;
    s.hits = nullptr;
    s.ray_stride = 0;
    if ((e = cudaMalloc(&s.rays, rs * 6 * 4)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.hits, rs * 5 * 4)) != cudaSuccess) return e;
    s.ray_stride = rs;
  }
  return workspace_reserve(s.ws, n, s.stream);
}

// Enqueue one request on its slot's stream (all asynchronous).
static cudaError_t launch(bvh_server* sv, Slot& s) {
  const bvh_serve_request& r = s.cur.req;
  const uint32_t n = r.mesh.n, nr = r.rays.n;
  cudaError_t e = grow(s, n, nr);
  if (e != cudaSuccess) return e;
  const float* src[9] = {r.mesh.v0x, r.mesh.v0y, r.mesh.v0z, r.mesh.v1x, r.mesh.v1y,
                         r.mesh.v1z, r.mesh.v2x, r.mesh.v2y, r.mesh.v2z};
  MeshPtrs m;
  for (int k = 0; k < 9; ++k) {
    float* d = s.mesh + s.mesh_stride * k;
    if ((e = cudaMemcpyAsync(d, src[k], (size_t)n * 4, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess) return e;
    m.v[k] = d;
  }
  const float* rsrc[6] = {r.rays.ox, r.rays.oy, r.rays.oz, r.rays.dx, r.rays.dy, r.rays.dz};
  RayPtrs rp;
  for (int k = 0; k < 6; ++k) {
    float* d = s.rays + s.ray_stride * k;
    if (nr && (e = cudaMemcpyAsync(d, rsrc[k], (size_t)nr * 4, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess)
      return e;
    (k < 3 ? rp.o[k] : rp.d[k - 3]) = d;
  }
  uint32_t* idx = nullptr;
  if ((e = lbvh_build(s.ws, m, n, sv->cfg.morton_bits, 0, s.stream, nullptr, &idx)) != cudaSuccess) return e;
  float* ht = reinterpret_cast<float*>(s.hits);
  int32_t* hi = reinterpret_cast<int32_t*>(s.hits);
  HitOut ho{ht, hi + s.ray_stride, hi + 2 * s.ray_stride, hi + 3 * s.ray_stride, hi + 4 * s.ray_stride};
  if ((e = trace_rays(s.ws.nodes, (int)(2 * n - 1), m, n, rp, nr, ho, s.stream)) != cudaSuccess) return e;
  void* dst[5] = {r.hits.t, r.hits.prim, r.hits.nodes_visited, r.hits.aabb_tests, r.hits.tri_tests};
  for (int k = 0; k < 5; ++k)
    if (nr && dst[k] &&
        (e = cudaMemcpyAsync(dst[k], hi + (size_t)k * s.ray_stride, (size_t)nr * 4, cudaMemcpyDeviceToHost,
                             s.stream)) != cudaSuccess)
      return e;
  const ScratchLayout L = scratch_layout(s.ws.cap_n);
  if ((e = cudaMemcpyAsync(s.h_status, s.ws.scratch + L.status, 4, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess)
    return e;
  return cudaEventRecord(s.done, s.stream);
}

static void run(bvh_server* sv) {
  cudaSetDevice(sv->cfg.device);
  std::unique_lock<std::mutex> lk(sv->mu);
  while (true) {
    bool progressed = false;
    // completions
    for (Slot& s : sv->slots) {
      if (!s.busy) continue;
      cudaError_t q = cudaEventQuery(s.done);
      if (q == cudaErrorNotReady) continue;
      bvh_serve_result res{};
      res.tag = s.cur.req.tag;
      res.status = q != cudaSuccess                                      ? BVH_ERR_DEVICE
                   : (*s.h_status & (kStatusSortTimeout | kStatusClimbTimeout)) ? BVH_ERR_TIMEOUT
                   : *s.h_status                                             ? BVH_ERR_DEVICE
                                                                             : BVH_OK;
      res.t_submit_ns = s.cur.t_submit;
      res.t_admit_ns = s.t_admit;
      res.t_done_ns = now_ns();
      res.triangles = s.cur.req.mesh.n;
      res.rays = s.cur.req.rays.n;
      sv->in_flight_bytes -= s.bytes;
      s.busy = false;
      sv->stats.completed++;
      sv->stats.triangles += res.triangles;
      sv->stats.rays += res.rays;
      sv->done.push_back(res);
      progressed = true;
    }
    // admissions: oldest first, while a slot is free and the budget allows
    while (!sv->queue.empty()) {
      Slot* free_slot = nullptr;
      for (Slot& s : sv->slots)
        if (!s.busy) { free_slot = &s; break; }
      if (!free_slot) break;
      const uint64_t need = request_bytes(sv->queue.front().req);
      if (need > sv->cfg.hbm_budget_bytes) {  // can never fit: reject
        bvh_serve_result res{};
        res.tag = sv->queue.front().req.tag;
        res.status = BVH_ERR_OUT_OF_MEMORY;
        res.t_submit_ns = sv->queue.front().t_submit;
        res.t_admit_ns = res.t_done_ns = now_ns();
        sv->queue.pop_front();
        sv->stats.rejected++;
        sv->done.push_back(res);
        progressed = true;
        continue;
      }
      if (sv->in_flight_bytes + need > sv->cfg.hbm_budget_bytes) {
        sv->stats.budget_waits++;
        break;
      }
      Slot& s = *free_slot;
      s.cur = sv->queue.front();
      sv->queue.pop_front();
      s.busy = true;
      s.bytes = need;
      s.t_admit = now_ns();
      sv->in_flight_bytes += need;
      if (sv->in_flight_bytes > sv->stats.peak_in_flight_bytes) sv->stats.peak_in_flight_bytes = sv->in_flight_bytes;
      lk.unlock();
      cudaError_t e = launch(sv, s);
      lk.lock();
      if (e != cudaSuccess) {
        sv->fatal = e == cudaErrorMemoryAllocation ? BVH_ERR_OUT_OF_MEMORY : BVH_ERR_DEVICE;
        bvh_serve_result res{};
        res.tag = s.cur.req.tag;
        res.status = sv->fatal;
        res.t_submit_ns = s.cur.t_submit;
        res.t_admit_ns = s.t_admit;
        res.t_done_ns = now_ns();
        sv->in_flight_bytes -= s.bytes;
        s.busy = false;
        sv->done.push_back(res);
      }
      sv->stats.admitted++;
      progressed = true;
    }
    if (progressed) sv->cv.notify_all();
    bool any_busy = false;
    for (Slot& s : sv->slots) any_busy |= s.busy;
    if (sv->stop && !any_busy && sv->queue.empty()) break;
    if (!progressed) {
      if (any_busy) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
        lk.lock();
      } else {
        sv->cv.wait_for(lk, std::chrono::milliseconds(5));
      }
    }
  }
}

// Frees every slot's stream, event and buffers (after its queued work has finished).
static void release_slots(bvh_server* sv) {
  for (Slot& s : sv->slots) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    workspace_free(s.ws);
    cudaFree(s.mesh);
    cudaFree(s.rays);
    cudaFree(s.hits);
    cudaFreeHost(s.h_status);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
    s = Slot();
  }
}

extern "C" bvh_serve_config bvh_serve_default_config(void) {
  bvh_serve_config c;
  memset(&c, 0, sizeof(c));
  c.hbm_budget_bytes = 40ull << 30;
  c.slots = 8;
  c.morton_bits = 30;
  c.device = 0;
  return c;
}

extern "C" bvh_status bvh_serve_open(const bvh_serve_config* cfg, bvh_server** out) {
  if (!cfg || !out || cfg->slots < 1 || cfg->slots > 256 || cfg->hbm_budget_bytes == 0) return BVH_ERR_INVALID_ARG;
  if (cfg->morton_bits != 30 && cfg->morton_bits != 60 && cfg->morton_bits != 63) return BVH_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || cfg->device < 0 || cfg->device >= count) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(cfg->device);
  if (prepare_kernels() != cudaSuccess) return BVH_ERR_DEVICE;
  bvh_server* sv = new bvh_server();
  sv->cfg = *cfg;
  sv->slots.resize(cfg->slots);
  for (Slot& s : sv->slots) {
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&s.h_status, 64) != cudaSuccess) {
      release_slots(sv);
      delete sv;
      return BVH_ERR_DEVICE;
    }
  }
  if (cfg->max_triangles || cfg->max_rays) {
    for (Slot& s : sv->slots) {
      if (grow(s, cfg->max_triangles ? cfg->max_triangles : 1024, cfg->max_rays) != cudaSuccess) {
        release_slots(sv);
        delete sv;
        return BVH_ERR_OUT_OF_MEMORY;
      }
    }
  }
  sv->worker = std::thread(run, sv);
  *out = sv;
  return BVH_OK;
}

extern "C" bvh_status bvh_serve_submit(bvh_server* sv, const bvh_serve_request* req) {
  if (!sv || !req) return BVH_ERR_INVALID_ARG;
  const bvh_mesh_soa& m = req->mesh;
  if (m.n == 0 || m.n > (1u << 30) - 1 || !m.v0x || !m.v0y || !m.v0z || !m.v1x || !m.v1y || !m.v1z || !m.v2x ||
      !m.v2y || !m.v2z)
    return BVH_ERR_INVALID_ARG;
  if (req->rays.n && (!req->rays.ox || !req->rays.oy || !req->rays.oz || !req->rays.dx || !req->rays.dy ||
                      !req->rays.dz))
    return BVH_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->stop) return BVH_ERR_INVALID_ARG;
  sv->queue.push_back(Pending{*req, now_ns()});
  sv->stats.submitted++;
  sv->cv.notify_all();
  return BVH_OK;
}

extern "C" int32_t bvh_serve_poll(bvh_server* sv, bvh_serve_result* out, int32_t max_results, int32_t wait_ms) {
  if (!sv || !out || max_results <= 0) return 0;
  std::unique_lock<std::mutex> lk(sv->mu);
  if (sv->done.empty() && wait_ms > 0)
    sv->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !sv->done.empty(); });
  int32_t k = 0;
  while (k < max_results && !sv->done.empty()) {
    out[k++] = sv->done.front();
    sv->done.pop_front();
  }
  return k;
}

extern "C" bvh_status bvh_serve_stats_get(bvh_server* sv, bvh_serve_stats* out) {
  if (!sv || !out) return BVH_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(sv->mu);
  *out = sv->stats;
  out->in_flight_bytes = sv->in_flight_bytes;
  out->queued = (uint64_t)sv->queue.size();
  return sv->fatal;
}

extern "C" bvh_status bvh_serve_close(bvh_server* sv) {
  if (!sv) return BVH_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
    sv->cv.notify_all();
  }
  if (sv->worker.joinable()) sv->worker.join();
  cudaSetDevice(sv->cfg.device);
  release_slots(sv);
  bvh_status f = sv->fatal;
  delete sv;
  return f;
}
