// serve.cu -- continuously batched build+trace serving (no reference counterpart).
//
// Requests (a host mesh, host rays, host hit buffers) are queued by bvh_serve_submit; a scheduler
// thread admits them oldest first and overlaps their work on the GPU.  Two modes:
//
// * Batched ticks (BVH_SERVE_BATCHED): whenever a batch slot is free, every waiting request that
//   fits (up to the per-batch request and triangle limits and the HBM budget) joins one batch,
//   which runs as one launch sequence on the slot's stream: one gather kernel pulls all meshes
//   and rays straight from the callers' buffers (page-locked, or any host memory on systems where
//   the GPU reads pageable memory; other buffers are copied with cudaMemcpyAsync), one batched
//   LBVH-30 build (batched.cu) builds every mesh, one traversal launch traces every request's
//   rays against its own tree (trace.cu, k_trace_seg), one scatter kernel writes every request's
//   hits back.  Requests that arrive meanwhile form the next batch on another slot.
// * Per-request slots (default): each admitted request runs alone on a slot's stream: upload,
//   LBVH build (30, 60 or 63-bit codes), traversal, download.
//
// A request's result does not depend on what else is in flight: the batched build gives every
// mesh exactly its single build, and each ray is traced against its own request's tree.
//
// Memory: every slot holds device buffers sized for the largest work it has run.  Admission
// keeps the sum of what all slots hold (busy or idle) within hbm_budget_bytes: a slot that must
// grow first takes memory back from idle slots, and waits when that is not enough.
#include <algorithm>
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

// Device bytes of an LBVH workspace for cap triangles (workspace_reserve's allocations).
uint64_t ws_bytes(uint64_t cap) {
  if (!cap) return 0;
  cap = std::max<uint64_t>(cap, 1024);
  return cap * (8 * 2 + 4 * 2 + sizeof(Box) + 2 * sizeof(Node) + 8 + 1) + 16 + scratch_layout((uint32_t)cap).total * 4;
}

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Workspace ws;
  float* mesh = nullptr;  // 9 SoA arrays, stride tri_cap
  size_t tri_cap = 0;
  float* rays = nullptr;  // 6 arrays, stride ray_cap
  void* hits = nullptr;   // t, prim, visited, aabb, tri (stride ray_cap)
  size_t ray_cap = 0;
  // batched slots: per-batch metadata (pinned staging and device copy), mesh boxes, indices
  uint32_t* h_meta = nullptr;
  uint32_t* d_meta = nullptr;
  size_t meta_cap = 0;  // words
  float* mbox = nullptr;
  uint32_t count_cap = 0;
  uint32_t* indices = nullptr;
  size_t idx_cap = 0;
  uint32_t* h_status = nullptr;  // pinned: the build's device status word, read at completion
  bool busy = false;
  std::vector<Pending> reqs;  // the request (per-request slot) or the batch
  uint64_t t_admit = 0;

  uint64_t held() const {
    return 36ull * tri_cap + ws_bytes(ws.cap_n) + 44ull * ray_cap + 4ull * meta_cap + 32ull * count_cap +
           4ull * idx_cap;
  }
};

}  // namespace

struct bvh_server {
  bvh_serve_config cfg;
  bool batched = false;
  uint32_t max_batch_requests = 64, max_batch_triangles = 8u << 20;
  bool pageable_access = false;  // the device reads pageable host memory (no copy needed)
  std::vector<Slot> slots;
  std::deque<Pending> queue;
  std::deque<bvh_serve_result> done;
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool stop = false;
  bvh_serve_stats stats{};
  bvh_status fatal = BVH_OK;
};

// Device bytes a slot needs for n triangles, nr rays and (batched) count meshes.
static uint64_t need_bytes(const bvh_server* sv, uint64_t n, uint64_t nr, uint64_t count) {
  n = (n + 3) & ~3ull;  // as grow() rounds the mesh and ray arrays
  nr = (nr + 3) & ~3ull;
  uint64_t b = 36 * n + ws_bytes(n) + 44 * nr;
  if (sv->batched) b += 4 * n + 32 * count + 4 * (64 + 16 * count + 6 * 20 * count + n / 4096);
  return b;
}

static uint64_t held_total(const bvh_server* sv) {
  uint64_t t = 0;
  for (const Slot& s : sv->slots) t += s.held();
  return t;
}

static void free_buffers(Slot& s) {
  if (s.stream) cudaStreamSynchronize(s.stream);
  workspace_free(s.ws);
  s.ws = Workspace();
  cudaFree(s.mesh); cudaFree(s.rays); cudaFree(s.hits);
  cudaFree(s.d_meta); cudaFreeHost(s.h_meta); cudaFree(s.mbox); cudaFree(s.indices);
  s.mesh = nullptr; s.rays = nullptr; s.hits = nullptr; s.d_meta = nullptr; s.h_meta = nullptr;
  s.mbox = nullptr; s.indices = nullptr;
  s.tri_cap = s.ray_cap = s.meta_cap = s.idx_cap = 0;
  s.count_cap = 0;
}

// Room for `need` bytes in slot s within the budget, taking buffers back from idle slots first.
static bool make_room(bvh_server* sv, Slot& s, uint64_t need) {
  const uint64_t budget = sv->cfg.hbm_budget_bytes;
  auto projected = [&] { return held_total(sv) - s.held() + std::max(s.held(), need); };
  if (projected() <= budget) return true;
  for (Slot& o : sv->slots) {
    if (&o == &s || o.busy || o.held() == 0) continue;
    free_buffers(o);
    if (projected() <= budget) return true;
  }
  return false;
}

static cudaError_t grow(bvh_server* sv, Slot& s, uint32_t n, uint32_t nr, uint32_t count, size_t meta_words) {
  cudaError_t e = cudaSuccess;
  if (n > s.tri_cap) {
    cudaFree(s.mesh);
    s.mesh = nullptr;
    s.tri_cap = 0;
    const size_t cap = ((size_t)n + 3) & ~size_t(3);
    if ((e = cudaMalloc(&s.mesh, cap * 9 * 4)) != cudaSuccess) return e;
    s.tri_cap = cap;
  }
  if (nr > s.ray_cap) {
    cudaFree(s.rays);
    cudaFree(s.hits);
    s.rays = nullptr;
    s.hits = nullptr;
    s.ray_cap = 0;
    const size_t cap = ((size_t)nr + 3) & ~size_t(3);
    if ((e = cudaMalloc(&s.rays, cap * 6 * 4)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&s.hits, cap * 5 * 4)) != cudaSuccess) return e;
    s.ray_cap = cap;
  }
  if (sv->batched) {
    if (meta_words > s.meta_cap) {
      cudaFree(s.d_meta);
      cudaFreeHost(s.h_meta);
      s.d_meta = nullptr;
      s.h_meta = nullptr;
      s.meta_cap = 0;
      if ((e = cudaMalloc(&s.d_meta, meta_words * 4)) != cudaSuccess) return e;
      if ((e = cudaMallocHost(&s.h_meta, meta_words * 4)) != cudaSuccess) return e;
      s.meta_cap = meta_words;
    }
    if (count > s.count_cap) {
      cudaFree(s.mbox);
      s.mbox = nullptr;
      s.count_cap = 0;
      if ((e = cudaMalloc(&s.mbox, (size_t)count * 32)) != cudaSuccess) return e;
      s.count_cap = count;
    }
    if (n > s.idx_cap) {
      cudaFree(s.indices);
      s.indices = nullptr;
      s.idx_cap = 0;
      if ((e = cudaMalloc(&s.indices, (size_t)n * 4)) != cudaSuccess) return e;
      s.idx_cap = n;
    }
  }
  return workspace_reserve(s.ws, n, s.stream);
}

// May the device read this host pointer directly?  Page-locked (or registered) memory, or any
// host memory where the device reads pageable memory.  Returns the address the device uses.
static const void* device_view(const bvh_server* sv, const void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  if (a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeDevice) return p;
  return sv->pageable_access ? p : nullptr;
}

// ---- per-request slots -----------------------------------------------------------------------
static cudaError_t launch_one(bvh_server* sv, Slot& s) {
  const bvh_serve_request& r = s.reqs[0].req;
  const uint32_t n = r.mesh.n, nr = r.rays.n;
  cudaError_t e = grow(sv, s, n, nr, 1, 0);
  if (e != cudaSuccess) return e;
  const float* src[9] = {r.mesh.v0x, r.mesh.v0y, r.mesh.v0z, r.mesh.v1x, r.mesh.v1y,
                         r.mesh.v1z, r.mesh.v2x, r.mesh.v2y, r.mesh.v2z};
  MeshPtrs m;
  for (int k = 0; k < 9; ++k) {
    float* d = s.mesh + s.tri_cap * k;
    if ((e = cudaMemcpyAsync(d, src[k], (size_t)n * 4, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess) return e;
    m.v[k] = d;
  }
  const float* rsrc[6] = {r.rays.ox, r.rays.oy, r.rays.oz, r.rays.dx, r.rays.dy, r.rays.dz};
  RayPtrs rp;
  for (int k = 0; k < 6; ++k) {
    float* d = s.rays + s.ray_cap * k;
    if (nr && (e = cudaMemcpyAsync(d, rsrc[k], (size_t)nr * 4, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess)
      return e;
    (k < 3 ? rp.o[k] : rp.d[k - 3]) = d;
  }
  uint32_t* idx = nullptr;
  s.ws.sort_variant = default_sort_variant(n);
  if ((e = lbvh_build(s.ws, m, n, sv->cfg.morton_bits, 0, s.stream, nullptr, &idx)) != cudaSuccess) return e;
  float* ht = reinterpret_cast<float*>(s.hits);
  int32_t* hi = reinterpret_cast<int32_t*>(s.hits);
  HitOut ho{ht, hi + s.ray_cap, hi + 2 * s.ray_cap, hi + 3 * s.ray_cap, hi + 4 * s.ray_cap};
  if ((e = trace_rays(s.ws.nodes, (int)(2 * n - 1), m, n, rp, nr, ho, s.stream)) != cudaSuccess) return e;
  void* dst[5] = {r.hits.t, r.hits.prim, r.hits.nodes_visited, r.hits.aabb_tests, r.hits.tri_tests};
  for (int k = 0; k < 5; ++k)
    if (nr && dst[k] &&
        (e = cudaMemcpyAsync(dst[k], hi + (size_t)k * s.ray_cap, (size_t)nr * 4, cudaMemcpyDeviceToHost,
                             s.stream)) != cudaSuccess)
      return e;
  const ScratchLayout L = scratch_layout(s.ws.cap_n);
  if ((e = cudaMemcpyAsync(s.h_status, s.ws.scratch + L.status, 4, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess)
    return e;
  return cudaEventRecord(s.done, s.stream);
}

// ---- batched ticks ---------------------------------------------------------------------------
// Metadata words of a batch: offsets (count + 1), work items (4 words each), ray segments
// (4 words each, count + 1), gather and scatter descriptors (6 words each: 15 + 5 per request).
struct MetaLayout {
  size_t offsets, items, segs, gather, scatter, total;
};
static MetaLayout meta_layout(uint32_t count, uint32_t n_items) {
  MetaLayout L;
  size_t o = 0;
  L.offsets = o; o += count + 1;
  o = (o + 3) & ~size_t(3);
  L.items = o; o += 4 * (size_t)n_items;
  L.segs = o; o += 4 * ((size_t)count + 1);
  o = (o + 1) & ~size_t(1);  // 8-byte aligned descriptors
  L.gather = o; o += 6 * 15 * (size_t)count;
  L.scatter = o; o += 6 * 5 * (size_t)count;
  L.total = o;
  return L;
}

static uint32_t batch_items(const std::vector<Pending>& reqs) {
  uint64_t k = 0;
  for (const Pending& p : reqs) k += div_up(p.req.mesh.n, kSegChunk);
  return (uint32_t)k;
}

static cudaError_t launch_batch(bvh_server* sv, Slot& s) {
  const uint32_t count = (uint32_t)s.reqs.size();
  uint64_t n64 = 0, nr64 = 0;
  for (const Pending& p : s.reqs) {
    n64 += p.req.mesh.n;
    nr64 += p.req.rays.n;
  }
  const uint32_t n = (uint32_t)n64, nr = (uint32_t)nr64, n_items = batch_items(s.reqs);
  const MetaLayout ML = meta_layout(count, n_items);
  cudaError_t e = grow(sv, s, n, nr, count, ML.total);
  if (e != cudaSuccess) return e;
  uint32_t* h = s.h_meta;
  SegItem* items = reinterpret_cast<SegItem*>(h + ML.items);
  RaySeg* segs = reinterpret_cast<RaySeg*>(h + ML.segs);
  CopyDesc* gather = reinterpret_cast<CopyDesc*>(h + ML.gather);
  CopyDesc* scatter = reinterpret_cast<CopyDesc*>(h + ML.scatter);
  uint32_t ng = 0, nsc = 0, gpieces = 0, spieces = 0, it = 0;
  struct Fallback {
    const void* src;
    void* dst;
    size_t bytes;
  };
  std::vector<Fallback> h2d, d2h;
  uint32_t off = 0, roff = 0;
  float* hits_f = reinterpret_cast<float*>(s.hits);
  for (uint32_t m = 0; m < count; ++m) {
    const bvh_serve_request& r = s.reqs[m].req;
    const uint32_t nm = r.mesh.n, nrm = r.rays.n;
    h[ML.offsets + m] = off;
    for (uint32_t b = 0; b < nm; b += kSegChunk) items[it++] = SegItem{m, off + b, off + std::min(nm, b + kSegChunk), 0};
    segs[m] = RaySeg{roff, 2 * off - m, off, nm};
    const float* msrc[9] = {r.mesh.v0x, r.mesh.v0y, r.mesh.v0z, r.mesh.v1x, r.mesh.v1y,
                            r.mesh.v1z, r.mesh.v2x, r.mesh.v2y, r.mesh.v2z};
    const float* rsrc[6] = {r.rays.ox, r.rays.oy, r.rays.oz, r.rays.dx, r.rays.dy, r.rays.dz};
    for (int k = 0; k < 15; ++k) {
      const float* src = k < 9 ? msrc[k] : rsrc[k - 9];
      const uint32_t len = k < 9 ? nm : nrm;
      float* dst = k < 9 ? s.mesh + s.tri_cap * k + off : s.rays + s.ray_cap * (k - 9) + roff;
      if (!len) continue;
      const void* v = device_view(sv, src);
      if (v) {
        gather[ng++] = CopyDesc{static_cast<const float*>(v), dst, len, gpieces};
        gpieces += copy_pieces(len);
      } else {
        h2d.push_back(Fallback{src, dst, (size_t)len * 4});
      }
    }
    void* hdst[5] = {r.hits.t, r.hits.prim, r.hits.nodes_visited, r.hits.aabb_tests, r.hits.tri_tests};
    for (int k = 0; k < 5; ++k) {
      if (!nrm || !hdst[k]) continue;
      float* src = hits_f + s.ray_cap * k + roff;
      const void* v = device_view(sv, hdst[k]);
      if (v) {
        scatter[nsc++] = CopyDesc{src, static_cast<float*>(const_cast<void*>(v)), nrm, spieces};
        spieces += copy_pieces(nrm);
      } else {
        d2h.push_back(Fallback{src, hdst[k], (size_t)nrm * 4});
      }
    }
    off += nm;
    roff += nrm;
  }
  h[ML.offsets + count] = off;
  segs[count] = RaySeg{roff, 2 * off - count, off, 0};
  // one copy of the metadata, then the gather (and copies of what the device cannot read)
  if ((e = cudaMemcpyAsync(s.d_meta, h, ML.total * 4, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess) return e;
  const CopyDesc* d_gather = reinterpret_cast<const CopyDesc*>(s.d_meta + ML.gather);
  const CopyDesc* d_scatter = reinterpret_cast<const CopyDesc*>(s.d_meta + ML.scatter);
  if ((e = copy_many(d_gather, ng, gpieces, s.stream)) != cudaSuccess) return e;
  for (const Fallback& f : h2d)
    if ((e = cudaMemcpyAsync(f.dst, f.src, f.bytes, cudaMemcpyHostToDevice, s.stream)) != cudaSuccess) return e;
  MeshPtrs mp;
  for (int k = 0; k < 9; ++k) mp.v[k] = s.mesh + s.tri_cap * k;
  StageEvents none;
  s.ws.sort_variant = default_sort_variant(n);
  if ((e = batched_build(s.ws, mp, n, s.d_meta + ML.offsets, count,
                         reinterpret_cast<const SegItem*>(s.d_meta + ML.items), n_items, s.mbox, s.indices, s.stream,
                         &none)) != cudaSuccess)
    return e;
  RayPtrs rp;
  for (int k = 0; k < 3; ++k) {
    rp.o[k] = s.rays + s.ray_cap * k;
    rp.d[k] = s.rays + s.ray_cap * (3 + k);
  }
  int32_t* hi = reinterpret_cast<int32_t*>(s.hits);
  HitOut ho{hits_f, hi + s.ray_cap, hi + 2 * s.ray_cap, hi + 3 * s.ray_cap, hi + 4 * s.ray_cap};
  if ((e = trace_rays_batched(s.ws.nodes, mp, rp, nr, reinterpret_cast<const RaySeg*>(s.d_meta + ML.segs), count, ho,
                              s.stream)) != cudaSuccess)
    return e;
  if ((e = copy_many(d_scatter, nsc, spieces, s.stream)) != cudaSuccess) return e;
  for (const Fallback& f : d2h)
    if ((e = cudaMemcpyAsync(f.dst, f.src, f.bytes, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess) return e;
  const ScratchLayout L = scratch_layout(s.ws.cap_n);
  if ((e = cudaMemcpyAsync(s.h_status, s.ws.scratch + L.status, 4, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess)
    return e;
  return cudaEventRecord(s.done, s.stream);
}

// ---- scheduler -------------------------------------------------------------------------------
static void finish(bvh_server* sv, Slot& s, int32_t status) {
  const uint64_t t = now_ns();
  for (const Pending& p : s.reqs) {
    bvh_serve_result res{};
    res.tag = p.req.tag;
    res.status = status;
    res.t_submit_ns = p.t_submit;
    res.t_admit_ns = s.t_admit;
    res.t_done_ns = t;
    res.triangles = p.req.mesh.n;
    res.rays = p.req.rays.n;
    if (status == BVH_OK) {
      sv->stats.completed++;
      sv->stats.triangles += res.triangles;
      sv->stats.rays += res.rays;
    }
    sv->done.push_back(res);
  }
  s.reqs.clear();
  s.busy = false;
}

static void reject_front(bvh_server* sv) {
  bvh_serve_result res{};
  res.tag = sv->queue.front().req.tag;
  res.status = BVH_ERR_OUT_OF_MEMORY;
  res.t_submit_ns = sv->queue.front().t_submit;
  res.t_admit_ns = res.t_done_ns = now_ns();
  sv->queue.pop_front();
  sv->stats.rejected++;
  sv->done.push_back(res);
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
      const int32_t st = q != cudaSuccess                                           ? BVH_ERR_DEVICE
                         : (*s.h_status & (kStatusSortTimeout | kStatusClimbTimeout)) ? BVH_ERR_TIMEOUT
                         : *s.h_status                                              ? BVH_ERR_DEVICE
                                                                                    : BVH_OK;
      finish(sv, s, st);
      progressed = true;
    }
    // admissions: oldest first, while a slot is free and the budget allows
    while (!sv->queue.empty()) {
      Slot* fs = nullptr;
      for (Slot& s : sv->slots)
        if (!s.busy) { fs = &s; break; }
      if (!fs) break;
      Slot& s = *fs;
      const bvh_serve_request& front = sv->queue.front().req;
      if (need_bytes(sv, front.mesh.n, front.rays.n, 1) > sv->cfg.hbm_budget_bytes) {  // can never fit
        reject_front(sv);
        progressed = true;
        continue;
      }
      // the batch: the oldest requests that fit the per-batch limits and the budget together
      uint64_t n = 0, nr = 0;
      size_t take = 0;
      const size_t max_take = sv->batched ? sv->max_batch_requests : 1;
      while (take < sv->queue.size() && take < max_take) {
        const bvh_serve_request& r = sv->queue[take].req;
        const uint64_t n2 = n + r.mesh.n, nr2 = nr + r.rays.n;
        if (take > 0 && (n2 > sv->max_batch_triangles || nr2 > 0xffffffffull ||
                         need_bytes(sv, n2, nr2, take + 1) > sv->cfg.hbm_budget_bytes))
          break;
        n = n2;
        nr = nr2;
        ++take;
      }
      if (!make_room(sv, s, need_bytes(sv, n, nr, take))) {
        sv->stats.budget_waits++;
        break;
      }
      s.reqs.assign(sv->queue.begin(), sv->queue.begin() + (ptrdiff_t)take);
      sv->queue.erase(sv->queue.begin(), sv->queue.begin() + (ptrdiff_t)take);
      s.busy = true;
      s.t_admit = now_ns();
      sv->stats.admitted += take;
      lk.unlock();
      cudaError_t e = sv->batched ? launch_batch(sv, s) : launch_one(sv, s);
      if (e != cudaSuccess) cudaStreamSynchronize(s.stream);  // nothing may still read the callers' buffers
      lk.lock();
      const uint64_t held = held_total(sv);
      if (held > sv->stats.peak_in_flight_bytes) sv->stats.peak_in_flight_bytes = held;
      if (e != cudaSuccess) {
        sv->fatal = e == cudaErrorMemoryAllocation ? BVH_ERR_OUT_OF_MEMORY : BVH_ERR_DEVICE;
        cudaGetLastError();
        finish(sv, s, sv->fatal);
      }
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
    free_buffers(s);
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
  const bool batched = cfg->reserved[0] == BVH_SERVE_BATCHED;
  if (cfg->reserved[0] != 0 && !batched) return BVH_ERR_INVALID_ARG;
  if (batched && cfg->morton_bits != 30) return BVH_ERR_UNSUPPORTED;  // batched builds use 30-bit codes
  if (cfg->reserved[1] < 0 || cfg->reserved[2] < 0) return BVH_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || cfg->device < 0 || cfg->device >= count) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(cfg->device);
  if (prepare_kernels() != cudaSuccess) return BVH_ERR_DEVICE;
  bvh_server* sv = new bvh_server();
  sv->cfg = *cfg;
  sv->batched = batched;
  if (cfg->reserved[1] > 0) sv->max_batch_requests = (uint32_t)cfg->reserved[1];
  if (cfg->reserved[2] > 0) sv->max_batch_triangles = (uint32_t)cfg->reserved[2];
  int pageable = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, cfg->device) == cudaSuccess)
    sv->pageable_access = pageable != 0;
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
    // per-request slots: room for the largest request; batched slots: for a full batch of them
    // (growing later would free buffers, which synchronises the whole device mid-stream)
    uint64_t n = cfg->max_triangles ? cfg->max_triangles : 1024, nr = cfg->max_rays, count = 1;
    if (batched) {
      count = sv->max_batch_requests;
      n = std::min<uint64_t>(std::max<uint64_t>(n * count, 1024), std::max<uint64_t>(sv->max_batch_triangles, n));
      nr = std::min<uint64_t>(nr * count, 0xffffffffull);
    }
    for (Slot& s : sv->slots) {
      if (held_total(sv) + need_bytes(sv, n, nr, count) > cfg->hbm_budget_bytes) break;  // grow later
      if (grow(sv, s, (uint32_t)n, (uint32_t)nr, (uint32_t)count,
               meta_layout((uint32_t)count, (uint32_t)(count + n / kSegChunk)).total) != cudaSuccess) {
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
  out->in_flight_bytes = held_total(sv);
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
