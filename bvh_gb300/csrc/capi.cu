// capi.cu -- the C ABI (include/bvh_gb300.h): contexts, builds, timing, traversal.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/bvh_gb300.h"
#include "lbvh.cuh"
#include "trace.cuh"

using namespace bvhgb;

struct BatchGraph {
  cudaGraphExec_t exec = nullptr;
  const float* ptrs[9] = {};
  uint32_t n = 0, count = 0;
  int32_t algo = -1, radius = 0, max_iter = 0, sort_variant = -1;
  uint32_t shape = 0;
  std::vector<uint32_t> offsets;
};

// Launch shapes for one (algorithm, size bucket) -- bvh_autotune_build's choice.  None of them
// changes the tree.  algo: bvh_algo, +256 for batched builds; bucket: floor(log2(triangles)).
struct TuneEntry {
  int32_t algo = -1, bucket = -1;
  int32_t sort_variant = 0;
  uint32_t tail_pairs = 100000;
  int32_t nn_bps = 3, mg_bps = 8;
  uint32_t grid_max = 0xffffffffu;  // PLOC: k_ploc_grid from this many live clusters (0: never)
};

// Base shapes of a new context: the sort variant by mesh size (-1) until bvh_tuning_set or
// bvh_autotune picks one.
static TuneEntry by_size() {
  TuneEntry t;
  t.sort_variant = -1;
  return t;
}

struct bvh_ctx {
  int device = 0;
  Workspace ws;
  TuneEntry base = by_size();     // shapes where no table entry matches (bvh_tuning_set sets its sort variant)
  std::vector<TuneEntry> table;   // bvh_autotune_build / bvh_tuning_import
  bool tuning_locked = false;     // bvh_autotune_build sets the shapes itself
  unsigned long long* hash_buf = nullptr;  // device word for tree_hash
  BatchGraph bgraph;
  cudaStream_t capture_stream = nullptr;  // for CUDA graph capture (never the legacy stream)
  void* eval_buf = nullptr;               // bvh_evaluate scratch
  size_t eval_bytes = 0;
  void* heat_buf = nullptr;               // bvh_heatmap scratch (heatmap_scratch_bytes())
  StageEvents evs;
  bvh_timing last{};
  int last_algo = -1;
  uint32_t last_n = 0;     // triangles of the last single build (0 after a batched one)
  int32_t last_bits = 30, last_rounds = 0;  // Morton bits and treelet passes of the last build
  bool last_host_loops = false;
  bool have_timing = false;
  uint32_t* h_status = nullptr;  // pinned copy of the device status word
  cudaStream_t last_stream = nullptr;
  // bvh_build_host: a second stream that copies the indices and leaves out while the build ends
  cudaStream_t dl_stream = nullptr;
  cudaEvent_t ev_leaves = nullptr, ev_dl = nullptr;
};

static bvh_status from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return BVH_OK;
  if (e == cudaErrorMemoryAllocation) return BVH_ERR_OUT_OF_MEMORY;
  return BVH_ERR_DEVICE;
}

extern "C" const char* bvh_status_string(bvh_status s) {
  switch (s) {
    case BVH_OK: return "ok";
    case BVH_ERR_INVALID_ARG: return "invalid argument";
    case BVH_ERR_OUT_OF_MEMORY: return "out of memory";
    case BVH_ERR_NO_PROGRESS: return "no progress (PLOC found no mutual pair or hit its iteration cap)";
    case BVH_ERR_DEVICE: return "CUDA device error";
    case BVH_ERR_TIMEOUT: return "device-side wait timed out";
    case BVH_ERR_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

extern "C" const char* bvh_version(void) { return "bvh_gb300 0.1 (sm_103a)"; }

extern "C" bvh_params bvh_default_params(int32_t algo) {
  bvh_params p;
  memset(&p, 0, sizeof(p));
  p.algo = algo;
  p.morton_bits = algo == BVH_ALGO_LBVH_PLUS ? 60 : 30;
  p.treelet_rounds = 1;
  p.ploc_radius = 25;
  p.max_iterations = 0;
  return p;
}

extern "C" bvh_status bvh_ctx_create(bvh_ctx** out, int device) {
  if (!out) return BVH_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return BVH_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return BVH_ERR_DEVICE;
  bvh_ctx* c = new (std::nothrow) bvh_ctx();
  if (!c) return BVH_ERR_OUT_OF_MEMORY;
  c->device = device;
  for (int k = 0; k < 8; ++k)
    if (cudaEventCreate(&c->evs.ev[k]) != cudaSuccess) { delete c; return BVH_ERR_DEVICE; }
  c->evs.use = true;
  if (cudaMallocHost(&c->h_status, 128) != cudaSuccess) { delete c; return BVH_ERR_OUT_OF_MEMORY; }
  if (prepare_kernels() != cudaSuccess) { delete c; return BVH_ERR_DEVICE; }
  if (cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BVH_ERR_DEVICE;
  }
  *out = c;
  return BVH_OK;
}

extern "C" bvh_status bvh_ctx_destroy(bvh_ctx* ctx) {
  if (!ctx) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  if (ctx->bgraph.exec) cudaGraphExecDestroy(ctx->bgraph.exec);
  if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
  if (ctx->dl_stream) cudaStreamDestroy(ctx->dl_stream);
  if (ctx->ev_leaves) cudaEventDestroy(ctx->ev_leaves);
  if (ctx->ev_dl) cudaEventDestroy(ctx->ev_dl);
  workspace_free(ctx->ws);
  cudaFree(ctx->eval_buf);
  cudaFree(ctx->heat_buf);
  for (int k = 0; k < 8; ++k) cudaEventDestroy(ctx->evs.ev[k]);
  cudaFreeHost(ctx->h_status);
  cudaFree(ctx->hash_buf);
  delete ctx;
  return BVH_OK;
}

extern "C" bvh_status bvh_ctx_reserve(bvh_ctx* ctx, uint32_t n, int32_t algo) {
  if (!ctx) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  // zero on the legacy stream and wait, so that builds on any stream see the cleared buffers
  cudaError_t e = workspace_reserve(ctx->ws, n, nullptr);
  if (e == cudaSuccess && algo == BVH_ALGO_PLOC) e = workspace_reserve_ploc(ctx->ws, n);
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  return from_cuda(e);
}

extern "C" bvh_status bvh_ctx_device_bytes(const bvh_ctx* ctx, uint64_t* bytes) {
  if (!ctx || !bytes) return BVH_ERR_INVALID_ARG;
  const Workspace& w = ctx->ws;
  uint64_t b = 0;
  if (w.cap_n) b += (uint64_t)w.cap_n * (8 * 2 + 4 * 2 + sizeof(Box) + 2 * sizeof(Node) + 8) + w.scratch_words * 4;
  if (w.ploc_cap) b += (uint64_t)w.ploc_cap * (2 * sizeof(Box) + 8 + 4) + (w.ploc_cap / 2048 + 8) * 8;
  b += (uint64_t)w.mesh_cap * 36;
  *bytes = b;
  return BVH_OK;
}

static bool valid_params(const bvh_params* p) {
  if (!p) return false;
  switch (p->algo) {
    case BVH_ALGO_LBVH:
      return p->morton_bits == 30 || p->morton_bits == 60 || p->morton_bits == 63;
    case BVH_ALGO_LBVH_PLUS:
      return (p->morton_bits == 30 || p->morton_bits == 60 || p->morton_bits == 63) && p->treelet_rounds >= 0 &&
             p->treelet_rounds <= 63;
    case BVH_ALGO_PLOC:
      return p->ploc_radius >= 1 && p->ploc_radius <= 512 && p->max_iterations >= 0;
  }
  return false;
}

static MeshPtrs mesh_ptrs(const bvh_mesh_soa* m) {
  MeshPtrs p;
  p.v[0] = m->v0x; p.v[1] = m->v0y; p.v[2] = m->v0z;
  p.v[3] = m->v1x; p.v[4] = m->v1y; p.v[5] = m->v1z;
  p.v[6] = m->v2x; p.v[7] = m->v2y; p.v[8] = m->v2z;
  return p;
}

static bool mesh_ok(const bvh_mesh_soa* m) {
  if (!m) return false;
  if (m->n == 0) return true;
  if (m->n > (1u << 30) - 1) return false;  // look-back descriptors hold 30-bit counts
  const float* a[9] = {m->v0x, m->v0y, m->v0z, m->v1x, m->v1y, m->v1z, m->v2x, m->v2y, m->v2z};
  for (int k = 0; k < 9; ++k)
    if (!a[k]) return false;
  return true;
}

static int size_bucket(uint32_t n) { return n ? 31 - __builtin_clz(n) : 0; }

static void set_shapes(Workspace& ws, const TuneEntry& t) {
  ws.sort_variant = t.sort_variant;
  ws.ploc_tail_pairs = t.tail_pairs;
  ws.ploc_nn_bps = t.nn_bps;
  ws.ploc_mg_bps = t.mg_bps;
  ws.ploc_grid_max = t.grid_max;
}

// The table entry for this algorithm and size, else the base shapes.
static void apply_tuning(bvh_ctx* ctx, int32_t algo_key, uint32_t n) {
  if (ctx->tuning_locked) return;
  const int b = size_bucket(n);
  for (const TuneEntry& t : ctx->table)
    if (t.algo == algo_key && t.bucket == b) {
      set_shapes(ctx->ws, t);
      return;
    }
  set_shapes(ctx->ws, ctx->base);
  if (ctx->base.sort_variant < 0) ctx->ws.sort_variant = default_sort_variant(n);
}

static bvh_status build_impl(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, cudaStream_t st,
                             bvh_tree* out) {
  const uint32_t n = mesh->n;
  ctx->last_n = n;
  ctx->last_bits = params->morton_bits;
  ctx->last_rounds = params->treelet_rounds;
  ctx->last_host_loops = params->reserved[1] == BVH_HOST_DRIVEN_LOOPS;
  ctx->ws.no_cooperative = params->reserved[2] == BVH_NO_COOPERATIVE;
  apply_tuning(ctx, params->algo, n);
  ctx->have_timing = false;
  ctx->last = bvh_timing{};
  ctx->last_algo = params->algo;
  ctx->last_stream = st;
  out->nodes = nullptr;
  out->indices = nullptr;
  out->n_nodes = 0;
  out->n_prims = n;
  if (n == 0) return BVH_OK;  // empty mesh: empty tree
  MeshPtrs m = mesh_ptrs(mesh);
  uint32_t* idx = nullptr;
  cudaError_t e;
  if (params->algo == BVH_ALGO_PLOC) {
    e = ploc_build(ctx->ws, m, n, params->ploc_radius, params->max_iterations, st, &ctx->evs, &idx,
                   params->reserved[1] == BVH_HOST_DRIVEN_LOOPS);
    if (e != cudaSuccess) return from_cuda(e);
  } else {
    int rounds = params->algo == BVH_ALGO_LBVH_PLUS ? params->treelet_rounds : 0;
    e = lbvh_build(ctx->ws, m, n, params->morton_bits, rounds, st, &ctx->evs, &idx,
                   params->reserved[1] == BVH_HOST_DRIVEN_LOOPS);
    if (e != cudaSuccess) return from_cuda(e);
  }
  ScratchLayout L = scratch_layout(ctx->ws.cap_n);
  cudaMemcpyAsync(ctx->h_status, ctx->ws.scratch + L.status, 4, cudaMemcpyDeviceToHost, st);
  if (params->algo == BVH_ALGO_PLOC)  // iterations and live-cluster sum, read at bvh_sync
    cudaMemcpyAsync(ctx->h_status + 4, ctx->ws.scratch + L.ploc, 20 * 4, cudaMemcpyDeviceToHost, st);
  if (params->algo == BVH_ALGO_LBVH_PLUS && params->treelet_rounds > 0 && n > 1)  // tree height, read at bvh_sync
    cudaMemcpyAsync(ctx->h_status + 4, ctx->ws.scratch + L.hist + kTlCtlWord, 3 * 4, cudaMemcpyDeviceToHost, st);
  cudaEventRecord(ctx->evs.ev[6], st);
  out->nodes = reinterpret_cast<const bvh_node*>(ctx->ws.nodes);
  out->indices = idx;
  out->n_nodes = 2 * n - 1;
  ctx->have_timing = true;
  return from_cuda(cudaGetLastError());
}

extern "C" bvh_status bvh_build_device(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, void* stream,
                                       bvh_tree* out) {
  if (!ctx || !out || !mesh_ok(mesh) || !valid_params(params)) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  return build_impl(ctx, mesh, params, reinterpret_cast<cudaStream_t>(stream), out);
}

static bvh_status check_status_word(bvh_ctx* ctx) {
  uint32_t s = *ctx->h_status;
  if (s & (kStatusSortTimeout | kStatusClimbTimeout | kStatusGridTimeout)) return BVH_ERR_TIMEOUT;
  if (s & kStatusNoProgress) return BVH_ERR_NO_PROGRESS;
  if (s & kStatusBadInput) return BVH_ERR_DEVICE;  // a kernel skipped an index outside its buffer
  return BVH_OK;
}

extern "C" bvh_status bvh_selftest_bounded_wait(int device, uint32_t polls) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count || polls == 0 ||
      polls > kSpinLimit)
    return BVH_ERR_INVALID_ARG;
  cudaSetDevice(device);
  uint32_t status = 0, grid_status = 0;
  cudaError_t e = wait_selftest(polls, &status);
  if (e != cudaSuccess) return from_cuda(e);
  if ((e = grid_wait_selftest(polls, &grid_status)) != cudaSuccess) return from_cuda(e);
  return (status & kStatusSortTimeout) && (grid_status & kStatusGridTimeout) ? BVH_ERR_TIMEOUT : BVH_ERR_DEVICE;
}

extern "C" bvh_status bvh_sync(bvh_ctx* ctx) {
  if (!ctx) return BVH_ERR_INVALID_ARG;
  if (!ctx->have_timing) return BVH_OK;
  cudaError_t e = cudaEventSynchronize(ctx->evs.ev[6]);
  if (e != cudaSuccess) return from_cuda(e);
  if (ctx->last_algo == BVH_ALGO_PLOC) {
    const uint32_t* w = ctx->h_status + 4;
    ctx->last.ploc_iterations = (int32_t)w[kPlocIterWord];
    ctx->last.ploc_cluster_sum = (uint64_t)w[kPlocSumWord + 1] << 32 | w[kPlocSumWord];
    // bounds, Morton, 4 sort passes, cluster init; 4 per iteration run as separate launches; the
    // middle-iterations and tail kernels (each one launch, whatever it ran); the root fix
    const int32_t one_launch_its = (int32_t)(w[16] + w[17]);
    ctx->last.kernel_launches = ctx->last_n == 0   ? 0  // batched: the caller counts
                                : ctx->last_n > 1 ? 7 + 4 * (ctx->last.ploc_iterations - one_launch_its) +
                                                      (int32_t)w[18] + (int32_t)w[19] + 1
                                                  : 7;
  } else if (ctx->last_algo == BVH_ALGO_LBVH_PLUS) {
    ctx->last.tree_height = (int32_t)ctx->h_status[5];
    // LBVH kernels, then per treelet pass: heights, counts, offsets, grouping, the fallback
    // check; heights 1 (growth, step), 2 (growth, DP, step) and 3 (growth, four DPs by size
    // class, step); then growth + DP + step per height of the loop (the graph runs at least
    // one), and k_tl_narrow for the rest (the last pass's heights stand for every pass)
    const uint32_t* c = ctx->h_status + 4;  // [0] too high, [1] largest height, [2] first height left
    int32_t loop_h;
    if (ctx->last_host_loops) loop_h = c[0] ? 0 : std::max(0, (int32_t)c[1] - 3);
    else loop_h = c[0] ? 1 : std::max(1, (ctx->ws.tl_narrow ? (int32_t)c[2] : (int32_t)c[1] + 1) - 4);
    const int32_t lbvh = 2 + 4 + (ctx->last_bits != 30 ? 2 : 0) + 2;
    ctx->last.kernel_launches =
        ctx->last_n > 1 ? lbvh + ctx->last_rounds * (5 + 11 + 3 * loop_h + (ctx->ws.tl_narrow ? 1 : 0)) : lbvh;
  }
  return check_status_word(ctx);
}

extern "C" bvh_status bvh_last_timing(bvh_ctx* ctx, bvh_timing* out) {
  if (!ctx || !out) return BVH_ERR_INVALID_ARG;
  bvh_status s = bvh_sync(ctx);
  bvh_timing t = ctx->last;
  if (ctx->have_timing) {
    cudaEvent_t* ev = ctx->evs.ev;
    float a = 0;
    if (cudaEventElapsedTime(&a, ev[0], ev[1]) == cudaSuccess) t.bounds_ms = a;
    if (cudaEventElapsedTime(&a, ev[1], ev[2]) == cudaSuccess) t.morton_ms = a;
    if (cudaEventElapsedTime(&a, ev[2], ev[3]) == cudaSuccess) t.sort_ms = a;
    if (cudaEventElapsedTime(&a, ev[3], ev[4]) == cudaSuccess) t.emit_ms = a;
    if (cudaEventElapsedTime(&a, ev[4], ev[5]) == cudaSuccess) t.optimize_ms = a;
    if (cudaEventElapsedTime(&a, ev[0], ev[5]) == cudaSuccess) t.total_ms = a;
  }
  *out = t;
  return s;
}

extern "C" bvh_status bvh_tree_download(bvh_ctx* ctx, const bvh_tree* tree, void* stream, bvh_node* host_nodes,
                                        uint32_t* host_indices) {
  if (!ctx || !tree) return BVH_ERR_INVALID_ARG;
  if (tree->n_nodes == 0) return BVH_OK;
  if (!host_nodes || !host_indices) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(host_nodes, tree->nodes, (size_t)tree->n_nodes * sizeof(bvh_node),
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host_indices, tree->indices, (size_t)tree->n_prims * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return from_cuda(e);
}

extern "C" bvh_status bvh_build_host(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, void* stream,
                                     bvh_node* host_nodes, uint32_t* host_indices, uint32_t* n_nodes) {
  if (!ctx || !mesh_ok(mesh) || !valid_params(params)) return BVH_ERR_INVALID_ARG;
  const uint32_t n = mesh->n;
  if (n_nodes) *n_nodes = 0;
  if (n == 0) return BVH_OK;
  if (!host_nodes || !host_indices) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace& ws = ctx->ws;
  if (ws.mesh_cap < n) {
    cudaFree(ws.mesh_dev);
    ws.mesh_dev = nullptr;
    ws.mesh_cap = 0;
    // nine arrays, each padded to a multiple of 4 floats so that all stay 16-byte aligned
    size_t stride = ((size_t)n + 3) & ~size_t(3);
    cudaError_t e = cudaMalloc(&ws.mesh_dev, stride * 9 * sizeof(float));
    if (e != cudaSuccess) return from_cuda(e);
    ws.mesh_cap = n;
  }
  const size_t stride = ((size_t)ws.mesh_cap + 3) & ~size_t(3);
  const float* src[9] = {mesh->v0x, mesh->v0y, mesh->v0z, mesh->v1x, mesh->v1y, mesh->v1z,
                         mesh->v2x, mesh->v2y, mesh->v2z};
  bvh_mesh_soa dm;
  float* dst[9];
  for (int k = 0; k < 9; ++k) {
    dst[k] = ws.mesh_dev + stride * k;
    cudaError_t e = cudaMemcpyAsync(dst[k], src[k], (size_t)n * 4, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return from_cuda(e);
  }
  dm.v0x = dst[0]; dm.v0y = dst[1]; dm.v0z = dst[2];
  dm.v1x = dst[3]; dm.v1y = dst[4]; dm.v1z = dst[5];
  dm.v2x = dst[6]; dm.v2y = dst[7]; dm.v2z = dst[8];
  dm.n = n;
  // A plain LBVH's indices are final after the sort and its leaves after the emission kernel:
  // a second stream copies those out while the rest of the build runs; the internal nodes
  // follow on the build's stream.  The copies use the link the whole time, which bounds the call.
  const bool early = params->algo == BVH_ALGO_LBVH && n > 1;
  if (early && !ctx->dl_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->dl_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_leaves, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_dl, cudaEventDisableTiming);
    if (e != cudaSuccess) return from_cuda(e);
  }
  bvh_tree tree;
  ws.leaves_ready = early ? ctx->ev_leaves : nullptr;
  bvh_status s = build_impl(ctx, &dm, params, st, &tree);
  ws.leaves_ready = nullptr;
  if (s != BVH_OK) return s;
  if (early) {
    cudaStream_t dl = ctx->dl_stream;
    cudaError_t e = cudaStreamWaitEvent(dl, ctx->evs.ev[3], 0);  // sort (and run fix-up) done
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_indices, tree.indices, (size_t)n * 4, cudaMemcpyDeviceToHost, dl);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(dl, ctx->ev_leaves, 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host_nodes + (n - 1), tree.nodes + (n - 1), (size_t)n * sizeof(bvh_node),
                          cudaMemcpyDeviceToHost, dl);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_dl, dl);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host_nodes, tree.nodes, (size_t)(n - 1) * sizeof(bvh_node), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->ev_dl, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(dl);
      return from_cuda(e);
    }
  } else {
    s = bvh_tree_download(ctx, &tree, stream, host_nodes, host_indices);
    if (s != BVH_OK) return s;
  }
  s = check_status_word(ctx);
  if (s == BVH_OK && n_nodes) *n_nodes = tree.n_nodes;
  return s;
}

// ---------------------------------------------------------------------------------------
// batched builds
// ---------------------------------------------------------------------------------------
// Staged batch layout (pinned host copy and device copy, 32-bit words):
//   [0, count]                  mesh offsets
//   [items_at, items_at + 4*k)  work items (mesh, begin, end, 0), meshes split every kSegChunk
static size_t items_at(uint32_t count) { return ((size_t)count + 1 + 3) & ~size_t(3); }
static uint32_t count_items(const uint32_t* offsets, uint32_t count) {
  uint64_t k = 0;
  for (uint32_t m = 0; m < count; ++m) k += div_up(offsets[m + 1] - offsets[m], kSegChunk);
  return (uint32_t)k;
}
static void stage_layout(uint32_t* dst, const uint32_t* offsets, uint32_t count) {
  memcpy(dst, offsets, ((size_t)count + 1) * 4);
  SegItem* it = reinterpret_cast<SegItem*>(dst + items_at(count));
  for (uint32_t m = 0; m < count; ++m)
    for (uint32_t b = offsets[m]; b < offsets[m + 1]; b += kSegChunk)
      *it++ = SegItem{m, b, std::min(offsets[m + 1], b + kSegChunk), 0};
}

static cudaError_t reserve_batch(Workspace& ws, uint32_t n, uint32_t count, size_t words, cudaStream_t st) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  if (ws.bat_words_cap < words || ws.bat_count_cap < count || !ws.bat_offsets) {
    cudaDeviceSynchronize();  // the staging buffer may still be read by queued copies
    cudaFree(ws.bat_offsets);
    cudaFreeHost(ws.bat_offsets_h);
    cudaFree(ws.bat_mbox);
    ws.bat_offsets = nullptr; ws.bat_offsets_h = nullptr; ws.bat_mbox = nullptr;
    ws.bat_count_cap = 0; ws.bat_words_cap = 0; ws.bat_items = 0;
    size_t wcap = words < 1024 ? 1024 : words;
    uint32_t ccap = count < 64 ? 64 : count;
    if ((e = cudaMalloc(&ws.bat_offsets, wcap * 4)) != cudaSuccess) return e;
    if ((e = cudaMallocHost(&ws.bat_offsets_h, wcap * 4)) != cudaSuccess) return e;
    memset(ws.bat_offsets_h, 0, wcap * 4);
    if ((e = cudaMalloc(&ws.bat_mbox, (size_t)ccap * 8 * 4)) != cudaSuccess) return e;
    ws.bat_count_cap = ccap;
    ws.bat_words_cap = wcap;
  }
  if (ws.bat_n_cap < n || !ws.bat_indices) {
    cudaFree(ws.bat_indices);
    ws.bat_indices = nullptr;
    ws.bat_n_cap = 0;
    if ((e = cudaMalloc(&ws.bat_indices, (size_t)(n ? n : 1) * 4)) != cudaSuccess) return e;
    ws.bat_n_cap = n;
  }
  return cudaSuccess;
}

static cudaError_t enqueue_batch(bvh_ctx* ctx, const MeshPtrs& m, uint32_t n, uint32_t count, size_t words,
                                 const bvh_params* params, cudaStream_t st, bool events) {
  Workspace& ws = ctx->ws;
  cudaError_t e = cudaMemcpyAsync(ws.bat_offsets, ws.bat_offsets_h, words * 4, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  StageEvents none;
  const SegItem* items = reinterpret_cast<const SegItem*>(ws.bat_offsets + items_at(count));
  if (params->algo == BVH_ALGO_PLOC)
    return batched_ploc_build(ws, m, n, ws.bat_offsets, count, items, ws.bat_items, ws.bat_mbox, ws.bat_indices,
                              params->ploc_radius, (uint32_t)params->max_iterations, st, events ? &ctx->evs : &none,
                              params->reserved[1] == BVH_HOST_DRIVEN_LOOPS);
  return batched_build(ws, m, n, ws.bat_offsets, count, items, ws.bat_items, ws.bat_mbox, ws.bat_indices, st,
                       events ? &ctx->evs : &none);
}

extern "C" bvh_status bvh_build_batched(bvh_ctx* ctx, const bvh_batch* batch, const bvh_params* params, void* stream,
                                        bvh_tree* out) {
  if (!ctx || !batch || !out || !params || !mesh_ok(&batch->mesh) || !batch->offsets) return BVH_ERR_INVALID_ARG;
  if (!valid_params(params)) return BVH_ERR_INVALID_ARG;
  const bool ploc = params->algo == BVH_ALGO_PLOC;
  if (!ploc && (params->algo != BVH_ALGO_LBVH || params->morton_bits != 30)) return BVH_ERR_UNSUPPORTED;
  const uint32_t n = batch->mesh.n, count = batch->count;
  if (count == 0 || count > n || count > (1u << 24) || batch->offsets[0] != 0 || batch->offsets[count] != n)
    return BVH_ERR_INVALID_ARG;
  for (uint32_t k = 0; k < count; ++k)
    if (batch->offsets[k + 1] <= batch->offsets[k]) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Workspace& ws = ctx->ws;
  ctx->have_timing = false;
  ctx->last = bvh_timing{};
  ctx->last_n = 0;
  ctx->last_algo = params->algo;
  apply_tuning(ctx, params->algo + 256, n);
  const uint32_t n_items = count_items(batch->offsets, count);
  const size_t words = items_at(count) + 4 * (size_t)n_items;
  cudaError_t e = reserve_batch(ws, n, count, words, st);
  if (e != cudaSuccess) return from_cuda(e);
  if (ploc) {  // everything a capture may not do: allocations, kernel attributes
    if ((e = workspace_reserve_ploc(ws, n)) != cudaSuccess) return from_cuda(e);
    if ((e = ploc_prepare(params->ploc_radius)) != cudaSuccess) return from_cuda(e);
    if (params->reserved[1] == BVH_HOST_DRIVEN_LOOPS && !ws.ploc_host &&
        (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess)
      return from_cuda(e);
  }
  // the device copy reads the pinned staging buffer when it executes: rewrite it only when the
  // layout changed, after the work that may still read it has finished
  const bool changed = ws.bat_items != n_items ||
                       memcmp(ws.bat_offsets_h, batch->offsets, ((size_t)count + 1) * 4) != 0;
  if (changed) {
    cudaDeviceSynchronize();
    stage_layout(ws.bat_offsets_h, batch->offsets, count);
    ws.bat_items = n_items;
  }
  MeshPtrs m = mesh_ptrs(&batch->mesh);
  // (a host-driven PLOC loop reads the device between iterations, so it cannot be captured)
  const bool use_graph = params->reserved[0] == BVH_BATCH_USE_GRAPH &&
                         !(ploc && params->reserved[1] == BVH_HOST_DRIVEN_LOOPS);
  if (use_graph) {
    BatchGraph& g = ctx->bgraph;
    bool same = g.exec && !changed && g.n == n && g.count == count && memcmp(g.ptrs, m.v, sizeof(g.ptrs)) == 0 &&
                g.algo == params->algo && g.radius == params->ploc_radius && g.max_iter == params->max_iterations &&
                g.sort_variant == ws.sort_variant && g.shape == ((uint32_t)ws.ploc_nn_bps << 16 | (uint32_t)ws.ploc_mg_bps);
    if (!same) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      // capture on the context's own stream: the caller's may be the legacy default stream,
      // which cannot be captured; the graph is launched on the caller's stream
      cudaGraph_t graph = nullptr;
      if ((e = cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return from_cuda(e);
      cudaError_t e2 = enqueue_batch(ctx, m, n, count, words, params, ctx->capture_stream, false);
      e = cudaStreamEndCapture(ctx->capture_stream, &graph);
      if (e2 != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return from_cuda(e2); }
      if (e != cudaSuccess) return from_cuda(e);
      e = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) { g.exec = nullptr; return from_cuda(e); }
      memcpy(g.ptrs, m.v, sizeof(g.ptrs));
      g.n = n;
      g.count = count;
      g.algo = params->algo;
      g.radius = params->ploc_radius;
      g.max_iter = params->max_iterations;
      g.sort_variant = ws.sort_variant;
      g.shape = (uint32_t)ws.ploc_nn_bps << 16 | (uint32_t)ws.ploc_mg_bps;
    }
    cudaEventRecord(ctx->evs.ev[0], st);
    if ((e = epoch_tick(ws, st)) != cudaSuccess) return from_cuda(e);  // the graph bumps the epoch
    if ((e = cudaGraphLaunch(g.exec, st)) != cudaSuccess) return from_cuda(e);
    for (int k = 1; k <= 5; ++k) cudaEventRecord(ctx->evs.ev[k], st);
  } else {
    if ((e = enqueue_batch(ctx, m, n, count, words, params, st, true)) != cudaSuccess) return from_cuda(e);
  }
  ScratchLayout L = scratch_layout(ws.cap_n);
  cudaMemcpyAsync(ctx->h_status, ws.scratch + L.status, 4, cudaMemcpyDeviceToHost, st);
  if (ploc)  // iterations and live-cluster sum, read at bvh_sync
    cudaMemcpyAsync(ctx->h_status + 4, ws.scratch + L.ploc, 20 * 4, cudaMemcpyDeviceToHost, st);
  cudaEventRecord(ctx->evs.ev[6], st);
  ctx->last_stream = st;
  ctx->have_timing = true;
  out->nodes = reinterpret_cast<const bvh_node*>(ws.nodes);
  out->indices = ws.bat_indices;
  out->n_nodes = 2 * n - count;
  out->n_prims = n;
  return from_cuda(cudaGetLastError());
}

// ---------------------------------------------------------------------------------------
// evaluation
// ---------------------------------------------------------------------------------------
extern "C" bvh_status bvh_evaluate(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, void* stream,
                                   bvh_eval_stats* out) {
  if (!ctx || !out || (n_nodes && !nodes) || n_nodes > 0x7fffffffu) return BVH_ERR_INVALID_ARG;
  *out = bvh_eval_stats{};
  if (n_nodes == 0) return BVH_OK;
  cudaSetDevice(ctx->device);
  const size_t need = evaluate_scratch_bytes(n_nodes);
  if (ctx->eval_bytes < need) {
    cudaFree(ctx->eval_buf);
    ctx->eval_buf = nullptr;
    ctx->eval_bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->eval_buf, need);
    if (e != cudaSuccess) return from_cuda(e);
    ctx->eval_bytes = need;
  }
  EvalResult r;
  cudaError_t e = evaluate_tree(reinterpret_cast<const Node*>(nodes), n_nodes, ctx->eval_buf,
                                reinterpret_cast<cudaStream_t>(stream), &r);
  if (e != cudaSuccess) return from_cuda(e);
  out->sah = r.sah;
  out->avg_leaf_depth = r.avg_leaf_depth;
  out->node_count = r.nodes;
  out->leaf_count = r.leaves;
  out->max_depth = r.max_depth;
  return BVH_OK;
}

// ---------------------------------------------------------------------------------------
// autotuning
// ---------------------------------------------------------------------------------------
extern "C" bvh_status bvh_autotune(bvh_ctx* ctx, uint32_t n, void* stream, char* json_out, size_t json_cap) {
  if (!ctx || n < 1024 || n > (1u << 30) - 1) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int nv = sort_variant_count();
  std::vector<float> ms(nv, 0.0f);
  cudaError_t e = autotune_sort(ctx->ws, n, st, ms.data());
  if (e != cudaSuccess) return from_cuda(e);
  ctx->base.sort_variant = ctx->ws.sort_variant;
  if (json_out && json_cap) {
    std::string js = "{\"n\": " + std::to_string(n) + ", \"sort\": {\"chosen\": " +
                     std::to_string(ctx->ws.sort_variant) + ", \"variants\": [";
    for (int v = 0; v < nv; ++v) {
      int ipt, w, mb;
      sort_variant_describe(v, &ipt, &w, &mb);
      char buf[160];
      snprintf(buf, sizeof(buf), "%s{\"items_per_thread\": %d, \"lookback_window\": %d, \"min_blocks\": %d, "
               "\"ms\": %.4f}", v ? ", " : "", ipt, w, mb, ms[v]);
      js += buf;
    }
    js += "]}}";
    if (js.size() + 1 > json_cap) return BVH_ERR_INVALID_ARG;
    memcpy(json_out, js.c_str(), js.size() + 1);
  }
  return BVH_OK;
}

extern "C" bvh_status bvh_tuning_get(const bvh_ctx* ctx, int32_t* variant) {
  if (!ctx || !variant) return BVH_ERR_INVALID_ARG;
  *variant = ctx->ws.sort_variant;
  return BVH_OK;
}

extern "C" bvh_status bvh_tuning_set(bvh_ctx* ctx, int32_t variant) {
  if (!ctx || variant < 0 || variant >= sort_variant_count()) return BVH_ERR_INVALID_ARG;
  ctx->ws.sort_variant = variant;
  ctx->base.sort_variant = variant;
  return BVH_OK;
}

// ---- autotuning of whole builds ------------------------------------------------------------
static std::string entry_json(const TuneEntry& t) {
  char buf[200];
  snprintf(buf, sizeof(buf),
           "{\"algo\": %d, \"bucket\": %d, \"sort_variant\": %d, \"ploc_tail_pairs\": %u, \"ploc_nn_bps\": %d, "
           "\"ploc_mg_bps\": %d, \"ploc_grid_max\": %u}",
           t.algo, t.bucket, t.sort_variant, t.tail_pairs, t.nn_bps, t.mg_bps, t.grid_max);
  return buf;
}

static bool valid_entry(const TuneEntry& t) {
  return t.sort_variant >= 0 && t.sort_variant < sort_variant_count() && t.nn_bps >= 1 && t.nn_bps <= 16 &&
         t.mg_bps >= 1 && t.mg_bps <= 32 && t.tail_pairs <= 10000000u && t.bucket >= 0 && t.bucket < 32;
}

static bvh_status write_json(const std::string& js, char* out, size_t cap) {
  if (!out || !cap) return BVH_OK;
  if (js.size() + 1 > cap) return BVH_ERR_INVALID_ARG;
  memcpy(out, js.c_str(), js.size() + 1);
  return BVH_OK;
}

// Builds the mesh `reps` times after one warm-up build: the mean device time, the tree's hash
// and (sah != NULL) its SAH.
static bvh_status timed_builds(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* p, cudaStream_t st, int reps,
                               float* ms, unsigned long long* hash, double* sah) {
  bvh_tree tr;
  bvh_status s = build_impl(ctx, mesh, p, st, &tr);
  if (s == BVH_OK) s = bvh_sync(ctx);
  if (s != BVH_OK) return s;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess) return BVH_ERR_DEVICE;
  if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return BVH_ERR_DEVICE; }
  cudaEventRecord(a, st);
  for (int k = 0; k < reps && s == BVH_OK; ++k) s = build_impl(ctx, mesh, p, st, &tr);
  cudaEventRecord(b, st);
  if (s == BVH_OK) s = bvh_sync(ctx);
  if (s == BVH_OK) s = from_cuda(cudaEventSynchronize(b));
  float t = 0;
  if (s == BVH_OK) s = from_cuda(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (s != BVH_OK) return s;
  *ms = t / (float)reps;
  if ((s = from_cuda(tree_hash(reinterpret_cast<const Node*>(tr.nodes), tr.n_nodes, ctx->hash_buf, st))) != BVH_OK)
    return s;
  if ((s = from_cuda(cudaMemcpyAsync(ctx->h_status + 24, ctx->hash_buf, 8, cudaMemcpyDeviceToHost, st))) != BVH_OK ||
      (s = from_cuda(cudaStreamSynchronize(st))) != BVH_OK)
    return s;
  memcpy(hash, ctx->h_status + 24, 8);  // (words 4-19 take PLOC's control words)
  if (sah) {
    bvh_eval_stats es;
    if ((s = bvh_evaluate(ctx, tr.nodes, tr.n_nodes, reinterpret_cast<void*>(st), &es)) != BVH_OK) return s;
    *sah = es.sah;
  }
  return BVH_OK;
}

extern "C" bvh_status bvh_autotune_build(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params,
                                         void* stream, char* json_out, size_t json_cap) {
  if (!ctx || !mesh_ok(mesh) || !valid_params(params) || mesh->n < 1024) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (!ctx->hash_buf && cudaMalloc(&ctx->hash_buf, 8) != cudaSuccess) return BVH_ERR_OUT_OF_MEMORY;
  const uint32_t n = mesh->n;
  const int32_t algo = params->algo;
  // start from the shapes the build would use now
  ctx->tuning_locked = false;
  apply_tuning(ctx, algo, n);
  TuneEntry best;
  best.sort_variant = ctx->ws.sort_variant;
  best.tail_pairs = ctx->ws.ploc_tail_pairs;
  best.nn_bps = ctx->ws.ploc_nn_bps;
  best.mg_bps = ctx->ws.ploc_mg_bps;
  best.grid_max = ctx->ws.ploc_grid_max;
  best.algo = algo;
  best.bucket = size_bucket(n);
  ctx->tuning_locked = true;
  const int reps = 3;
  std::string trials;
  float best_ms = 0;
  unsigned long long ref_hash = 0;
  auto trial = [&](const TuneEntry& t, bool first) -> bvh_status {
    set_shapes(ctx->ws, t);
    float ms = 0;
    unsigned long long h = 0;
    bvh_status s = timed_builds(ctx, mesh, params, st, reps, &ms, &h, nullptr);
    if (s != BVH_OK) return s;
    if (first) ref_hash = h;
    const bool same = h == ref_hash;
    char buf[320];
    snprintf(buf, sizeof(buf),
             "%s{\"sort_variant\": %d, \"ploc_tail_pairs\": %u, \"ploc_nn_bps\": %d, \"ploc_mg_bps\": %d, "
             "\"ploc_grid_max\": %u, "
             "\"ms\": %.4f, \"same_tree\": %s}",
             trials.empty() ? "" : ", ", t.sort_variant, t.tail_pairs, t.nn_bps, t.mg_bps, t.grid_max, ms,
             same ? "true" : "false");
    trials += buf;
    if (!same) return BVH_ERR_DEVICE;  // a launch shape changed the tree: never expected
    if (first || ms < best_ms) {
      best = t;
      best_ms = ms;
    }
    return BVH_OK;
  };
  bvh_status s = trial(best, true);
  for (int v = 0; s == BVH_OK && v < sort_variant_count(); ++v) {
    TuneEntry t = best;
    t.sort_variant = v;
    if (v != best.sort_variant) s = trial(t, false);
  }
  if (algo == BVH_ALGO_PLOC) {
    for (uint32_t pairs : {0u, 50000u, 100000u, 200000u}) {
      TuneEntry t = best;
      t.tail_pairs = pairs;
      if (s == BVH_OK && pairs != best.tail_pairs) s = trial(t, false);
    }
    for (int k : {2, 3, 4}) {
      TuneEntry t = best;
      t.nn_bps = k;
      if (s == BVH_OK && k != best.nn_bps) s = trial(t, false);
    }
    for (int k : {4, 8, 16}) {
      TuneEntry t = best;
      t.mg_bps = k;
      if (s == BVH_OK && k != best.mg_bps) s = trial(t, false);
    }
    for (uint32_t g : {0u, 65536u, 150000u, 300000u, 0xffffffffu}) {
      TuneEntry t = best;
      t.grid_max = g;
      if (s == BVH_OK && g != best.grid_max) s = trial(t, false);
    }
  }
  // choices that change the tree are reported with their cost and SAH, not chosen
  std::string quality;
  if (s == BVH_OK) {
    set_shapes(ctx->ws, best);
    std::vector<bvh_params> alts;
    const char* what = "";
    if (algo == BVH_ALGO_PLOC) {
      what = "ploc_radius";
      for (int r : {10, 25, 50, 100}) { bvh_params q = *params; q.ploc_radius = r; alts.push_back(q); }
    } else if (algo == BVH_ALGO_LBVH_PLUS) {
      what = "treelet_rounds";
      for (int r : {1, 2, 3}) { bvh_params q = *params; q.treelet_rounds = r; alts.push_back(q); }
    } else {
      what = "morton_bits";
      for (int b : {30, 60, 63}) { bvh_params q = *params; q.morton_bits = b; alts.push_back(q); }
    }
    for (const bvh_params& q : alts) {
      float ms = 0;
      unsigned long long h = 0;
      double sah = 0;
      if ((s = timed_builds(ctx, mesh, &q, st, reps, &ms, &h, &sah)) != BVH_OK) break;
      const int val = algo == BVH_ALGO_PLOC ? q.ploc_radius : algo == BVH_ALGO_LBVH_PLUS ? q.treelet_rounds : q.morton_bits;
      char buf[160];
      snprintf(buf, sizeof(buf), "%s{\"%s\": %d, \"ms\": %.4f, \"sah\": %.17g}", quality.empty() ? "" : ", ", what,
               val, ms, sah);
      quality += buf;
    }
  }
  ctx->tuning_locked = false;
  if (s != BVH_OK) return s;
  bool replaced = false;
  for (TuneEntry& t : ctx->table)
    if (t.algo == best.algo && t.bucket == best.bucket) {
      t = best;
      replaced = true;
    }
  if (!replaced) ctx->table.push_back(best);
  apply_tuning(ctx, algo, n);
  return write_json("{\"n\": " + std::to_string(n) + ", \"chosen\": " + entry_json(best) + ", \"best_ms\": " +
                        std::to_string(best_ms) + ", \"trials\": [" + trials + "], \"tree_changing\": [" + quality +
                        "]}",
                    json_out, json_cap);
}

extern "C" bvh_status bvh_tuning_export(const bvh_ctx* ctx, char* json_out, size_t json_cap) {
  if (!ctx || !json_out || !json_cap) return BVH_ERR_INVALID_ARG;
  std::string js = "{\"base\": " + entry_json(ctx->base) + ", \"entries\": [";
  for (size_t k = 0; k < ctx->table.size(); ++k) js += (k ? ", " : "") + entry_json(ctx->table[k]);
  return write_json(js + "]}", json_out, json_cap);
}

// Reads the integer after "key": in [p, end); false when absent.
static bool json_int(const char* p, const char* end, const char* key, long long* v) {
  const std::string k = std::string("\"") + key + "\"";
  const char* f = std::search(p, end, k.begin(), k.end());
  if (f == end) return false;
  f += k.size();
  while (f < end && (*f == ' ' || *f == ':' || *f == '\t' || *f == '\n')) ++f;
  char* stop = nullptr;
  *v = strtoll(f, &stop, 10);
  return stop != f;
}

extern "C" bvh_status bvh_tuning_import(bvh_ctx* ctx, const char* json) {
  if (!ctx || !json) return BVH_ERR_INVALID_ARG;
  // the objects of the "entries" array (flat objects, no nested arrays); anything else in the
  // document (a "base" entry, reports) is ignored
  const char* ent = strstr(json, "\"entries\"");
  const char* lb = ent ? strchr(ent, '[') : nullptr;
  const char* rb = lb ? strchr(lb, ']') : nullptr;
  if (!rb) return BVH_ERR_INVALID_ARG;
  std::vector<TuneEntry> table;
  for (const char* o = std::find(lb, rb, '{'); o < rb; o = std::find(o + 1, rb, '{')) {
    const char* c = std::find(o, rb, '}');
    if (c == rb) return BVH_ERR_INVALID_ARG;
    TuneEntry t;
    long long v;
    if (!json_int(o, c, "algo", &v)) return BVH_ERR_INVALID_ARG;
    t.algo = (int32_t)v;
    if (!json_int(o, c, "bucket", &v)) return BVH_ERR_INVALID_ARG;
    t.bucket = (int32_t)v;
    if (json_int(o, c, "sort_variant", &v)) t.sort_variant = (int32_t)v;
    if (json_int(o, c, "ploc_tail_pairs", &v)) {
      if (v < 0 || v > 10000000ll) return BVH_ERR_INVALID_ARG;
      t.tail_pairs = (uint32_t)v;
    }
    if (json_int(o, c, "ploc_nn_bps", &v)) t.nn_bps = (int32_t)v;
    if (json_int(o, c, "ploc_mg_bps", &v)) t.mg_bps = (int32_t)v;
    if (json_int(o, c, "ploc_grid_max", &v)) {
      if (v < 0 || v > 0xffffffffll) return BVH_ERR_INVALID_ARG;
      t.grid_max = (uint32_t)v;
    }
    if (!valid_entry(t)) return BVH_ERR_INVALID_ARG;
    table.push_back(t);
    o = c;
  }
  ctx->table = table;
  return BVH_OK;
}

// ---------------------------------------------------------------------------------------
// traversal
// ---------------------------------------------------------------------------------------
extern "C" bvh_status bvh_trace(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, const bvh_mesh_soa* mesh,
                                const bvh_rays* rays, const bvh_hits* hits, void* stream) {
  if (!ctx || !mesh_ok(mesh) || !rays || !hits) return BVH_ERR_INVALID_ARG;
  if (rays->n == 0) return BVH_OK;
  if (n_nodes > 0 && !nodes) return BVH_ERR_INVALID_ARG;
  if (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz) return BVH_ERR_INVALID_ARG;
  if (!hits->t || !hits->prim || !hits->nodes_visited || !hits->aabb_tests || !hits->tri_tests)
    return BVH_ERR_INVALID_ARG;
  if (n_nodes > 0x7fffffffu) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  RayPtrs rp;
  rp.o[0] = rays->ox; rp.o[1] = rays->oy; rp.o[2] = rays->oz;
  rp.d[0] = rays->dx; rp.d[1] = rays->dy; rp.d[2] = rays->dz;
  HitOut ho{hits->t, hits->prim, hits->nodes_visited, hits->aabb_tests, hits->tri_tests};
  return from_cuda(trace_rays(reinterpret_cast<const Node*>(nodes), (int)n_nodes, mesh_ptrs(mesh), mesh->n, rp,
                              rays->n, ho, reinterpret_cast<cudaStream_t>(stream)));
}

// The camera as the kernels take it; generateRay's basis is derived on the device, per ray.
static bool make_cam(const bvh_camera* cam, int32_t w, int32_t h, PinholeCam* b) {
  if (!cam || w <= 0 || h <= 0) return false;
  if ((uint64_t)w * (uint64_t)h > 0xffffffffull) return false;
  for (int k = 0; k < 3; ++k) { b->eye[k] = cam->eye[k]; b->look[k] = cam->look_at[k]; b->up[k] = cam->up[k]; }
  b->fov_deg = cam->fov_y_deg;
  b->width = w;
  b->height = h;
  return true;
}

extern "C" bvh_status bvh_trace_pinhole(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, const bvh_mesh_soa* mesh,
                                        const bvh_camera* cam, int32_t width, int32_t height, const bvh_hits* hits,
                                        void* stream) {
  if (!ctx || !mesh_ok(mesh) || !hits) return BVH_ERR_INVALID_ARG;
  if (!hits->t || !hits->prim || !hits->nodes_visited || !hits->aabb_tests || !hits->tri_tests)
    return BVH_ERR_INVALID_ARG;
  if (n_nodes > 0 && !nodes) return BVH_ERR_INVALID_ARG;
  PinholeCam b;
  if (!make_cam(cam, width, height, &b)) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  HitOut ho{hits->t, hits->prim, hits->nodes_visited, hits->aabb_tests, hits->tri_tests};
  return from_cuda(trace_pinhole(reinterpret_cast<const Node*>(nodes), (int)n_nodes, mesh_ptrs(mesh), mesh->n, b, ho,
                                 reinterpret_cast<cudaStream_t>(stream)));
}

extern "C" bvh_status bvh_pinhole_rays(const bvh_camera* cam, int32_t width, int32_t height, float* ox, float* oy,
                                       float* oz, float* dx, float* dy, float* dz, void* stream) {
  PinholeCam b;
  if (!make_cam(cam, width, height, &b)) return BVH_ERR_INVALID_ARG;
  if (!ox || !oy || !oz || !dx || !dy || !dz) return BVH_ERR_INVALID_ARG;
  return from_cuda(pinhole_rays(b, ox, oy, oz, dx, dy, dz, reinterpret_cast<cudaStream_t>(stream)));
}

extern "C" bvh_status bvh_shade(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_camera* cam, int32_t width,
                                int32_t height, const bvh_hits* hits, int32_t mode, float scene_diag,
                                const float* light_dir, float* rgb, void* stream) {
  if (!ctx || !mesh_ok(mesh) || !hits || !hits->t || !hits->prim || !hits->nodes_visited || !rgb || !light_dir)
    return BVH_ERR_INVALID_ARG;
  PinholeCam b;
  if (!make_cam(cam, width, height, &b)) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  ShadeIn in{hits->t, hits->prim, hits->nodes_visited};
  return from_cuda(shade_pixels(b, mesh_ptrs(mesh), mesh->n, in, mode, scene_diag,
                                make_float3(light_dir[0], light_dir[1], light_dir[2]), rgb,
                                reinterpret_cast<cudaStream_t>(stream)));
}

extern "C" bvh_status bvh_heatmap(bvh_ctx* ctx, const int32_t* nodes_visited, uint32_t n_pixels, const float* colormap,
                                  float fixed_max, float* rgb, float* used_max, void* stream) {
  if (!ctx || (n_pixels && (!nodes_visited || !colormap || !rgb))) return BVH_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if (!ctx->heat_buf) {
    cudaError_t e = cudaMalloc(&ctx->heat_buf, heatmap_scratch_bytes());
    if (e != cudaSuccess) return from_cuda(e);
  }
  return from_cuda(heatmap(nodes_visited, n_pixels, colormap, fixed_max, ctx->heat_buf, rgb, used_max,
                           reinterpret_cast<cudaStream_t>(stream)));
}

extern "C" bvh_status bvh_rgb8(const float* rgb, uint32_t n_values, uint8_t* out, void* stream) {
  if (n_values && (!rgb || !out)) return BVH_ERR_INVALID_ARG;
  return from_cuda(rgb_to_bytes(rgb, n_values, out, reinterpret_cast<cudaStream_t>(stream)));
}

// autoCamera, src/render_engine.cu:601-637.
extern "C" bvh_status bvh_auto_camera(const bvh_node* root, bvh_camera* cam) {
  if (!cam) return BVH_ERR_INVALID_ARG;
  cam->fov_y_deg = 60.0f;
  cam->up[0] = 0.0f; cam->up[1] = 1.0f; cam->up[2] = 0.0f;
  if (!root) {
    cam->eye[0] = 0.0f; cam->eye[1] = 0.0f; cam->eye[2] = 5.0f;
    cam->look_at[0] = cam->look_at[1] = cam->look_at[2] = 0.0f;
    return BVH_OK;
  }
  float c[3] = {(root->min_x + root->max_x) * 0.5f, (root->min_y + root->max_y) * 0.5f,
                (root->min_z + root->max_z) * 0.5f};
  float e[3] = {root->max_x - root->min_x, root->max_y - root->min_y, root->max_z - root->min_z};
  float diag = sqrtf((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]);
  if (diag < 1e-6f) diag = 2.0f;
  float fov = cam->fov_y_deg * 3.14159265358979f / 180.0f;
  float dist = (diag * 0.5f) / tanf(fov * 0.5f) * 1.2f;
  cam->eye[0] = c[0] + dist * 0.6f;
  cam->eye[1] = c[1] + dist * 0.3f;
  cam->eye[2] = c[2] + dist * 0.7f;
  for (int k = 0; k < 3; ++k) cam->look_at[k] = c[k];
  return BVH_OK;
}
