// ref_runner.cu -- runs the reference's own GPU kernels (TEST INFRASTRUCTURE).
//
// The reference's .cu files are compiled, unmodified, into sm_103a fatbins under oracle/_ref/
// by oracle/ref_build.py (device code only).  This file is our own host code: it loads those
// fatbins with the driver API and replays the reference builders' host sequences --
// LBVHBuilderCUDA::build (src/cuda/lbvh_builder.cu:334-488), LBVHPlusBuilderCUDA::build
// (src/cuda/lbvh_plus_builder.cu:419-533), PLOCBuilderCUDA::build (src/cuda/ploc_builder.cu:403-586)
// and renderImage (src/render_engine.cu:711-853) -- with the same CUB/Thrust calls, the same
// allocations inside the timed regions and the same event placement, so that
// getLastBuildTimeMS-equivalent times and outputs are the reference's.
//
// Used by tests/ as a second oracle and by bench.py's reference arm.  Never part of the library.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/fill.h>
#include <thrust/reduce.h>
#include <thrust/sort.h>

#include <chrono>
#include <cfloat>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace {

// Layouts of the reference's data model (include/common.h, mesh.h, bvh_node.h,
// src/cuda/lbvh_builder.cuh:9-14, include/render_engine.h:24-33).
struct __align__(16) F3 { float x, y, z; };
struct __align__(16) Box { F3 mn, mx; };
struct Tris { float* v[9]; };
struct __align__(16) LNode { Box box; uint32_t l, r, parent; };
struct __align__(16) Node { Box box; int32_t l, r; };
struct Cam { F3 eye, look, up; float fov; };
static_assert(sizeof(Box) == 32 && sizeof(LNode) == 48 && sizeof(Node) == 48, "layout");
static_assert(sizeof(Cam) == 64, "Camera layout");

struct BoxUnion {
  __host__ __device__ Box operator()(const Box& a, const Box& b) const {
    Box r;
#ifdef __CUDA_ARCH__
    r.mn.x = fminf(a.mn.x, b.mn.x); r.mn.y = fminf(a.mn.y, b.mn.y); r.mn.z = fminf(a.mn.z, b.mn.z);
    r.mx.x = fmaxf(a.mx.x, b.mx.x); r.mx.y = fmaxf(a.mx.y, b.mx.y); r.mx.z = fmaxf(a.mx.z, b.mx.z);
#else
    r.mn.x = a.mn.x < b.mn.x ? a.mn.x : b.mn.x; r.mn.y = a.mn.y < b.mn.y ? a.mn.y : b.mn.y;
    r.mn.z = a.mn.z < b.mn.z ? a.mn.z : b.mn.z; r.mx.x = a.mx.x > b.mx.x ? a.mx.x : b.mx.x;
    r.mx.y = a.mx.y > b.mx.y ? a.mx.y : b.mx.y; r.mx.z = a.mx.z > b.mx.z ? a.mx.z : b.mx.z;
#endif
    return r;
  }
};

struct Mod {
  CUmodule m = nullptr;
};
Mod g_lbvh, g_plus, g_ploc, g_render, g_trace;
std::string g_dir;
std::string g_err;

#define CK(x)                                                               \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) {                                                \
      g_err = std::string(#x) + ": " + cudaGetErrorString(e_);              \
      return 1;                                                             \
    }                                                                       \
  } while (0)
#define DK(x)                                                               \
  do {                                                                      \
    CUresult e_ = (x);                                                      \
    if (e_ != CUDA_SUCCESS) {                                               \
      const char* s_ = nullptr;                                             \
      cuGetErrorString(e_, &s_);                                            \
      g_err = std::string(#x) + ": " + (s_ ? s_ : "?");                     \
      return 1;                                                             \
    }                                                                       \
  } while (0)

CUfunction fn(Mod& m, const char* name) {
  CUfunction f = nullptr;
  if (cuModuleGetFunction(&f, m.m, name) != CUDA_SUCCESS) return nullptr;
  return f;
}

template <typename... A>
CUresult launch(CUfunction f, unsigned grid, unsigned block, A... args) {
  if (!f) return CUDA_ERROR_NOT_FOUND;
  if (grid == 0) return CUDA_SUCCESS;  // the reference launches empty grids (n == 1) and ignores the error
  void* p[] = {(void*)&args...};
  return cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, nullptr, p, nullptr);
}

int load(Mod& m, const std::string& path) {
  if (m.m) return 0;
  DK(cuModuleLoad(&m.m, path.c_str()));
  return 0;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

const char* ref_error(void) { return g_err.c_str(); }

// Load the four fatbins from `dir` (suffix "" = default flags, "_fast" = Release flags).
int ref_init(const char* dir, const char* suffix) {
  CK(cudaSetDevice(0));
  CK(cudaFree(nullptr));
  std::string d(dir), s(suffix ? suffix : "");
  g_dir = d;
  if (load(g_lbvh, d + "/ref_lbvh" + s + ".fatbin")) return 1;
  if (load(g_plus, d + "/ref_lbvh_plus" + s + ".fatbin")) return 1;
  if (load(g_ploc, d + "/ref_ploc" + s + ".fatbin")) return 1;
  if (load(g_render, d + "/ref_render" + s + ".fatbin")) return 1;
  return 0;
}

// LBVHBuilderCUDA::build.  ms[0] = getLastBuildTimeMS (sum of its event intervals), ms[1..5] =
// bounds, morton, sort, topology, refit, ms[6] = wall time of the whole build() call.
int ref_lbvh(const float* const* hv, uint32_t n, void* out_nodes, uint32_t* out_idx, float* ms) {
  double w0 = now_ms();
  const int bs = 256;
  const int grid = (int)((n + bs - 1) / bs);
  // prepareData (:334-374)
  float* dv[9];
  for (int k = 0; k < 9; ++k) CK(cudaMalloc(&dv[k], (size_t)n * 4));
  for (int k = 0; k < 9; ++k) CK(cudaMemcpy(dv[k], hv[k], (size_t)n * 4, cudaMemcpyHostToDevice));
  Box* boxes; F3* cent; uint32_t *codes, *idx; LNode* nodes; int* flags;
  CK(cudaMalloc(&boxes, (size_t)n * sizeof(Box)));
  CK(cudaMalloc(&cent, (size_t)n * sizeof(F3)));
  CK(cudaMalloc(&codes, (size_t)n * 4));
  CK(cudaMalloc(&idx, (size_t)n * 4));
  CK(cudaMalloc(&nodes, (2 * (size_t)n - 1) * sizeof(LNode)));
  CK(cudaMalloc(&flags, (2 * (size_t)n - 1) * sizeof(int)));
  DK(launch(fn(g_lbvh, "_Z12kFillZero_ntPii"), grid, bs, flags, (int)(2 * n - 1)));
  CK(cudaDeviceSynchronize());
  Tris t;
  for (int k = 0; k < 9; ++k) t.v[k] = dv[k];
  // runCompute (:376-463)
  cudaEvent_t ev[6];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0]));
  DK(launch(fn(g_lbvh, "_Z29kComputeBoundsAndCentroids_nt18TrianglesSoADeviceiP7AABB_cwP9float3_cw"), grid, bs, t,
            (int)n, boxes, cent));
  Box* red;
  CK(cudaMalloc(&red, (size_t)grid * sizeof(Box)));
  DK(launch(fn(g_lbvh, "_Z22kReduceBounds_Step1_ntPK7AABB_cwPS_i"), grid, bs, (const Box*)boxes, red, (int)n));
  if (grid > 1) DK(launch(fn(g_lbvh, "_Z22kReduceBounds_Step2_ntP7AABB_cwi"), 1, bs, red, grid));
  Box scene;
  CK(cudaMemcpy(&scene, red, sizeof(Box), cudaMemcpyDeviceToHost));
  CK(cudaFree(red));
  CK(cudaEventRecord(ev[1]));
  DK(launch(fn(g_lbvh, "_Z22kComputeMortonCodes_ntPK9float3_cwi7AABB_cwPjS3_"), grid, bs, (const F3*)cent, (int)n,
            scene, codes, idx));
  CK(cudaEventRecord(ev[2]));
  uint32_t *codes_out, *idx_out;
  CK(cudaMalloc(&codes_out, (size_t)n * 4));
  CK(cudaMalloc(&idx_out, (size_t)n * 4));
  void* temp = nullptr;
  size_t temp_bytes = 0;
  CK(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, codes, codes_out, idx, idx_out, (int)n));
  CK(cudaMalloc(&temp, temp_bytes));
  CK(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, codes, codes_out, idx, idx_out, (int)n));
  CK(cudaMemcpy(codes, codes_out, (size_t)n * 4, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(idx, idx_out, (size_t)n * 4, cudaMemcpyDeviceToDevice));
  CK(cudaFree(temp));
  CK(cudaFree(codes_out));
  CK(cudaFree(idx_out));
  CK(cudaEventRecord(ev[3]));
  const int igrid = (int)((n - 1 + bs - 1) / bs);
  DK(launch(fn(g_lbvh, "_Z22kBuildInternalNodes_ntPKjS0_P8LBVHNodei"), igrid, bs, (const uint32_t*)codes,
            (const uint32_t*)idx, nodes, (int)n));
  DK(launch(fn(g_lbvh, "_Z17kInitLeafNodes_ntP8LBVHNodePK7AABB_cwPKji"), grid, bs, nodes, (const Box*)boxes,
            (const uint32_t*)idx, (int)n));
  CK(cudaEventRecord(ev[4]));
  DK(launch(fn(g_lbvh, "_Z18kRefitHierarchy_ntP8LBVHNodePii"), grid, bs, nodes, flags, (int)n));
  CK(cudaEventRecord(ev[5]));
  CK(cudaEventSynchronize(ev[5]));
  float tot = 0;
  for (int k = 0; k < 5; ++k) {
    float a = 0;
    CK(cudaEventElapsedTime(&a, ev[k], ev[k + 1]));
    if (ms) ms[1 + k] = a;
    tot += a;
  }
  if (ms) ms[0] = tot;
  // downloadResults (:465-482): LBVHNode -> BVHNode
  std::vector<LNode> ln(2 * (size_t)n - 1);
  CK(cudaMemcpy(ln.data(), nodes, ln.size() * sizeof(LNode), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(out_idx, idx, (size_t)n * 4, cudaMemcpyDeviceToHost));
  Node* on = reinterpret_cast<Node*>(out_nodes);
  for (size_t k = 0; k < ln.size(); ++k) {
    memset(&on[k], 0, sizeof(Node));
    on[k].box = ln[k].box;
    on[k].l = (int32_t)ln[k].l;
    on[k].r = (int32_t)ln[k].r;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int k = 0; k < 9; ++k) cudaFree(dv[k]);
  cudaFree(boxes); cudaFree(cent); cudaFree(codes); cudaFree(idx); cudaFree(nodes); cudaFree(flags);
  CK(cudaDeviceSynchronize());
  if (ms) ms[6] = (float)(now_ms() - w0);
  return 0;
}

// LBVHPlusBuilderCUDA::build.  ms[0] = getLastBuildTimeMS, ms[1..6] = its intervals,
// ms[7] = wall time of build().
int ref_lbvh_plus(const float* const* hv, uint32_t n, void* out_nodes, uint32_t* out_idx, float* ms) {
  double w0 = now_ms();
  const int bs = 256;
  const int grid = (int)((n + bs - 1) / bs);
  thrust::device_vector<float> dv[9];
  for (int k = 0; k < 9; ++k) dv[k].assign(hv[k], hv[k] + n);
  thrust::device_vector<Box> boxes(n);
  thrust::device_vector<F3> cent(n);
  thrust::device_vector<unsigned long> codes(n);
  thrust::device_vector<uint32_t> idx(n);
  thrust::device_vector<LNode> nodes(2 * (size_t)n - 1);
  thrust::device_vector<int> counters(2 * (size_t)n - 1);
  Tris t;
  for (int k = 0; k < 9; ++k) t.v[k] = thrust::raw_pointer_cast(dv[k].data());
  Box* pb = thrust::raw_pointer_cast(boxes.data());
  F3* pc = thrust::raw_pointer_cast(cent.data());
  unsigned long* pk = thrust::raw_pointer_cast(codes.data());
  uint32_t* pi = thrust::raw_pointer_cast(idx.data());
  LNode* pn = thrust::raw_pointer_cast(nodes.data());
  int* pf = thrust::raw_pointer_cast(counters.data());
  cudaEvent_t ev[7];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0]));
  DK(launch(fn(g_plus, "_Z28kComputeBoundsAndCentroids_P18TrianglesSoADeviceiP7AABB_cwP9float3_cw"), grid, bs, t,
            (int)n, pb, pc));
  Box init;
  init.mn = F3{FLT_MAX, FLT_MAX, FLT_MAX};
  init.mx = F3{-FLT_MAX, -FLT_MAX, -FLT_MAX};
  Box scene = thrust::reduce(boxes.begin(), boxes.end(), init, BoxUnion());
  CK(cudaEventRecord(ev[1]));
  DK(launch(fn(g_plus, "_Z21kComputeMortonCodes_PPK9float3_cwi7AABB_cwPmPj"), grid, bs, (const F3*)pc, (int)n, scene,
            pk, pi));
  CK(cudaEventRecord(ev[2]));
  thrust::sort_by_key(codes.begin(), codes.end(), idx.begin());
  CK(cudaEventRecord(ev[3]));
  DK(launch(fn(g_plus, "_Z21kBuildInternalNodes_PPKmPKjP8LBVHNodei"), grid, bs, (const unsigned long*)pk,
            (const uint32_t*)pi, pn, (int)n));
  DK(launch(fn(g_plus, "_Z16kInitLeafNodes_PP8LBVHNodePK7AABB_cwPKji"), grid, bs, pn, (const Box*)pb,
            (const uint32_t*)pi, (int)n));
  CK(cudaEventRecord(ev[4]));
  thrust::fill(counters.begin(), counters.end(), 0);
  DK(launch(fn(g_plus, "_Z17kRefitAndOptimizeP8LBVHNodePiib"), grid, bs, pn, pf, (int)n, false));
  CK(cudaEventRecord(ev[5]));
  thrust::fill(counters.begin(), counters.end(), 0);
  DK(launch(fn(g_plus, "_Z17kRefitAndOptimizeP8LBVHNodePiib"), grid, bs, pn, pf, (int)n, true));
  CK(cudaEventRecord(ev[6]));
  CK(cudaEventSynchronize(ev[6]));
  float tot = 0;
  for (int k = 0; k < 6; ++k) {
    float a = 0;
    CK(cudaEventElapsedTime(&a, ev[k], ev[k + 1]));
    if (ms) ms[1 + k] = a;
    tot += a;
  }
  if (ms) ms[0] = tot;
  std::vector<LNode> ln(nodes.size());
  thrust::copy(nodes.begin(), nodes.end(), ln.begin());
  thrust::copy(idx.begin(), idx.end(), out_idx);
  Node* on = reinterpret_cast<Node*>(out_nodes);
  for (size_t k = 0; k < ln.size(); ++k) {
    memset(&on[k], 0, sizeof(Node));
    on[k].box = ln[k].box;
    on[k].l = (int32_t)ln[k].l;
    on[k].r = (int32_t)ln[k].r;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  CK(cudaDeviceSynchronize());
  if (ms) ms[7] = (float)(now_ms() - w0);
  return 0;
}

// PLOCBuilderCUDA::build.  Returns 2 if the loop exceeds max_iter (the reference would spin
// forever).  *n_nodes = allocated nodes; ms[0] = getLastBuildTimeMS (includes the upload).
int ref_ploc(const float* const* hv, uint32_t n, int radius, int max_iter, void* out_nodes, uint32_t* out_idx,
             uint32_t* n_nodes, int* iterations, float* ms) {
  double w0 = now_ms();
  *n_nodes = 0;
  if (n == 0) return 0;
  const int bs = 256;
  const int grid = (int)((n + bs - 1) / bs);
  float* dv[9];
  for (int k = 0; k < 9; ++k) CK(cudaMalloc(&dv[k], (size_t)n * 4));
  Box *boxes, *cbox, *cbox2; F3* cent; uint32_t *codes, *idx; int *cid, *cid2, *nb, *valid, *offs, *next;
  float* dist; Node* nodes;
  CK(cudaMalloc(&boxes, (size_t)n * sizeof(Box)));
  CK(cudaMalloc(&cent, (size_t)n * sizeof(F3)));
  CK(cudaMalloc(&codes, (size_t)n * 4));
  CK(cudaMalloc(&idx, (size_t)n * 4));
  CK(cudaMalloc(&cbox, (size_t)n * sizeof(Box)));
  CK(cudaMalloc(&cid, (size_t)n * 4));
  CK(cudaMalloc(&cbox2, (size_t)n * sizeof(Box)));
  CK(cudaMalloc(&cid2, (size_t)n * 4));
  CK(cudaMalloc(&nb, (size_t)n * 4));
  CK(cudaMalloc(&dist, (size_t)n * 4));
  CK(cudaMalloc(&valid, (size_t)n * 4));
  CK(cudaMalloc(&offs, (size_t)n * 4));
  CK(cudaMalloc(&nodes, (2 * (size_t)n - 1) * sizeof(Node)));
  CK(cudaMalloc(&next, 4));
  float t_init = 0, t_search = 0, t_merge = 0, t_compact = 0, a = 0;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0));
  for (int k = 0; k < 9; ++k) CK(cudaMemcpy(dv[k], hv[k], (size_t)n * 4, cudaMemcpyHostToDevice));
  Tris t;
  for (int k = 0; k < 9; ++k) t.v[k] = dv[k];
  DK(launch(fn(g_ploc, "_Z30kComputeAABBsAndCentroids_ploc18TrianglesSoADeviceiP7AABB_cwP9float3_cw"), grid, bs, t,
            (int)n, boxes, cent));
  Box* red;
  CK(cudaMalloc(&red, (size_t)grid * sizeof(Box)));
  DK(launch(fn(g_ploc, "_Z24kReduceBounds_Step1_plocPK7AABB_cwPS_i"), grid, bs, (const Box*)boxes, red, (int)n));
  if (grid > 1) DK(launch(fn(g_ploc, "_Z24kReduceBounds_Step2_plocP7AABB_cwi"), 1, bs, red, grid));
  Box scene;
  CK(cudaMemcpy(&scene, red, sizeof(Box), cudaMemcpyDeviceToHost));
  CK(cudaFree(red));
  DK(launch(fn(g_ploc, "_Z23kAssignMortonCodes_plocPK9float3_cwi7AABB_cwPjS3_"), grid, bs, (const F3*)cent, (int)n,
            scene, codes, idx));
  {
    thrust::device_ptr<uint32_t> tk(codes), ti(idx);
    thrust::sort_by_key(tk, tk + n, ti);
  }
  DK(launch(fn(g_ploc, "_Z12kGatherAABBsPKjPK7AABB_cwPS1_i"), grid, bs, (const uint32_t*)idx, (const Box*)boxes, cbox,
            (int)n));
  DK(launch(fn(g_ploc, "_Z19kInitLeafNodes_plocP7BVHNodePK7AABB_cwPKji"), grid, bs, nodes, (const Box*)cbox,
            (const uint32_t*)idx, (int)n));
  DK(launch(fn(g_ploc, "_Z19kInitializeSequencePii"), grid, bs, cid, (int)n));
  int init_cnt = (int)n;
  CK(cudaMemcpy(next, &init_cnt, 4, cudaMemcpyHostToDevice));
  void* temp = nullptr;
  size_t temp_bytes = 0;
  CK(cub::DeviceScan::ExclusiveSum(temp, temp_bytes, valid, offs, (int)n));
  CK(cudaMalloc(&temp, temp_bytes));
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  CK(cudaEventElapsedTime(&a, e0, e1));
  t_init = a;
  int cur = (int)n, it = 0, rc = 0;
  CUfunction f_nn = fn(g_ploc, "_Z26kFindNearestNeighbors_plocPK7AABB_cwiiPiPf");
  CUfunction f_merge = fn(g_ploc, "_Z19kMergeClusters_plocPKiPKfiPiP7AABB_cwP7BVHNodeS3_S3_");
  CUfunction f_ci = fn(g_ploc, "_Z15kCompactIndicesPKiPiS0_S0_i");
  CUfunction f_ca = fn(g_ploc, "_Z13kCompactAABBsPK7AABB_cwPS_PKiS4_i");
  while (cur > 1) {
    if (max_iter > 0 && it >= max_iter) { rc = 2; break; }
    int nbk = (cur + bs - 1) / bs;
    CK(cudaEventRecord(e0));
    DK(launch(f_nn, nbk, bs, (const Box*)cbox, cur, radius, nb, dist));
    CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaEventElapsedTime(&a, e0, e1)); t_search += a;
    CK(cudaEventRecord(e0));
    DK(launch(f_merge, nbk, bs, (const int*)nb, (const float*)dist, cur, cid, cbox, nodes, next, valid));
    CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaEventElapsedTime(&a, e0, e1)); t_merge += a;
    CK(cudaEventRecord(e0));
    CK(cub::DeviceScan::ExclusiveSum(temp, temp_bytes, valid, offs, cur));
    int lv = 0, lo = 0;
    CK(cudaMemcpy(&lv, valid + cur - 1, 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&lo, offs + cur - 1, 4, cudaMemcpyDeviceToHost));
    int nc = lo + lv;
    DK(launch(f_ci, nbk, bs, (const int*)cid, cid2, (const int*)valid, (const int*)offs, cur));
    DK(launch(f_ca, nbk, bs, (const Box*)cbox, cbox2, (const int*)valid, (const int*)offs, cur));
    std::swap(cid, cid2);
    std::swap(cbox, cbox2);
    CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaEventElapsedTime(&a, e0, e1)); t_compact += a;
    it++;
    if (nc >= cur) { rc = 3; break; }
    cur = nc;
  }
  if (ms) {
    ms[0] = t_init + t_search + t_merge + t_compact;
    ms[1] = t_init; ms[2] = t_search; ms[3] = t_merge; ms[4] = t_compact;
  }
  if (iterations) *iterations = it;
  if (rc == 0) {
    int alloc = 0;
    CK(cudaMemcpy(&alloc, next, 4, cudaMemcpyDeviceToHost));
    Node* on = reinterpret_cast<Node*>(out_nodes);
    CK(cudaMemcpy(on, nodes, (size_t)alloc * sizeof(Node), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out_idx, idx, (size_t)n * 4, cudaMemcpyDeviceToHost));
    // root (last allocated) to index 0 (:563-582)
    if (alloc > 1) {
      int root = alloc - 1;
      std::swap(on[0], on[root]);
      for (int k = 0; k < alloc; ++k) {
        Node& nd = on[k];
        if (nd.l < 0) continue;
        if (nd.l == 0) nd.l = root; else if (nd.l == root) nd.l = 0;
        if (nd.r >= 0) { if (nd.r == 0) nd.r = root; else if (nd.r == root) nd.r = 0; }
      }
    }
    *n_nodes = (uint32_t)alloc;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int k = 0; k < 9; ++k) cudaFree(dv[k]);
  cudaFree(boxes); cudaFree(cent); cudaFree(codes); cudaFree(idx); cudaFree(cbox); cudaFree(cid); cudaFree(cbox2);
  cudaFree(cid2); cudaFree(nb); cudaFree(dist); cudaFree(valid); cudaFree(offs); cudaFree(nodes); cudaFree(next);
  cudaFree(temp);
  CK(cudaDeviceSynchronize());
  if (ms) ms[5] = (float)(now_ms() - w0);
  return rc;
}

// renderImage's kernel (src/render_engine.cu:744-807): per-pixel node visits, AABB tests,
// triangle tests and RGB for one shading mode.  ms[0] = kernel time.
int ref_render(const void* host_nodes, uint32_t n_nodes, const float* const* hv, uint32_t n, const float* cam10,
               int width, int height, int mode, float scene_diag, const float* light3, int* visits, int* aabb,
               int* tri, float* rgb, float* ms) {
  const size_t np = (size_t)width * height;
  Node* dn;
  CK(cudaMalloc(&dn, (size_t)n_nodes * sizeof(Node)));
  CK(cudaMemcpy(dn, host_nodes, (size_t)n_nodes * sizeof(Node), cudaMemcpyHostToDevice));
  float* dv[9];
  for (int k = 0; k < 9; ++k) {
    CK(cudaMalloc(&dv[k], (size_t)n * 4));
    CK(cudaMemcpy(dv[k], hv[k], (size_t)n * 4, cudaMemcpyHostToDevice));
  }
  Tris t;
  for (int k = 0; k < 9; ++k) t.v[k] = dv[k];
  float* drgb; int *dvis, *dat, *dtt;
  CK(cudaMalloc(&drgb, np * 3 * 4));
  CK(cudaMalloc(&dvis, np * 4));
  CK(cudaMalloc(&dat, np * 4));
  CK(cudaMalloc(&dtt, np * 4));
  CK(cudaMemset(drgb, 0, np * 12)); CK(cudaMemset(dvis, 0, np * 4)); CK(cudaMemset(dat, 0, np * 4));
  CK(cudaMemset(dtt, 0, np * 4));
  Cam cam;
  cam.eye = F3{cam10[0], cam10[1], cam10[2]};
  cam.look = F3{cam10[3], cam10[4], cam10[5]};
  cam.up = F3{cam10[6], cam10[7], cam10[8]};
  cam.fov = cam10[9];
  F3 light{light3[0], light3[1], light3[2]};
  CUfunction f = fn(g_render, "_Z13kRenderKernelPK7BVHNodei18TrianglesSoADevice6Cameraiiif9float3_cwPfPiS6_S6_");
  if (!f) { g_err = "kRenderKernel not found"; return 1; }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const Node* cdn = dn;
  int nn = (int)n_nodes;
  void* p[] = {(void*)&cdn, (void*)&nn, (void*)&t, (void*)&cam, (void*)&width, (void*)&height, (void*)&mode,
               (void*)&scene_diag, (void*)&light, (void*)&drgb, (void*)&dvis, (void*)&dat, (void*)&dtt};
  CK(cudaEventRecord(e0));
  DK(cuLaunchKernel(f, (width + 15) / 16, (height + 15) / 16, 1, 16, 16, 1, 0, nullptr, p, nullptr));
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float a = 0;
  CK(cudaEventElapsedTime(&a, e0, e1));
  if (ms) ms[0] = a;
  CK(cudaMemcpy(visits, dvis, np * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(aabb, dat, np * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(tri, dtt, np * 4, cudaMemcpyDeviceToHost));
  if (rgb) CK(cudaMemcpy(rgb, drgb, np * 12, cudaMemcpyDeviceToHost));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dn);
  for (int k = 0; k < 9; ++k) cudaFree(dv[k]);
  cudaFree(drgb); cudaFree(dvis); cudaFree(dat); cudaFree(dtt);
  return 0;
}

// generateRay (src/render_engine.cu:155-188) for every pixel of a width x height image, run by the
// reference's own device code (ref_trace.fatbin, built from ref_trace_shim.cu).  Host outputs.
int ref_generate_rays(const float* cam10, int width, int height, float* const* out6) {
  if (load(g_trace, g_dir + "/ref_trace.fatbin")) return 1;
  const size_t np = (size_t)width * height;
  float* d[6];
  for (int k = 0; k < 6; ++k) CK(cudaMalloc(&d[k], np * 4));
  Cam cam;
  cam.eye = F3{cam10[0], cam10[1], cam10[2]};
  cam.look = F3{cam10[3], cam10[4], cam10[5]};
  cam.up = F3{cam10[6], cam10[7], cam10[8]};
  cam.fov = cam10[9];
  DK(launch(fn(g_trace, "shim_generate_rays"), (unsigned)((np + 255) / 256), 256u, cam, width, height, d[0], d[1],
            d[2], d[3], d[4], d[5]));
  CK(cudaDeviceSynchronize());
  for (int k = 0; k < 6; ++k) CK(cudaMemcpy(out6[k], d[k], np * 4, cudaMemcpyDeviceToHost));
  for (int k = 0; k < 6; ++k) cudaFree(d[k]);
  return 0;
}

// traverseBVH (src/render_engine.cu:289-356) on nr given rays (six host SoA arrays), run by the
// reference's own device code.  Outputs per ray: t, prim (-1 on a miss), node visits, AABB tests,
// triangle tests, and the hit normal (3 floats, 0 on a miss).  ms[0] = kernel time.
int ref_traverse(const void* host_nodes, uint32_t n_nodes, const float* const* hv, uint32_t n,
                 const float* const* rays6, uint32_t nr, float* t, int* prim, int* visits, int* aabb, int* tri,
                 float* normal, float* ms) {
  if (load(g_trace, g_dir + "/ref_trace.fatbin")) return 1;
  Node* dn;
  CK(cudaMalloc(&dn, (size_t)n_nodes * sizeof(Node) + 16));
  CK(cudaMemcpy(dn, host_nodes, (size_t)n_nodes * sizeof(Node), cudaMemcpyHostToDevice));
  Tris tr;
  for (int k = 0; k < 9; ++k) {
    CK(cudaMalloc(&tr.v[k], (size_t)n * 4 + 16));
    CK(cudaMemcpy(tr.v[k], hv[k], (size_t)n * 4, cudaMemcpyHostToDevice));
  }
  float* dr[6];
  for (int k = 0; k < 6; ++k) {
    CK(cudaMalloc(&dr[k], (size_t)nr * 4 + 16));
    CK(cudaMemcpy(dr[k], rays6[k], (size_t)nr * 4, cudaMemcpyHostToDevice));
  }
  float *dt, *dnorm;
  int *dp, *dv, *da, *dtt;
  CK(cudaMalloc(&dt, (size_t)nr * 4 + 16));
  CK(cudaMalloc(&dp, (size_t)nr * 4 + 16));
  CK(cudaMalloc(&dv, (size_t)nr * 4 + 16));
  CK(cudaMalloc(&da, (size_t)nr * 4 + 16));
  CK(cudaMalloc(&dtt, (size_t)nr * 4 + 16));
  CK(cudaMalloc(&dnorm, (size_t)nr * 12 + 16));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const Node* cdn = dn;
  const float *r0 = dr[0], *r1 = dr[1], *r2 = dr[2], *r3 = dr[3], *r4 = dr[4], *r5 = dr[5];
  CK(cudaEventRecord(e0));
  DK(launch(fn(g_trace, "shim_traverse"), (nr + 127) / 128, 128u, cdn, (int)n_nodes, tr, r0, r1, r2, r3, r4, r5,
            (int)nr, dt, dp, dv, da, dtt, dnorm));
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float a = 0;
  CK(cudaEventElapsedTime(&a, e0, e1));
  if (ms) ms[0] = a;
  CK(cudaMemcpy(t, dt, (size_t)nr * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(prim, dp, (size_t)nr * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(visits, dv, (size_t)nr * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(aabb, da, (size_t)nr * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(tri, dtt, (size_t)nr * 4, cudaMemcpyDeviceToHost));
  if (normal) CK(cudaMemcpy(normal, dnorm, (size_t)nr * 12, cudaMemcpyDeviceToHost));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dn);
  for (int k = 0; k < 9; ++k) cudaFree(tr.v[k]);
  for (int k = 0; k < 6; ++k) cudaFree(dr[k]);
  cudaFree(dt); cudaFree(dp); cudaFree(dv); cudaFree(da); cudaFree(dtt); cudaFree(dnorm);
  return 0;
}

// Reference PLOC nearest-neighbour kernel on given cluster boxes (used to pin the area form).
int ref_ploc_nn(const void* host_boxes, int n, int radius, int* nbr, float* dist) {
  Box* db;
  int* dn;
  float* dd;
  CK(cudaMalloc(&db, (size_t)n * sizeof(Box)));
  CK(cudaMalloc(&dn, (size_t)n * 4));
  CK(cudaMalloc(&dd, (size_t)n * 4));
  CK(cudaMemcpy(db, host_boxes, (size_t)n * sizeof(Box), cudaMemcpyHostToDevice));
  DK(launch(fn(g_ploc, "_Z26kFindNearestNeighbors_plocPK7AABB_cwiiPiPf"), (unsigned)((n + 255) / 256), 256u,
            (const Box*)db, n, radius, dn, dd));
  CK(cudaMemcpy(nbr, dn, (size_t)n * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(dist, dd, (size_t)n * 4, cudaMemcpyDeviceToHost));
  cudaFree(db); cudaFree(dn); cudaFree(dd);
  return 0;
}

}  // extern "C"
