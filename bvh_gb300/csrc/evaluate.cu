// evaluate.cu -- tree quality statistics on the GPU.
//
// Reference: BVHEvaluator::computeSAH (src/evaluator.cpp:38-88) and computeDepthStats
// (:90-113): SAH = sum over internal nodes of 3 * A(node)/A(root) plus sum over leaves of
// 2 * A(leaf)/A(root), node/leaf counts, maximum and average leaf depth.  The reference adds the
// terms in float in depth-first order on one host thread; here every node's term is formed with
// the host's rounding (surface area without contraction, the float division) and summed in
// double in parallel, so the SAH agrees with the host evaluator to float rounding of the sum.
// A node's depth is the length of its walk to the root through a parent array.
#include <algorithm>

#include "lbvh.cuh"

namespace bvhgb {

// AABB_cw::surfaceArea as the host evaluator computes it (no fused multiply-add).
__device__ __forceinline__ float area_plain(float4 lo, float4 hi) {
  const float x = __fsub_rn(hi.x, lo.x), y = __fsub_rn(hi.y, lo.y), z = __fsub_rn(hi.z, lo.z);
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(x, y), __fmul_rn(y, z)), __fmul_rn(z, x)));
}

// parent[] of every node referenced as a child; parent[root] = -1.  Child indices outside
// [0, n) are ignored, as in the reference recursion (:80-85).
__global__ void k_parents(const Node* __restrict__ nodes, uint32_t n, int32_t* __restrict__ parent) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int2 ch = __ldg(reinterpret_cast<const int2*>(&nodes[k].left));
    if (ch.x < 0) continue;  // leaf
    if (ch.x < (int32_t)n) parent[ch.x] = (int32_t)k;
    if (ch.y >= 0 && ch.y < (int32_t)n) parent[ch.y] = (int32_t)k;
  }
}

// Per node: depth (walk to the root through parent[]), SAH term; block sums in double.
__global__ void __launch_bounds__(256) k_eval(const Node* __restrict__ nodes, uint32_t n,
                                              const int32_t* __restrict__ parent, double* __restrict__ acc,
                                              unsigned long long* __restrict__ cnt, uint32_t* __restrict__ max_depth) {
  __shared__ double s_sum[8], s_depth[8];
  __shared__ unsigned long long s_leaves[8], s_reach[8];
  __shared__ uint32_t s_max[8];
  const float4 rlo = __ldg(reinterpret_cast<const float4*>(nodes)), rhi = __ldg(reinterpret_cast<const float4*>(nodes) + 1);
  const float root_area = area_plain(rlo, rhi);
  double sum = 0.0, dsum = 0.0;
  unsigned long long leaves = 0, reach = 0;
  uint32_t dmax = 0;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    // reachable from the root?  walk up; unreachable nodes do not count (as in the reference)
    uint32_t depth = 0;
    int32_t x = (int32_t)k;
    bool ok = true;
    while (x != 0) {
      x = __ldg(parent + x);
      if (x < 0 || ++depth > n) { ok = false; break; }
    }
    if (!ok) continue;
    reach++;
    const float4* p = reinterpret_cast<const float4*>(nodes + k);
    const float prob = __fdiv_rn(area_plain(__ldg(p), __ldg(p + 1)), root_area);
    const bool leaf = __ldg(&nodes[k].left) < 0;
    sum += (double)__fmul_rn(prob, leaf ? 2.0f : 3.0f);
    if (leaf) {
      leaves++;
      dsum += (double)depth;
    }
    dmax = max(dmax, depth);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    leaves += __shfl_xor_sync(0xffffffffu, leaves, o);
    reach += __shfl_xor_sync(0xffffffffu, reach, o);
    dmax = max(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
  }
  if (lane == 0) {
    s_sum[w] = sum; s_depth[w] = dsum; s_leaves[w] = leaves; s_reach[w] = reach; s_max[w] = dmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      sum += s_sum[k]; dsum += s_depth[k]; leaves += s_leaves[k]; reach += s_reach[k]; dmax = max(dmax, s_max[k]);
    }
    atomicAdd(acc, sum);
    atomicAdd(acc + 1, dsum);
    atomicAdd(cnt, leaves);
    atomicAdd(cnt + 1, reach);
    atomicMax(max_depth, dmax);
  }
}

size_t evaluate_scratch_bytes(uint32_t n_nodes) { return 64 + (size_t)n_nodes * 4; }

cudaError_t evaluate_tree(const Node* nodes, uint32_t n_nodes, void* scratch, cudaStream_t st, EvalResult* out) {
  *out = EvalResult{};
  if (n_nodes == 0) return cudaSuccess;
  char* base = static_cast<char*>(scratch);
  double* acc = reinterpret_cast<double*>(base);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(base + 16);
  uint32_t* maxd = reinterpret_cast<uint32_t*>(base + 32);
  int32_t* parent = reinterpret_cast<int32_t*>(base + 64);
  cudaError_t e = cudaMemsetAsync(base, 0, 64, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(parent, 0xff, (size_t)n_nodes * 4, st);
  if (e != cudaSuccess) return e;
  const uint32_t grid = std::min<uint32_t>(div_up(n_nodes, 256), 152 * 8);
  k_parents<<<grid, 256, 0, st>>>(nodes, n_nodes, parent);
  k_eval<<<grid, 256, 0, st>>>(nodes, n_nodes, parent, acc, cnt, maxd);
  double hacc[2];
  unsigned long long hcnt[2];
  uint32_t hmax = 0;
  Node root;
  if ((e = cudaMemcpyAsync(hacc, acc, 16, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(hcnt, cnt, 16, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&hmax, maxd, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&root, nodes, sizeof(Node), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return e;
  // computeSAH returns 0 when the root area is not positive (src/evaluator.cpp:44-45)
  const float x = root.hi.x - root.lo.x, y = root.hi.y - root.lo.y, z = root.hi.z - root.lo.z;
  const float ra = 2.0f * ((x * y + y * z) + z * x);
  out->sah = ra > 0.0f ? hacc[0] : 0.0;
  out->nodes = hcnt[1];
  out->leaves = hcnt[0];
  out->max_depth = hmax;
  out->avg_leaf_depth = hcnt[0] ? hacc[1] / (double)hcnt[0] : 0.0;
  return cudaSuccess;
}

}  // namespace bvhgb
