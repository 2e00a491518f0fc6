// batched.cu -- many independent meshes built together (no reference counterpart).
//
// Every mesh gets exactly the tree LBVHBuilderCUDA would build for it alone (30-bit Morton
// normalised to that mesh's own box, src/cuda/lbvh_builder.cu:167-181; Karras topology with
// ties on the mesh-local original index, :33-43).  All meshes share one launch sequence:
//   k_seg_init    per-mesh boxes to (FLT_MAX, -FLT_MAX); sort scratch zeroed
//   k_seg_bounds  per-mesh scene boxes (warp-aggregated, ordered-int atomics = fminf/fmaxf)
//   k_seg_morton  key = mesh << 30 | code30, triangle boxes, radix histograms
//   k_onesweep    ceil((30 + mesh bits) / 8) stable passes over the 64-bit keys
//   k_delta/k_emit  segmented Karras emission: delta = -1 across meshes, node ids per mesh
// The sequence has no host synchronisation and can be captured into a CUDA graph.  Batched PLOC
// (ploc.cu) shares everything up to the sort and then clusters all meshes at once.
#include <algorithm>
#include <cstring>

#include "emit.cuh"
#include "lbvh.cuh"

namespace bvhgb {

// fminf/fmaxf through integer atomics: -0 < +0, NaN ignored (callers skip NaN).
__device__ __forceinline__ void atomic_fmin(float* a, float v) {
  if (signbit(v)) atomicMax(reinterpret_cast<unsigned int*>(a), __float_as_uint(v));
  else atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
}
__device__ __forceinline__ void atomic_fmax(float* a, float v) {
  if (signbit(v)) atomicMin(reinterpret_cast<unsigned int*>(a), __float_as_uint(v));
  else atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
}

__global__ void k_seg_init(float* __restrict__ mbox, uint32_t count, uint32_t* __restrict__ scratch, ScratchLayout L) {
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gsz = gridDim.x * blockDim.x;
  for (uint32_t m = gtid; m < count; m += gsz) {
    float4* b = reinterpret_cast<float4*>(mbox + 8 * (size_t)m);
    b[0] = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
    b[1] = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
  }
  for (size_t w = L.zero_begin + gtid; w < L.zero_end; w += gsz) scratch[w] = 0;
  if (gtid == 0) {
    scratch[L.status] = 0;
    uint32_t e = scratch[L.epoch] + kEpochStride;
    scratch[L.epoch] = e < kEpochStride ? kEpochStride : e;
  }
}

// Block-wide min/max of six floats (fminf/fmaxf; NaN ignored); result valid in thread 0.
__device__ __forceinline__ void block_box_reduce(float v[6], float (*s_red)[6]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
      v[3 + k] = fmaxf(v[3 + k], __shfl_xor_sync(0xffffffffu, v[3 + k], o));
    }
  }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) s_red[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        v[k] = fminf(v[k], s_red[ww][k]);
        v[3 + k] = fmaxf(v[3 + k], s_red[ww][3 + k]);
      }
}

// Per-mesh scene boxes.  Persistent blocks walk work items (a mesh and a triangle range of at
// most kSegChunk); one set of atomics per item.
__global__ void __launch_bounds__(256) k_seg_bounds(MeshPtrs m, const SegItem* __restrict__ items, uint32_t n_items,
                                                    float* __restrict__ mbox) {
  __shared__ float s_red[8][6];
  for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const SegItem w = items[it];
    float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = w.begin + threadIdx.x; i < w.end; i += blockDim.x) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float a0 = __ldcs(m.v[k] + i), a1 = __ldcs(m.v[3 + k] + i), a2 = __ldcs(m.v[6 + k] + i);
        v[k] = fminf(v[k], fminf(a0, fminf(a1, a2)));
        v[3 + k] = fmaxf(v[3 + k], fmaxf(a0, fmaxf(a1, a2)));
      }
    }
    block_box_reduce(v, s_red);
    if (threadIdx.x == 0) {
      float* b = mbox + 8 * (size_t)w.mesh;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (v[k] == v[k]) atomic_fmin(b + k, v[k]);
        if (v[3 + k] == v[3 + k]) atomic_fmax(b + 4 + k, v[3 + k]);
      }
    }
    __syncthreads();
  }
}

// Keys mesh << 30 | code30 are written split: hkeys = key >> shift0 (the passes sort these 32
// bits) and, when shift0 > 0, lows = the rest, in input order.
__global__ void __launch_bounds__(256) k_seg_morton(MeshPtrs m, const SegItem* __restrict__ items, uint32_t n_items,
                                                    const float* __restrict__ mbox, int passes, int shift0,
                                                    uint32_t* __restrict__ hkeys, uint32_t* __restrict__ lows,
                                                    Box* __restrict__ boxes, uint32_t* __restrict__ scratch,
                                                    ScratchLayout L) {
  __shared__ uint32_t s_hist[kMaxPasses][256];
  __shared__ float s_scene[6];
  for (int k = threadIdx.x; k < kMaxPasses * 256; k += blockDim.x) (&s_hist[0][0])[k] = 0;
  for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const SegItem w = items[it];
    __syncthreads();
    if (threadIdx.x < 3) {
      const float* b = mbox + 8 * (size_t)w.mesh;
      const float mn = b[threadIdx.x];
      const float e = __fsub_rn(b[4 + threadIdx.x], mn);
      s_scene[threadIdx.x] = mn;
      s_scene[3 + threadIdx.x] = (e > 1e-6f) ? e : 1.0f;  // lbvh_builder.cu:175-177
    }
    __syncthreads();
    const unsigned long long mesh_bits = (unsigned long long)w.mesh << 30;
    for (uint32_t i = w.begin + threadIdx.x; i < w.end; i += blockDim.x) {
      float lo[3], hi[3], nc[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float a0 = __ldcs(m.v[k] + i), a1 = __ldcs(m.v[3 + k] + i), a2 = __ldcs(m.v[6 + k] + i);
        lo[k] = fminf(a0, fminf(a1, a2));
        hi[k] = fmaxf(a0, fmaxf(a1, a2));
        const float c = __fmul_rn(__fadd_rn(lo[k], hi[k]), 0.5f);
        nc[k] = __fdiv_rn(__fsub_rn(c, s_scene[k]), s_scene[3 + k]);
      }
      const unsigned long long key = mesh_bits | morton_code<30>(nc[0], nc[1], nc[2]);
      hkeys[i] = (uint32_t)(key >> shift0);
      if (shift0) lows[i] = (uint32_t)(key & ((1ull << shift0) - 1ull));
      float4* bp = reinterpret_cast<float4*>(boxes + i);
      bp[0] = make_float4(lo[0], lo[1], lo[2], 0.f);
      bp[1] = make_float4(hi[0], hi[1], hi[2], 0.f);
      for (int p = 0; p < passes; ++p) atomicAdd(&s_hist[p][(uint32_t)(key >> (shift0 + 8 * p)) & 255u], 1u);
    }
  }
  __syncthreads();
  uint32_t* gh = scratch + L.hist;
  for (int k = threadIdx.x; k < passes * 256; k += blockDim.x) {
    uint32_t c = (&s_hist[0][0])[k];
    if (c) atomicAdd(gh + k, c);
  }
}

// The per-mesh boxes, keys and sort shared by the batched LBVH and PLOC: on return the sorted
// (mesh, code30, index) order is in ws.vals[*fb] (global triangle indices) and ws.keys[*fb]
// holds the high 32 bits of the keys.
cudaError_t batched_prefix(Workspace& ws, const MeshPtrs& m, uint32_t n, uint32_t count, const SegItem* d_items,
                           uint32_t n_items, float* d_mbox, cudaStream_t st, StageEvents* evs, BatchedSort* out) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  int mbits = 1;
  while (mbits < 34 && (1ull << mbits) < count) ++mbits;
  // keys have 30 + mbits bits: up to 32 are sorted whole; longer keys are sorted by their high
  // 32 bits and the runs of equal high bits are then ordered by the rest (sort_fix_runs_split);
  // mbits <= 32 (count is 32-bit), so shift0 <= 30
  const int kbits = 30 + mbits;
  const int shift0 = kbits > 32 ? kbits - 32 : 0;
  const int passes = kbits > 32 ? 4 : (kbits + 7) / 8;
  L.zero_end = L.desc + (size_t)passes * div_up(std::max<uint32_t>(n, 1),
                                                 (uint32_t)sort_variant_tile(ws.sort_variant)) * 256;
  // the low key bits live at the start of the node buffer until the delta pass has read them
  uint32_t* lows = reinterpret_cast<uint32_t*>(ws.nodes);
  unsigned long long* run_scratch = reinterpret_cast<unsigned long long*>(
      reinterpret_cast<unsigned char*>(ws.nodes) + (((size_t)n * 4 + 15) & ~(size_t)15));
  if (evs && evs->use) cudaEventRecord(evs->ev[0], st);
  if ((e = epoch_tick(ws, st)) != cudaSuccess) return e;
  k_seg_init<<<152 * 4, 256, 0, st>>>(d_mbox, count, ws.scratch, L);
  const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(n_items, 152 * 8));
  k_seg_bounds<<<grid, 256, 0, st>>>(m, d_items, n_items, d_mbox);
  if (evs && evs->use) cudaEventRecord(evs->ev[1], st);
  k_seg_morton<<<grid, 256, 0, st>>>(m, d_items, n_items, d_mbox, passes, shift0,
                                     reinterpret_cast<uint32_t*>(ws.keys[0]), lows, ws.boxes, ws.scratch, L);
  if (evs && evs->use) cudaEventRecord(evs->ev[2], st);
  int fb = 0;
  if ((e = run_sort_u32(ws, n, passes, st, L, &fb)) != cudaSuccess) return e;
  const uint32_t* hkeys = reinterpret_cast<const uint32_t*>(ws.keys[fb]);
  if (shift0 > 0 &&
      (e = sort_fix_runs_split(hkeys, ws.vals[fb], lows, n, shift0,
                               reinterpret_cast<unsigned long long*>(ws.keys[fb ^ 1]), run_scratch, ws.vals[fb ^ 1],
                               reinterpret_cast<uint32_t*>(ws.delta), ws.scratch + L.counters + kLongRunCounter,
                               nullptr, st)) != cudaSuccess)
    return e;
  if (evs && evs->use) cudaEventRecord(evs->ev[3], st);
  out->fb = fb;
  out->shift0 = shift0;
  out->lows = lows;
  return cudaSuccess;
}

cudaError_t batched_build(Workspace& ws, const MeshPtrs& m, uint32_t n, const uint32_t* d_offsets, uint32_t count,
                          const SegItem* d_items, uint32_t n_items, float* d_mbox, uint32_t* d_indices,
                          cudaStream_t st, StageEvents* evs) {
  BatchedSort bs;
  cudaError_t e = batched_prefix(ws, m, n, count, d_items, n_items, d_mbox, st, evs, &bs);
  if (e != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  const int fb = bs.fb;
  const uint32_t* hkeys = reinterpret_cast<const uint32_t*>(ws.keys[fb]);
  k_delta_seg_split<<<div_up(n, 256), 256, 0, st>>>(hkeys, ws.vals[fb], bs.lows, d_offsets, bs.shift0, ws.delta, n);
  uint32_t* fcount = ws.scratch + L.counters + kFrontierCounter;
  uint2* frontier = reinterpret_cast<uint2*>(ws.keys[fb ^ 1]);  // the sort's other key buffer
  const SegBatch seg{hkeys, d_offsets, 30 - bs.shift0};
  k_emit<SegBatch, false, kEmitTile><<<div_up(n, kEmitTile), kEmitTile, 0, st>>>(
      ws.delta, nullptr, ws.vals[fb], ws.boxes, ws.nodes, n, seg, d_indices, frontier, fcount, kEmitMaxSteps);
  k_emit_climb<SegBatch, false><<<std::min<uint32_t>(div_up(n, 256), 152 * 16), 256, 0, st>>>(
      ws.delta, ws.nodes, ws.slots, ws.scratch + L.epoch, n, seg, frontier, fcount);
  if (evs && evs->use) {
    cudaEventRecord(evs->ev[4], st);
    cudaEventRecord(evs->ev[5], st);
  }
  return cudaGetLastError();
}

}  // namespace bvhgb
