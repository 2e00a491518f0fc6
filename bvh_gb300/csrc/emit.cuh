// emit.cuh -- bottom-up Karras hierarchy + refit, shared by single-mesh and batched builds.
//
// Reference: kBuildInternalNodes_nt (src/cuda/lbvh_builder.cu:183-229), kInitLeafNodes_nt
// (:231-241) and kRefitHierarchy_nt (:243-274); same node ids, children and boxes.
//
// Step 1: D[k] = delta(k, k+1) + 1 for adjacent sorted positions, one byte each (delta_nt,
// lbvh_builder.cu:33-43: common-prefix length of the codes, or 32/64 + clz(origIdx_k ^
// origIdx_k+1) when the codes are equal; 0 marks a segment boundary).  30-bit codes: k_emit
// computes them for its tile; 60/63-bit codes: the run fix-up writes them; batched keys:
// k_delta_seg_split.
// Step 2 (k_emit): one thread per sorted position climbs; merges whose two children belong to
// threads of one block happen in shared memory.  Nodes whose sibling is built by another block,
// and nodes still climbing after kEmitMaxSteps levels, are listed as a frontier, from which
// k_emit_climb continues through global rendezvous words.  A node with range [f, l] has its
// parent's split on the side whose adjacent delta is larger (Apetrei 2014): gamma = l when
// D[l] > D[f-1], else gamma = f-1.  The second child to reach gamma's rendezvous word completes
// the parent.  Karras ids: leaf i -> n-1+i, a left child's id is its last index, a right
// child's its first, the root is 0.  Segments (batched meshes) number their nodes from their
// own base and see delta = -1 across their boundaries.
#pragma once
#include "common.cuh"

namespace bvhgb {

// Single mesh: one segment [0, n) with node base 0; original indices are global.
struct SegSingle {
  uint32_t n;
  __device__ __forceinline__ void get(uint32_t /*i*/, uint32_t& off, uint32_t& cnt, uint32_t& nbase) const {
    off = 0;
    cnt = n;
    nbase = 0;
  }
  __device__ __forceinline__ uint32_t mesh_of_key(unsigned long long) const { return 0; }
};

// Batched meshes: key = mesh << 30 | code30; mesh m owns sorted positions
// [offsets[m], offsets[m+1]) and node ids [2*offsets[m] - m, ...).
// hkeys = (mesh << 30 | code30) >> shift0, so the mesh is hkeys >> (30 - shift0).
struct SegBatch {
  const uint32_t* hkeys;
  const uint32_t* offsets;
  int mshift;  // 30 - shift0
  __device__ __forceinline__ void get(uint32_t i, uint32_t& off, uint32_t& cnt, uint32_t& nbase) const {
    const uint32_t m = __ldg(hkeys + i) >> mshift;
    off = __ldg(offsets + m);
    cnt = __ldg(offsets + m + 1) - off;
    nbase = 2 * off - m;
  }
};

// In-tile climbs stop after this many levels and continue in k_emit_climb (k_emit's max_steps):
// the longest chain of a block no longer holds its 512 threads.
constexpr uint32_t kEmitMaxSteps = 8;
constexpr uint32_t kEmitTile = 512;  // sorted positions (threads) per k_emit block

__device__ __forceinline__ void store_node(Node* nodes, uint32_t idx, const Box& b, int32_t l, int32_t r, int32_t aux0) {
  float4* p = reinterpret_cast<float4*>(nodes + idx);
  __stcg(p, b.lo);
  __stcg(p + 1, b.hi);
  __stcg(reinterpret_cast<int4*>(p + 2), make_int4(l, r, aux0, 0));
}
__device__ __forceinline__ Box load_node_box(const Node* nodes, uint32_t idx) {
  const float4* p = reinterpret_cast<const float4*>(nodes + idx);
  Box b;
  b.lo = __ldcg(p);
  b.hi = __ldcg(p + 1);
  return b;
}

__device__ __forceinline__ uint32_t atom_or_acq_rel_cta(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.cta.shared::cta.or.b32 %0, [%1], %2;"
               : "=r"(old)
               : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(v)
               : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long atom_exch_acq_rel(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}

// Batched meshes: keys mesh << 30 | code30 held split as hk = key >> shift0 (sorted) and lows =
// key & (2^shift0 - 1) by original index.  delta = -1 across meshes, the clz of the 30-bit code
// XOR within a mesh, 32 + clz of the in-mesh indices' XOR for equal codes.
static __global__ void __launch_bounds__(256)
    k_delta_seg_split(const uint32_t* __restrict__ hk, const uint32_t* __restrict__ vals,
                      const uint32_t* __restrict__ lows, const uint32_t* __restrict__ offsets, int shift0,
                      uint8_t* __restrict__ D, uint32_t n) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k + 1 >= n) return;
  const uint32_t a = __ldg(hk + k), b = __ldg(hk + k + 1);
  const uint32_t ma = a >> (30 - shift0), mb = b >> (30 - shift0);
  int d;
  if (ma != mb) {
    d = -1;
  } else if (a != b) {
    d = __clz((uint32_t)((unsigned long long)(a ^ b) << shift0));
  } else {
    const uint32_t va = __ldg(vals + k), vb = __ldg(vals + k + 1);
    const uint32_t la = shift0 ? __ldg(lows + va) : 0u, lb = shift0 ? __ldg(lows + vb) : 0u;
    const uint32_t off = __ldg(offsets + ma);
    d = la != lb ? __clz(la ^ lb) : 32 + __clz((va - off) ^ (vb - off));
  }
  D[k] = (uint8_t)(d + 1);
}

template <bool PARENTS>
__device__ __forceinline__ void write_internal(Node* nodes, uint32_t nb, int32_t my, const Box& box, int32_t lc,
                                               int32_t rc) {
  store_node(nodes, nb + (uint32_t)my, box, lc, rc, -1);
  if (PARENTS) {
    __stcg(&nodes[nb + lc].aux0, my);
    __stcg(&nodes[nb + rc].aux0, my);
  }
}

// Climb state of one lane: the node it currently owns covers sorted positions [f, l].
struct Climb {
  uint32_t f, l;
  Box box;
  int32_t lc, rc, my;
  bool internal;
};

// T sorted positions per block, one thread each (a larger block leaves fewer nodes whose sibling
// lies in another block to the frontier pass).
// KEYS30: the tile's delta bytes are computed here from the sorted 30-bit keys (the delta_nt
// rule, as k_delta) and written to D for k_emit_climb; otherwise they are read from D.
template <typename Seg, bool PARENTS, uint32_t T = 256, bool KEYS30 = false>
__global__ void __launch_bounds__(T, 2048 / T) k_emit(uint8_t* __restrict__ D, const uint32_t* __restrict__ keys30,
                                            const uint32_t* __restrict__ vals,
                                            const Box* __restrict__ tri_boxes, Node* __restrict__ nodes,
                                            uint32_t n, Seg seg, uint32_t* __restrict__ out_idx,
                                            uint2* __restrict__ frontier, uint32_t* __restrict__ frontier_count,
                                            uint32_t max_steps) {
  // D of positions bbase-1 .. bbase+T-1 (0 outside [0, n-1) : a segment boundary)
  __shared__ uint8_t s_D[T + 1];
  // KEYS30: keys and values of positions bbase-1 .. bbase+T
  __shared__ uint32_t s_k[KEYS30 ? T + 2 : 1], s_v[KEYS30 ? T + 2 : 1];
  // rendezvous slot k <-> split gamma = bbase + k: one side per child (0 left, 1 right); the
  // child's box with its id in lo.w and its far end (f of a left child, l of a right child) in hi.w
  __shared__ uint32_t s_flag[T];
  __shared__ float4 s_lo[2][T];
  __shared__ float4 s_hi[2][T];
  const uint32_t tid = threadIdx.x;
  const uint32_t i = blockIdx.x * T + tid;
  const uint32_t bbase = blockIdx.x * T;  // sorted position of thread 0
  bool active = i < n;
  uint32_t off = 0, cnt = 1, nb = 0;
  Climb c;
  c.f = c.l = i;
  c.lc = c.rc = -1;
  c.internal = false;
  c.my = 0;
  if (active) {
    seg.get(i, off, cnt, nb);
    const uint32_t prim_g = __ldg(vals + i);
    const uint32_t prim = prim_g - off;  // original index within the mesh
    if (out_idx) out_idx[i] = prim;
    const float4* bp = reinterpret_cast<const float4*>(tri_boxes + prim_g);
    c.box.lo = __ldg(bp);
    c.box.hi = __ldg(bp + 1);
    c.my = (int32_t)(cnt - 1) + (int32_t)(i - off);
    store_node(nodes, nb + (uint32_t)c.my, c.box, (int32_t)(prim | kLeafBit), -1, -1);
    if (cnt == 1) active = false;  // a one-triangle mesh: the leaf is the root
    if (KEYS30) {
      s_k[tid + 1] = __ldg(keys30 + i);
      s_v[tid + 1] = prim_g;
    }
  }
  if (KEYS30) {
    if (tid == 0 && bbase > 0) {
      s_k[0] = __ldg(keys30 + bbase - 1);
      s_v[0] = __ldg(vals + bbase - 1);
    }
    if (tid == T - 1 && bbase + T < n) {
      s_k[T + 1] = __ldg(keys30 + bbase + T);
      s_v[T + 1] = __ldg(vals + bbase + T);
    }
    __syncthreads();
    // s_D[k] = D[bbase - 1 + k]; position j and j + 1 sit at s_k[k], s_k[k + 1]
    for (uint32_t k = tid; k <= T; k += T) {
      const int64_t j = (int64_t)bbase - 1 + k;
      uint8_t d = 0;
      if (j >= 0 && j + 1 < (int64_t)n) {
        const uint32_t a = s_k[k], b = s_k[k + 1];
        d = (uint8_t)((a == b ? 32 + __clz(s_v[k] ^ s_v[k + 1]) : __clz(a ^ b)) + 1);
        if (k >= 1) D[j] = d;  // the tile's own positions bbase .. bbase + T - 1
      }
      s_D[k] = d;
    }
  } else {
    const int64_t j = (int64_t)bbase - 1 + tid;
    s_D[tid] = (j >= 0 && j + 1 < (int64_t)n) ? __ldg(D + j) : (uint8_t)0;
    if (tid == 0) {
      const uint64_t jl = (uint64_t)bbase + T - 1;
      s_D[T] = jl + 1 < n ? __ldg(D + jl) : (uint8_t)0;
    }
  }
  s_flag[tid] = 0;
  __syncthreads();
  // ---- climb inside the block: the second child to reach a split completes the parent ----
  // A node [f, l] with both ends in this block reads D[f-1] and D[l] from s_D; its parent's
  // split is gamma = l (it is the left child) when D[l] > D[f-1], else gamma = f-1.
  bool to_frontier = false;
  for (uint32_t step = 0; active; ++step) {
    const int dl = (int)s_D[c.f - bbase] - 1;
    const int dr = (int)s_D[c.l - bbase + 1] - 1;
    if (dl < 0 && dr < 0) {  // segment root
      write_internal<PARENTS>(nodes, nb, 0, c.box, c.lc, c.rc);
      break;
    }
    const bool is_left = dr > dl;
    const uint32_t gamma = is_left ? c.l : c.f - 1;
    const bool pending = c.internal;  // complete; its id is known now: a left child is named by its last index
    if (pending) c.my = (int32_t)((is_left ? c.l : c.f) - off);
    // sibling starts outside the block, or the climb has gone max_steps levels: the node
    // continues in k_emit_climb, so that one long chain does not hold the block
    if (step >= max_steps || (is_left ? gamma + 1 >= bbase + T : gamma < bbase)) {
      if (pending) write_internal<PARENTS>(nodes, nb, c.my, c.box, c.lc, c.rc);
      to_frontier = true;
      break;
    }
    // with parent links the node is written before the rendezvous, so that the parent's later
    // write of its aux0 lands last
    if (PARENTS && pending) write_internal<PARENTS>(nodes, nb, c.my, c.box, c.lc, c.rc);
    const uint32_t k = gamma - bbase;
    const int side = is_left ? 0 : 1;
    s_lo[side][k] = make_float4(c.box.lo.x, c.box.lo.y, c.box.lo.z, __int_as_float(c.my));
    s_hi[side][k] = make_float4(c.box.hi.x, c.box.hi.y, c.box.hi.z, __uint_as_float(is_left ? c.f : c.l));
    // release: the slot is visible before the flag bit; acquire: the sibling's slot is read after
    const uint32_t prev = atom_or_acq_rel_cta(&s_flag[k], 1u << side);
    if (!PARENTS && pending) write_internal<PARENTS>(nodes, nb, c.my, c.box, c.lc, c.rc);
    if (prev == 0u) break;  // first to arrive
    const float4 a = s_lo[side ^ 1][k], b = s_hi[side ^ 1][k];
    Box sb;
    sb.lo = make_float4(a.x, a.y, a.z, 0.f);
    sb.hi = make_float4(b.x, b.y, b.z, 0.f);
    if (is_left) {
      c.lc = c.my;
      c.rc = __float_as_int(a.w);
      c.l = __float_as_uint(b.w);
      c.box = box_union(c.box, sb);
    } else {
      c.lc = __float_as_int(a.w);
      c.rc = c.my;
      c.f = __float_as_uint(b.w);
      c.box = box_union(sb, c.box);
    }
    c.internal = true;
  }
  __syncthreads();
  // ---- finished nodes whose parent needs a sibling built elsewhere continue in k_emit_climb:
  // those stopped at the block edge and those whose in-block sibling never completed ----
  uint2 fr0 = make_uint2(c.f, c.l), fr1 = make_uint2(0u, 0u);
  uint32_t nf = to_frontier ? 1u : 0u;
  if (tid < T - 1) {
    const uint32_t fl = s_flag[tid];
    const uint32_t g = bbase + tid;
    uint2 e = fl == 1u ? make_uint2(__float_as_uint(s_hi[0][tid].w), g)
                       : make_uint2(g + 1, __float_as_uint(s_hi[1][tid].w));
    if (fl == 1u || fl == 2u) {
      if (nf) fr1 = e;
      else fr0 = e;
      ++nf;
    }
  }
  __shared__ uint32_t s_count, s_base;
  if (tid == 0) s_count = 0;
  __syncthreads();
  uint32_t slot_in_block = 0;
  if (nf) slot_in_block = atomicAdd(&s_count, nf);
  __syncthreads();
  if (tid == 0 && s_count) s_base = atomicAdd(frontier_count, s_count);
  __syncthreads();
  if (nf) frontier[s_base + slot_in_block] = fr0;
  if (nf > 1) frontier[s_base + slot_in_block + 1] = fr1;
}

// Climb from every frontier node (a finished node whose parent needs a sibling built by
// another block) through the rendezvous words; the second child to arrive completes the parent.
template <typename Seg, bool PARENTS>
__global__ void __launch_bounds__(256) k_emit_climb(const uint8_t* __restrict__ D, Node* __restrict__ nodes,
                                                    unsigned long long* __restrict__ slots,
                                                    const uint32_t* epoch_word, uint32_t n, Seg seg,
                                                    const uint2* __restrict__ frontier,
                                                    const uint32_t* __restrict__ frontier_count) {
  const uint32_t count = __ldcg(frontier_count);
  const unsigned long long tag = (unsigned long long)__ldcg(epoch_word) << 32;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
    const uint2 fl = __ldcg(frontier + e);
    Climb c;
    c.f = fl.x;
    c.l = fl.y;
    uint32_t off, cnt, nb;
    seg.get(c.f, off, cnt, nb);
    int dl = c.f == 0 ? -1 : (int)__ldg(D + c.f - 1) - 1;
    int dr = c.l + 1 >= n ? -1 : (int)__ldg(D + c.l) - 1;
    bool is_left = dr > dl;
    uint32_t gamma = is_left ? c.l : c.f - 1;
    c.my = c.f == c.l ? (int32_t)(cnt - 1 + (c.f - off)) : (int32_t)((is_left ? c.l : c.f) - off);
    c.box = load_node_box(nodes, nb + (uint32_t)c.my);
    while (true) {
      const uint32_t far = is_left ? c.f : c.l;
      const unsigned long long old = atom_exch_acq_rel(slots + gamma, tag | far);
      if ((old & 0xffffffff00000000ull) != tag) break;  // first child to arrive
      const uint32_t other = (uint32_t)old;
      const int32_t g = (int32_t)(gamma - off);
      int32_t sib;
      if (is_left) {
        sib = (other == gamma + 1) ? (int32_t)cnt + g : g + 1;
        c.lc = c.my;
        c.rc = sib;
        c.l = other;
        c.box = box_union(c.box, load_node_box(nodes, nb + (uint32_t)sib));
      } else {
        sib = (other == gamma) ? (int32_t)cnt - 1 + g : g;
        c.lc = sib;
        c.rc = c.my;
        c.f = other;
        c.box = box_union(load_node_box(nodes, nb + (uint32_t)sib), c.box);
      }
      dl = c.f == 0 ? -1 : (int)__ldg(D + c.f - 1) - 1;
      dr = c.l + 1 >= n ? -1 : (int)__ldg(D + c.l) - 1;
      if (dl < 0 && dr < 0) {
        write_internal<PARENTS>(nodes, nb, 0, c.box, c.lc, c.rc);
        break;
      }
      is_left = dr > dl;
      gamma = is_left ? c.l : c.f - 1;
      c.my = (int32_t)((is_left ? c.l : c.f) - off);
      write_internal<PARENTS>(nodes, nb, c.my, c.box, c.lc, c.rc);
    }
  }
}

}  // namespace bvhgb
