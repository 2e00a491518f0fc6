// treelet.cu -- LBVH+ treelet restructuring passes.
//
// Reference: kRefitAndOptimize(doOptimize=true) with optimizeTreeletSerial,
// src/cuda/lbvh_plus_builder.cu:71-247 and :341-366.  One pass climbs from every leaf; the
// second child to arrive at a node refits its box and restructures the treelet rooted there
// (up to 7 treelet leaves, grown by expanding the largest-area internal leaf; subset DP with
// cost = min split + area; internal node ids reused in DFS order).
//
// A treelet at X only reads and writes nodes of X's subtree, all of which are final when the
// second child arrives, so the result is independent of scheduling and equal to any
// children-before-parent order (the oracle uses post-order).
//
// The DP is warp-cooperative: every warp keeps looping while any lane still climbs; lanes that
// reached a node needing work are served one at a time by all 32 lanes.
#include "emit.cuh"
#include "lbvh.cuh"

namespace bvhgb {

constexpr int kTlMax = 7;
constexpr float kTlInf = 1e30f;

__device__ __forceinline__ Box ldcg_box(const Node* nodes, int32_t idx) {
  const float4* p = reinterpret_cast<const float4*>(nodes + idx);
  Box b;
  b.lo = __ldcg(p);
  b.hi = __ldcg(p + 1);
  return b;
}
__device__ __forceinline__ int2 ldcg_children(const Node* nodes, int32_t idx) {
  return __ldcg(reinterpret_cast<const int2*>(&nodes[idx].left));
}

// Per-warp shared state for one treelet.
struct TreeletSmem {
  float cost[1 << kTlMax];
  float area[1 << kTlMax];
  uint8_t part[1 << kTlMax];
  Box leafbox[kTlMax];
  int32_t act[kTlMax];
  int32_t n;
};

// pdep of the low bits of m into the set bits of mask (m-th nonempty subset of mask in
// increasing numeric order, m >= 1).
__device__ __forceinline__ uint32_t deposit_bits(uint32_t m, uint32_t mask) {
  uint32_t r = 0;
  for (uint32_t bit = 1; mask; bit <<= 1) {
    uint32_t low = mask & (0u - mask);
    if (m & bit) r |= low;
    mask ^= low;
  }
  return r;
}

// Warp-cooperative optimizeTreeletSerial at `root` (lbvh_plus_builder.cu:71-247).
__device__ void treelet_warp(Node* nodes, int32_t root, TreeletSmem& S) {
  const int lane = threadIdx.x & 31;
  // 1. grow the treelet (:73-114): lane 0 walks, others wait
  if (lane == 0) {
    int cnt = 1;
    S.act[0] = root;
    S.leafbox[0] = ldcg_box(nodes, root);
    for (int step = 0; step < kTlMax - 1; ++step) {
      int best = -1;
      float max_area = -1.0f;
      for (int i = 0; i < cnt; ++i) {
        int2 ch = ldcg_children(nodes, S.act[i]);
        if (!((uint32_t)ch.x & kLeafBit)) {
          float a = box_area(S.leafbox[i]);
          if (a > max_area) { max_area = a; best = i; }
        }
      }
      if (best == -1) break;
      int2 ch = ldcg_children(nodes, S.act[best]);
      S.act[best] = ch.x;
      S.leafbox[best] = ldcg_box(nodes, ch.x);
      S.act[cnt] = ch.y;
      S.leafbox[cnt] = ldcg_box(nodes, ch.y);
      cnt++;
    }
    S.n = cnt;
  }
  __syncwarp();
  const int n = S.n;
  if (n < 2) return;
  const uint32_t full = (1u << n) - 1u;
  // 2. subset areas and leaf costs (:119-129); the union is exact in any order
  for (uint32_t s = 1 + lane; s <= full; s += 32) {
    Box b = box_empty();
    for (int i = 0; i < n; ++i)
      if ((s >> i) & 1u) b = box_union(b, S.leafbox[i]);
    S.area[s] = box_area(b);
    S.cost[s] = __popc(s) == 1 ? 0.0f : kTlInf;
  }
  __syncwarp();
  // 3. DP by subset size (:131-165).  Work items are (subset, partition) pairs; the best
  //    partition is the minimum cost, first in the reference's enumeration order on ties.
  for (int k = 2; k <= n; ++k) {
    const uint32_t nparts = (1u << (k - 1)) - 1u;
    // lanes per subset: spread partitions over several lanes for the large subsets
    const uint32_t lps = nparts >= 32 ? 32u : (nparts >= 16 ? 16u : (nparts >= 8 ? 8u : (nparts >= 4 ? 4u : 1u)));
    const uint32_t groups = 32u / lps;
    // enumerate subsets of size k in increasing numeric order, `groups` at a time
    uint32_t s_iter = (1u << k) - 1u;  // smallest subset with k bits
    while (s_iter <= full) {
      // each group takes the g-th next subset
      const uint32_t g = (uint32_t)lane / lps, sub = (uint32_t)lane % lps;
      uint32_t s = s_iter;
      for (uint32_t t = 0; t < g && s <= full; ++t) {  // Gosper's hack: next subset with k bits
        uint32_t c = s & (0u - s), r = s + c;
        s = (((r ^ s) >> 2) / c) | r;
      }
      float best = kTlInf;
      uint32_t best_ord = 0xffffffffu, best_p = 0;
      if (s <= full) {
        const uint32_t delta = (s - 1u) & s;
        for (uint32_t ord = sub; ord < nparts; ord += lps) {
          uint32_t p = deposit_bits(ord + 1u, delta);
          float c = __fadd_rn(S.cost[p], S.cost[s ^ p]);
          if (c < best) { best = c; best_ord = ord; best_p = p; }
        }
      }
      // reduce within the lane group: min cost, then smallest enumeration order
      for (uint32_t o = 1; o < lps; o <<= 1) {
        float ob = __shfl_xor_sync(0xffffffffu, best, o);
        uint32_t oo = __shfl_xor_sync(0xffffffffu, best_ord, o);
        uint32_t op = __shfl_xor_sync(0xffffffffu, best_p, o);
        if (ob < best || (ob == best && oo < best_ord)) { best = ob; best_ord = oo; best_p = op; }
      }
      if (sub == 0 && s <= full) {
        // the reference starts from INF with strict <, so an all-INF subset keeps INF / -1
        S.cost[s] = __fadd_rn(best, S.area[s]);
        S.part[s] = (uint8_t)(best_ord == 0xffffffffu ? 0xffu : best_p);
      }
      // advance s_iter by `groups` subsets
      for (uint32_t t = 0; t < groups && s_iter <= full; ++t) {
        uint32_t c = s_iter & (0u - s_iter), r = s_iter + c;
        s_iter = (((r ^ s_iter) >> 2) / c) | r;
      }
      __syncwarp();
    }
    __syncwarp();
  }
  // 4. reuse internal ids (DFS, right child popped first, :167-191) and rebuild breadth-first
  //    (:194-246); at most 6 internal nodes, done by lane 0
  if (lane == 0) {
    int avail[kTlMax];
    int n_avail = 0;
    int stack[kTlMax + 8];
    int top = 0;
    stack[top++] = root;
    while (top > 0) {
      int cur = stack[--top];
      bool in_leaves = false;
      for (int i = 0; i < n; ++i)
        if (S.act[i] == cur) { in_leaves = true; break; }
      if (!in_leaves && n_avail < kTlMax && top + 2 <= kTlMax + 8) {
        avail[n_avail++] = cur;
        int2 ch = ldcg_children(nodes, cur);
        stack[top++] = ch.x;
        stack[top++] = ch.y;
      }
    }
    // A subset whose partitions all cost >= INF (NaN areas) has no valid split; the
    // reference would index out of bounds there, this leaves the treelet unchanged.
    {
      int vm[kTlMax], vh = 0, vt = 0;
      bool ok = true;
      vm[vt++] = (int)full;
      while (vh < vt && ok) {
        int mask = vm[vh++];
        int lm = S.part[mask], rm = mask ^ lm;
        if (lm == 0 || rm == 0 || (lm & ~mask)) { ok = false; break; }
        if (__popc(lm) > 1) { if (vt >= kTlMax) { ok = false; break; } vm[vt++] = lm; }
        if (__popc(rm) > 1) { if (vt >= kTlMax) { ok = false; break; } vm[vt++] = rm; }
      }
      if (!ok || n_avail != n - 1) S.n = 0;
    }
    int qm[kTlMax], qn[kTlMax];
    int qh = 0, qt = 0, used = 1;
    if (S.n) {
      qm[qt] = (int)full;
      qn[qt++] = avail[0];
    }
    while (qh < qt) {
      int mask = qm[qh], cur = qn[qh];
      qh++;
      int lm = S.part[mask], rm = mask ^ lm;
      int li, ri;
      if (__popc(lm) == 1) li = S.act[__ffs(lm) - 1];
      else { li = avail[used++]; qm[qt] = lm; qn[qt++] = li; }
      if (__popc(rm) == 1) ri = S.act[__ffs(rm) - 1];
      else { ri = avail[used++]; qm[qt] = rm; qn[qt++] = ri; }
      Box b = box_empty();
      for (int i = 0; i < n; ++i)
        if ((mask >> i) & 1) b = box_union(b, S.leafbox[i]);
      float4* p = reinterpret_cast<float4*>(nodes + cur);
      __stcg(p, b.lo);
      __stcg(p + 1, b.hi);
      __stcg(reinterpret_cast<int2*>(&nodes[cur].left), make_int2(li, ri));
      __stcg(&nodes[li].aux0, cur);
      __stcg(&nodes[ri].aux0, cur);
    }
  }
  __syncwarp();
}

// One refit+optimise pass (kRefitAndOptimize(true)).  Warp-synchronous climb: lanes never
// leave the loop early so that all 32 can serve each lane's treelet.
__global__ void __launch_bounds__(128) k_treelet_round(Node* __restrict__ nodes, unsigned long long* __restrict__ slots,
                                                       const uint32_t* epoch_word, uint32_t round, uint32_t n) {
  __shared__ TreeletSmem S[4];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool active = i < n;
  int32_t idx = (int32_t)(n - 1 + i);
  const unsigned long long tag = (unsigned long long)(__ldcg(epoch_word) + 1u + round) << 32;
  while (__any_sync(0xffffffffu, active)) {
    bool work = false;
    if (active) {
      if (idx == 0) {
        active = false;
      } else {
        int32_t parent = __ldcg(&nodes[idx].aux0);
        __threadfence();
        unsigned long long old = atomicExch(slots + parent, tag | 1u);
        if ((old & 0xffffffff00000000ull) != tag) {
          active = false;  // first child to arrive
        } else {
          __threadfence();
          int2 ch = ldcg_children(nodes, parent);
          Box b = box_union(ldcg_box(nodes, ch.x), ldcg_box(nodes, ch.y));
          float4* p = reinterpret_cast<float4*>(nodes + parent);
          __stcg(p, b.lo);
          __stcg(p + 1, b.hi);
          idx = parent;
          work = true;
        }
      }
    }
    uint32_t ballot = __ballot_sync(0xffffffffu, work);
    while (ballot) {
      int src = __ffs(ballot) - 1;
      ballot &= ballot - 1;
      int32_t root = __shfl_sync(0xffffffffu, idx, src);
      treelet_warp(nodes, root, S[w]);
    }
    __threadfence();
  }
}

cudaError_t treelet_rounds_run(Workspace& ws, uint32_t n, int rounds, cudaStream_t st) {
  ScratchLayout L = scratch_layout(ws.cap_n);
  for (int r = 0; r < rounds && r + 1 < (int)kEpochStride; ++r)
    k_treelet_round<<<div_up(n, 128), 128, 0, st>>>(ws.nodes, ws.slots, ws.scratch + L.epoch, (uint32_t)r, n);
  return cudaGetLastError();
}

}  // namespace bvhgb
