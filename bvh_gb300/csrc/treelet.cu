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
// Every warp keeps looping while any lane still climbs.  Lanes that reached a node grow and
// rebuild their own treelets in parallel; the subset DP of each is done by all 32 lanes.
#include <algorithm>

#include "emit.cuh"
#include "lbvh.cuh"

namespace bvhgb {

constexpr int kTlMax = 7;
constexpr float kTlInf = 1e30f;
}  // namespace bvhgb
#include "treelet_dp_unrolled.cuh"
namespace bvhgb {

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

// Subsets of {0..6} with 2..7 members, by size, increasing within a size.  For a treelet of
// n < 7 leaves the subsets of its full mask are the entries <= (1 << n) - 1, in the same order.
__constant__ uint8_t c_subsets[120] = {
    3, 5, 6, 9, 10, 12, 17, 18, 20, 24, 33, 34, 36, 40, 48, 65, 66, 68, 72, 80, 96,
    7, 11, 13, 14, 19, 21, 22, 25, 26, 28, 35, 37, 38, 41, 42, 44, 49, 50, 52, 56, 67, 69, 70, 73, 74, 76, 81,
    82, 84, 88, 97, 98, 100, 104, 112,
    15, 23, 27, 29, 30, 39, 43, 45, 46, 51, 53, 54, 57, 58, 60, 71, 75, 77, 78, 83, 85, 86, 89, 90, 92, 99,
    101, 102, 105, 106, 108, 113, 114, 116, 120,
    31, 47, 55, 59, 61, 62, 79, 87, 91, 93, 94, 103, 107, 109, 110, 115, 117, 118, 121, 122, 124,
    63, 95, 111, 119, 123, 125, 126,
    127};
__constant__ uint8_t c_sub_off[9] = {0, 0, 0, 21, 56, 91, 112, 119, 120};  // first entry of size k

// One lane's treelet: its leaves (node ids, boxes, cached children), the expansions that grew
// it (which the id reuse walks instead of reloading nodes) and the DP's best partitions.
struct LaneTreelet {
  float box[6][kTlMax];  // lo.x lo.y lo.z hi.x hi.y hi.z of each leaf
  int32_t act[kTlMax];
  int32_t chl[kTlMax], chr[kTlMax];  // children of each leaf node (left has kLeafBit for a BVH leaf)
  int32_t exp_node[kTlMax - 1], exp_l[kTlMax - 1], exp_r[kTlMax - 1];
  uint8_t part[1 << kTlMax];
  int32_t n;
};

__device__ __forceinline__ Box leaf_box(const LaneTreelet& T, int i) {
  Box b;
  b.lo = make_float4(T.box[0][i], T.box[1][i], T.box[2][i], 0.f);
  b.hi = make_float4(T.box[3][i], T.box[4][i], T.box[5][i], 0.f);
  return b;
}
__device__ __forceinline__ void set_leaf(LaneTreelet& T, int i, int32_t id, const Box& b, int2 ch) {
  T.act[i] = id;
  T.box[0][i] = b.lo.x; T.box[1][i] = b.lo.y; T.box[2][i] = b.lo.z;
  T.box[3][i] = b.hi.x; T.box[4][i] = b.hi.y; T.box[5][i] = b.hi.z;
  T.chl[i] = ch.x;
  T.chr[i] = ch.y;
}

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

// 1. Grow the treelet at `root` (lbvh_plus_builder.cu:73-114): up to 6 times, expand the leaf
//    with the largest area among those that are internal nodes (first such on ties).  Run by
//    one lane; the lanes of a warp grow their own treelets side by side.
__device__ void treelet_grow(const Node* nodes, int32_t root, LaneTreelet& T) {
  set_leaf(T, 0, root, ldcg_box(nodes, root), ldcg_children(nodes, root));
  int cnt = 1;
  for (int step = 0; step < kTlMax - 1; ++step) {
    int best = -1;
    float max_area = -1.0f;
#pragma unroll
    for (int i = 0; i < kTlMax; ++i) {
      if (i < cnt && !((uint32_t)T.chl[i] & kLeafBit)) {
        const float a = box_area(leaf_box(T, i));
        if (a > max_area) { max_area = a; best = i; }
      }
    }
    if (best < 0) break;
    const int32_t l = T.chl[best], r = T.chr[best];
    T.exp_node[step] = T.act[best];
    T.exp_l[step] = l;
    T.exp_r[step] = r;
    const Box bl = ldcg_box(nodes, l), br = ldcg_box(nodes, r);
    const int2 cl = ldcg_children(nodes, l), cr = ldcg_children(nodes, r);
    set_leaf(T, best, l, bl, cl);
    set_leaf(T, cnt, r, br, cr);
    ++cnt;
  }
  T.n = cnt;
}

// 2+3. Subset areas and the DP over subsets by size (:119-165), by the whole warp for one
//    lane's treelet.  cost[s] = min over splits (cost[p] + cost[s^p]) + area[s], leaves cost 0;
//    the best split is the first minimum in the enumeration p = increasing nonempty subsets of
//    s without its lowest member.  Sizes 2..5 take one lane per subset, size 6 four lanes and
//    size 7 the whole warp, each lane scanning a contiguous run of that enumeration.
__device__ void treelet_dp(LaneTreelet& T, float* cost, float* area) {
  const int lane = threadIdx.x & 31;
  const int n = T.n;
  const uint32_t full = (1u << n) - 1u;
  for (uint32_t s = 1 + lane; s <= full; s += 32) {
    Box b = box_empty();
#pragma unroll
    for (int i = 0; i < kTlMax; ++i)
      if ((s >> i) & 1u) b = box_union(b, leaf_box(T, i));
    area[s] = box_area(b);
    cost[s] = __popc(s) == 1 ? 0.0f : kTlInf;
  }
  __syncwarp();
  for (int k = 2; k <= n; ++k) {
    const uint32_t L = k <= 5 ? 1u : (k == 6 ? 4u : 32u);
    const uint32_t base = c_sub_off[k], count = c_sub_off[k + 1] - base;
    const uint32_t nparts = (1u << (k - 1)) - 1u;
    const uint32_t chunk = (nparts + L - 1) / L;
    for (uint32_t r0 = 0; r0 < count * L; r0 += 32) {
      const uint32_t slot = r0 + (uint32_t)lane, e = slot / L, j = slot % L;
      const uint32_t s = e < count ? c_subsets[base + e] : 0u;
      const bool valid = e < count && s <= full;
      float best = kTlInf;
      uint32_t best_ord = 0xffffffffu, best_p = 0;
      if (valid) {
        const uint32_t delta = s & (s - 1u);
        const uint32_t o0 = j * chunk, o1 = min(o0 + chunk, nparts);
        uint32_t p = o0 < o1 ? deposit_bits(o0 + 1u, delta) : 0u;
        for (uint32_t ord = o0; ord < o1; ++ord) {
          const float c = __fadd_rn(cost[p], cost[s ^ p]);
          if (c < best) { best = c; best_ord = ord; best_p = p; }
          p = (p - delta) & delta;  // next subset of delta
        }
      }
      for (uint32_t o = 1; o < L; o <<= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t oo = __shfl_xor_sync(0xffffffffu, best_ord, o);
        const uint32_t op = __shfl_xor_sync(0xffffffffu, best_p, o);
        if (ob < best || (ob == best && oo < best_ord)) { best = ob; best_ord = oo; best_p = op; }
      }
      if (valid && j == 0) {
        // the reference starts from INF with strict <, so an all-INF subset keeps INF / -1
        cost[s] = __fadd_rn(best, area[s]);
        T.part[s] = (uint8_t)(best_ord == 0xffffffffu ? 0xffu : best_p);
      }
    }
    __syncwarp();
  }
}

// 4. Reuse the treelet's internal ids (DFS from the root, right child popped first,
//    :167-191) and rebuild it breadth-first from the partitions (:194-246).  One lane.
__device__ void treelet_rebuild(Node* nodes, int32_t root, LaneTreelet& T) {
  const int n = T.n;
  if (n < 2) return;
  const uint32_t full = (1u << n) - 1u;
  int avail[kTlMax];
  int n_avail = 0;
  int stack[kTlMax + 8];
  int top = 0;
  stack[top++] = root;
  while (top > 0) {
    const int cur = stack[--top];
    bool in_leaves = false;
    for (int i = 0; i < n; ++i)
      if (T.act[i] == cur) { in_leaves = true; break; }
    if (!in_leaves && n_avail < kTlMax && top + 2 <= kTlMax + 8) {
      avail[n_avail++] = cur;
      int2 ch = make_int2(0, 0);
      bool known = false;
      for (int e = 0; e < n - 1; ++e)
        if (T.exp_node[e] == cur) { ch = make_int2(T.exp_l[e], T.exp_r[e]); known = true; break; }
      if (!known) ch = ldcg_children(nodes, cur);
      stack[top++] = ch.x;
      stack[top++] = ch.y;
    }
  }
  // A subset whose partitions all cost >= INF (NaN areas) has no valid split; the reference
  // would index out of bounds there, this leaves the treelet unchanged.
  {
    int vm[kTlMax], vh = 0, vt = 0;
    bool ok = true;
    vm[vt++] = (int)full;
    while (vh < vt && ok) {
      const int mask = vm[vh++];
      const int lm = T.part[mask], rm = mask ^ lm;
      if (lm == 0 || rm == 0 || (lm & ~mask)) { ok = false; break; }
      if (__popc(lm) > 1) { if (vt >= kTlMax) { ok = false; break; } vm[vt++] = lm; }
      if (__popc(rm) > 1) { if (vt >= kTlMax) { ok = false; break; } vm[vt++] = rm; }
    }
    if (!ok || n_avail != n - 1) return;
  }
  int qm[kTlMax], qn[kTlMax];
  int qh = 0, qt = 0, used = 1;
  qm[qt] = (int)full;
  qn[qt++] = avail[0];
  while (qh < qt) {
    const int mask = qm[qh], cur = qn[qh];
    qh++;
    const int lm = T.part[mask], rm = mask ^ lm;
    int li, ri;
    if (__popc(lm) == 1) li = T.act[__ffs(lm) - 1];
    else { li = avail[used++]; qm[qt] = lm; qn[qt++] = li; }
    if (__popc(rm) == 1) ri = T.act[__ffs(rm) - 1];
    else { ri = avail[used++]; qm[qt] = rm; qn[qt++] = ri; }
    Box b = box_empty();
    for (int i = 0; i < n; ++i)
      if ((mask >> i) & 1) b = box_union(b, leaf_box(T, i));
    float4* p = reinterpret_cast<float4*>(nodes + cur);
    __stcg(p, b.lo);
    __stcg(p + 1, b.hi);
    __stcg(reinterpret_cast<int2*>(&nodes[cur].left), make_int2(li, ri));
    __stcg(&nodes[li].aux0, cur);
    __stcg(&nodes[ri].aux0, cur);
  }
}

// ---------------------------------------------------------------------------------------
// Level-synchronous pass.  Any children-before-parent order gives the same tree, and nodes of
// equal height have disjoint subtrees (neither is an ancestor of the other), so each height
// is one parallel step: every lane owns one treelet and does its refit, growth, DP and rebuild
// alone, so the 32 lanes of a warp run the same 7-leaf work in step.  Heights come from a
// climb that carries them in the rendezvous words; node ids are then grouped by height.
// Trees higher than kTlMaxHeight (not reachable by a Karras tree: its depth is at most the
// key bits plus 32) fall back to the climb-ordered kernel above.
// ---------------------------------------------------------------------------------------
constexpr int kTlMaxHeight = 254;
constexpr int kLvThreads = 32;  // one warp per block; its DP tables are 20 KB of shared memory

// A lane's treelet in registers (all indexing below is unrolled to constant indices).
struct RegTreelet {
  Box b[kTlMax];
  int32_t id[kTlMax], cl[kTlMax], cr[kTlMax];
  float area[kTlMax];
  int32_t en[kTlMax - 1], el[kTlMax - 1], er[kTlMax - 1];  // expansions: node and its children
  int n;
};

__device__ __forceinline__ void reg_set(RegTreelet& T, int i, int32_t id, const Box& b, int2 ch) {
#pragma unroll
  for (int k = 0; k < kTlMax; ++k)
    if (k == i) {
      T.id[k] = id;
      T.b[k] = b;
      T.cl[k] = ch.x;
      T.cr[k] = ch.y;
      T.area[k] = box_area(b);
    }
}
__device__ __forceinline__ int32_t reg_id(const RegTreelet& T, int i) {
  int32_t v = 0;
#pragma unroll
  for (int k = 0; k < kTlMax; ++k)
    if (k == i) v = T.id[k];
  return v;
}
__device__ __forceinline__ Box reg_union(const RegTreelet& T, uint32_t mask) {
  Box b = box_empty();
#pragma unroll
  for (int k = 0; k < kTlMax; ++k)
    if ((mask >> k) & 1u) b = box_union(b, T.b[k]);
  return b;
}

// Growth state without the leaf boxes (only their areas are compared).
struct GrowTreelet {
  int32_t id[kTlMax], cl[kTlMax], cr[kTlMax];
  float area[kTlMax];
  int32_t en[kTlMax - 1], el[kTlMax - 1], er[kTlMax - 1];
  int n;
};
__device__ __forceinline__ void reg_set(GrowTreelet& T, int i, int32_t id, const Box& b, int2 ch) {
#pragma unroll
  for (int k = 0; k < kTlMax; ++k)
    if (k == i) {
      T.id[k] = id;
      T.cl[k] = ch.x;
      T.cr[k] = ch.y;
      T.area[k] = box_area(b);
    }
}

// Growth (lbvh_plus_builder.cu:73-114) with each leaf's children and area cached on entry.
template <typename TL>
__device__ __forceinline__ void reg_grow(const Node* nodes, int32_t root, const Box& rootbox, int2 rootch, TL& T) {
  reg_set(T, 0, root, rootbox, rootch);
  int cnt = 1;
#pragma unroll
  for (int step = 0; step < kTlMax - 1; ++step) {
    int best = -1;
    float max_area = -1.0f;
    int32_t bl = 0, br = 0, bn = 0;
#pragma unroll
    for (int i = 0; i < kTlMax; ++i) {
      if (i < cnt && !((uint32_t)T.cl[i] & kLeafBit) && T.area[i] > max_area) {
        max_area = T.area[i];
        best = i;
        bl = T.cl[i];
        br = T.cr[i];
        bn = T.id[i];
      }
    }
    if (best < 0) break;
    T.en[step] = bn;
    T.el[step] = bl;
    T.er[step] = br;
    const Box lb = ldcg_box(nodes, bl), rb = ldcg_box(nodes, br);
    const int2 lc = ldcg_children(nodes, bl), rc = ldcg_children(nodes, br);
    reg_set(T, best, bl, lb, lc);
    reg_set(T, cnt, br, rb, rc);
    ++cnt;
  }
  T.n = cnt;
}

// reg_grow after its first step, the root's expansion, whose loads the caller has made: leaves
// (left, right) with their boxes and children, then the same steps from there.
__device__ __forceinline__ void reg_grow_expanded(const Node* nodes, int32_t root, int2 rootch, const Box& lb,
                                                  const Box& rb, int2 lc, int2 rc, GrowTreelet& T) {
  reg_set(T, 0, rootch.x, lb, lc);
  reg_set(T, 1, rootch.y, rb, rc);
  T.en[0] = root;
  T.el[0] = rootch.x;
  T.er[0] = rootch.y;
  int cnt = 2;
#pragma unroll
  for (int step = 1; step < kTlMax - 1; ++step) {
    int best = -1;
    float max_area = -1.0f;
    int32_t bl = 0, br = 0, bn = 0;
#pragma unroll
    for (int i = 0; i < kTlMax; ++i) {
      if (i < cnt && !((uint32_t)T.cl[i] & kLeafBit) && T.area[i] > max_area) {
        max_area = T.area[i];
        best = i;
        bl = T.cl[i];
        br = T.cr[i];
        bn = T.id[i];
      }
    }
    if (best < 0) break;
    T.en[step] = bn;
    T.el[step] = bl;
    T.er[step] = br;
    const Box lb2 = ldcg_box(nodes, bl), rb2 = ldcg_box(nodes, br);
    const int2 lc2 = ldcg_children(nodes, bl), rc2 = ldcg_children(nodes, br);
    reg_set(T, best, bl, lb2, lc2);
    reg_set(T, cnt, br, rb2, rc2);
    ++cnt;
  }
  T.n = cnt;
}

// Areas of the subsets s < 2^nv with two or more leaves into this lane's column A (stride 32):
// the box of s is (its leaves among 3..6) U (its leaves among 0..2).  NVMAX: nv's bound.
template <int NVMAX = kTlMax>
__device__ __forceinline__ void reg_areas(const RegTreelet& T, int nv, float* A) {
  const uint32_t full = (1u << nv) - 1u;
  Box lo8[8];
  lo8[0] = box_empty();
  lo8[1] = box_union(lo8[0], T.b[0]);
  lo8[2] = box_union(lo8[0], T.b[1]);
  lo8[3] = box_union(lo8[1], T.b[1]);
  lo8[4] = box_union(lo8[0], T.b[2]);
  lo8[5] = box_union(lo8[1], T.b[2]);
  lo8[6] = box_union(lo8[2], T.b[2]);
  lo8[7] = box_union(lo8[3], T.b[2]);
  for (uint32_t hi = 0; hi * 8u <= full; ++hi) {
    Box bh = box_empty();
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (3 + j < NVMAX && ((hi >> j) & 1u)) bh = box_union(bh, T.b[3 + j]);
#pragma unroll
    for (int lo = 0; lo < 8; ++lo) {
      const uint32_t s = hi * 8u + (uint32_t)lo;
      if (s <= full && __popc(s) > 1) A[s * 32u] = box_area(box_union(bh, lo8[lo]));
    }
  }
}

// Subset DP (:119-165) by one lane for up to nv leaves, straight-line code with the costs in
// registers (treelet_dp_unrolled.cuh); best splits into this lane's column P.
template <int NVMAX = kTlMax>
__device__ __forceinline__ void reg_dp(int nv, const float* A, uint8_t* P) {
  if (NVMAX <= 4 || nv <= 4) dp_unrolled_4(A, P);
  else if (NVMAX <= 5 || nv == 5) dp_unrolled_5(A, P);
  else if (NVMAX <= 6 || nv == 6) dp_unrolled_6(A, P);
  else dp_unrolled_7(A, P);
}

// Id reuse (:167-191): the treelet's internal nodes in DFS order from the root, right child
// popped first, from the cached expansions.  Returns how many were found.
template <typename TL>
__device__ __forceinline__ int reg_avail(const Node* nodes, int32_t root, const TL& T, int* avail) {
  const int n = T.n;
  int n_avail = 0;
  int stack[kTlMax + 8];
  int top = 0;
  stack[top++] = root;
  while (top > 0) {
    const int cur = stack[--top];
    bool in_leaves = false;
#pragma unroll
    for (int i = 0; i < kTlMax; ++i)
      if (i < n && T.id[i] == cur) in_leaves = true;
    if (!in_leaves && n_avail < kTlMax && top + 2 <= kTlMax + 8) {
      avail[n_avail++] = cur;
      int2 ch = make_int2(0, 0);
      bool known = false;
#pragma unroll
      for (int e = 0; e < kTlMax - 1; ++e)
        if (!known && e < n - 1 && T.en[e] == cur) {
          ch = make_int2(T.el[e], T.er[e]);
          known = true;
        }
      if (!known) ch = ldcg_children(nodes, cur);
      stack[top++] = ch.x;
      stack[top++] = ch.y;
    }
  }
  return n_avail;
}

// Rebuild (:194-246) from the partitions P (this lane's column, stride 32), breadth-first,
// handing out the reused ids in order.  A subset with no finite split (NaN areas) leaves the
// treelet unchanged.
template <int PSTRIDE>
__device__ __forceinline__ void reg_build(Node* nodes, const RegTreelet& T, const uint8_t* P, const int* avail,
                                          int n_avail) {
  const int n = T.n;
  const uint32_t full = (1u << n) - 1u;
  {
    int vm[kTlMax], vh = 0, vt = 0;
    vm[vt++] = (int)full;
    while (vh < vt) {
      const int mask = vm[vh++];
      const int lm = P[mask * PSTRIDE], rm = mask ^ lm;
      if (lm == 0 || rm == 0 || (lm & ~mask)) return;
      if (__popc(lm) > 1) { if (vt >= kTlMax) return; vm[vt++] = lm; }
      if (__popc(rm) > 1) { if (vt >= kTlMax) return; vm[vt++] = rm; }
    }
    if (n_avail != n - 1) return;
  }
  int qm[kTlMax], qn[kTlMax];
  int qh = 0, qt = 0, used = 1;
  qm[qt] = (int)full;
  qn[qt++] = avail[0];
  while (qh < qt) {
    const int mask = qm[qh], cur = qn[qh];
    qh++;
    const int lm = P[mask * PSTRIDE], rm = mask ^ lm;
    int li, ri;
    if (__popc(lm) == 1) li = reg_id(T, __ffs(lm) - 1);
    else { li = avail[used++]; qm[qt] = lm; qn[qt++] = li; }
    if (__popc(rm) == 1) ri = reg_id(T, __ffs(rm) - 1);
    else { ri = avail[used++]; qm[qt] = rm; qn[qt++] = ri; }
    const Box b = reg_union(T, (uint32_t)mask);
    float4* p = reinterpret_cast<float4*>(nodes + cur);
    __stcg(p, b.lo);
    __stcg(p + 1, b.hi);
    __stcg(reinterpret_cast<int2*>(&nodes[cur].left), make_int2(li, ri));
    __stcg(&nodes[li].aux0, cur);
    __stcg(&nodes[ri].aux0, cur);
  }
}

// Heights: a climb from every leaf; the first child to reach a parent leaves its height in the
// rendezvous word, the second computes the parent's.
__global__ void __launch_bounds__(256) k_tl_heights(const Node* __restrict__ nodes, unsigned long long* __restrict__ slots,
                                                    const uint32_t* epoch_word, uint32_t round, uint32_t n,
                                                    uint8_t* __restrict__ hgt, uint32_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long tag = (unsigned long long)(__ldcg(epoch_word) + 1u + round) << 32;
  int32_t idx = (int32_t)(n - 1 + i);
  uint32_t h = 0;
  while (idx != 0) {
    const int32_t parent = __ldcg(&nodes[idx].aux0);
    const unsigned long long old = atomicExch(slots + parent, tag | h);
    if ((old & 0xffffffff00000000ull) != tag) return;  // first child to arrive
    h = 1u + max(h, (uint32_t)old);
    if (h > (uint32_t)kTlMaxHeight) {
      atomicOr(flags, 1u);
      h = kTlMaxHeight + 1;
    }
    hgt[parent] = (uint8_t)h;
    idx = parent;
  }
}

// Nodes per height (block histograms in shared memory, one global add per nonzero bin).
__global__ void __launch_bounds__(256) k_tl_count(const uint8_t* __restrict__ hgt, uint32_t m, uint32_t* __restrict__ cnt) {
  __shared__ uint32_t s_cnt[256];
  s_cnt[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    atomicAdd(&s_cnt[hgt[i]], 1u);
  __syncthreads();
  const uint32_t c = s_cnt[threadIdx.x];
  if (c) atomicAdd(cnt + threadIdx.x, c);
}

// off[h] = first list position of height h (exclusive scan of cnt over 256 heights), cursor
// copy for the scatter, off[256] = total, flags[1] = the largest height.  A total other than
// the m internal nodes (a malformed tree) hands the pass to the fallback.
__global__ void __launch_bounds__(256) k_tl_offsets(const uint32_t* __restrict__ cnt, uint32_t m,
                                                    uint32_t* __restrict__ off, uint32_t* __restrict__ cursor,
                                                    uint32_t* __restrict__ flags) {
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_maxh;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) s_maxh = 0;
  const uint32_t v = cnt[t];
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[w] = x;
  __syncthreads();
  if (v) atomicMax(&s_maxh, (uint32_t)t);
  uint32_t before = 0;
  for (int k = 0; k < w; ++k) before += s_w[k];
  off[t] = before + x - v;
  cursor[t] = before + x - v;
  if (t == 255) {
    off[256] = before + x;
    if (before + x != m) atomicOr(flags, 2u);
  }
  __syncthreads();
  if (t == 0) {
    flags[1] = s_maxh;
    flags[2] = 1;  // the first height processed
  }
}

// Internal node ids grouped by height (order within a height is irrelevant).
__global__ void __launch_bounds__(256) k_tl_scatter(const uint8_t* __restrict__ hgt, uint32_t m,
                                                    uint32_t* __restrict__ cursor, uint32_t* __restrict__ list) {
  __shared__ uint32_t s_cnt[256], s_base[256];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t h = i < m ? hgt[i] : 0u;
  const uint32_t rank = i < m ? atomicAdd(&s_cnt[h], 1u) : 0u;
  __syncthreads();
  const uint32_t c = s_cnt[threadIdx.x];
  if (c) s_base[threadIdx.x] = atomicAdd(cursor + threadIdx.x, c);
  __syncthreads();
  if (i < m) {
    const uint32_t pos = s_base[h] + rank;
    if (pos < m) list[pos] = i;
  }
}

// Per height, two kernels: k_tl_grow (latency-bound: many warps, few registers) refits each
// node, grows its treelet and writes a descriptor; k_tl_dp (compute-bound) reloads the leaf
// boxes, runs the DP and rebuilds.  Descriptors are structure-of-arrays, kTlDescWords words per
// node at stride `stride` (>= the largest height's node count): [0] n | n_avail << 8,
// [1..7] leaf ids, [8..13] reused internal ids in order.  ctl: [0] too high, [1] largest
// height, [2] current height.
constexpr int kGrowThreads = 128;

__global__ void __launch_bounds__(kGrowThreads, 8) k_tl_grow(Node* __restrict__ nodes, const uint32_t* __restrict__ list,
                                                          const uint32_t* __restrict__ off,
                                                          const uint32_t* __restrict__ ctl, uint32_t* __restrict__ desc,
                                                          uint32_t stride) {
  if (__ldcg(ctl) != 0u) return;  // too high: the fallback pass does the work
  const uint32_t h = __ldcg(ctl + 2);
  const uint32_t b = __ldcg(off + h), e = __ldcg(off + h + 1);
  for (uint32_t k = b + blockIdx.x * blockDim.x + threadIdx.x; k < e; k += gridDim.x * blockDim.x) {
    const int32_t x = (int32_t)__ldcg(list + k);
    const int2 ch = ldcg_children(nodes, x);
    // the children's boxes (the refit) and their own children (the root's expansion) together
    const Box lb = ldcg_box(nodes, ch.x), rb = ldcg_box(nodes, ch.y);
    const int2 lc = h == 1 ? make_int2(0, 0) : ldcg_children(nodes, ch.x);
    const int2 rc = h == 1 ? make_int2(0, 0) : ldcg_children(nodes, ch.y);
    const Box box = box_union(lb, rb);
    float4* p = reinterpret_cast<float4*>(nodes + x);
    __stcg(p, box.lo);
    __stcg(p + 1, box.hi);
    const uint32_t q = k - b;
    // growth expands the root first, unless its area is not above -1 (NaN): then n = 1
    const bool expand = box_area(box) > -1.0f;
    if (h == 1) {  // both children are BVH leaves: the two-leaf treelet below, without growing it
      if (expand) __stcg(reinterpret_cast<int2*>(&nodes[x].left), make_int2(ch.y, ch.x));
      desc[q] = 0u;
      continue;
    }
    GrowTreelet T;
    if (expand) reg_grow_expanded(nodes, x, ch, lb, rb, lc, rc, T);
    else reg_grow(nodes, x, box, ch, T);
    if (T.n == 2) {
      // Two leaves (the root's children; both are BVH leaves): the DP's only split puts the
      // second leaf left, so the rebuild swaps the children (box and parent links stay).
      __stcg(reinterpret_cast<int2*>(&nodes[x].left), make_int2(T.id[1], T.id[0]));
      desc[q] = 0u;  // nothing left for k_tl_dp
      continue;
    }
    int avail[kTlMax];
    const int na = T.n >= 2 ? reg_avail(nodes, x, T, avail) : 0;
    desc[q] = (uint32_t)T.n | ((uint32_t)na << 8);
#pragma unroll
    for (int i = 0; i < kTlMax; ++i) desc[(size_t)(1 + i) * stride + q] = (uint32_t)T.id[i];
#pragma unroll
    for (int i = 0; i < kTlMax - 1; ++i) desc[(size_t)(8 + i) * stride + q] = i < na ? (uint32_t)avail[i] : 0u;
  }
}

// One lane's treelet q of the current height (act: a real one): leaf ids and boxes from its
// descriptor and the nodes, subset areas and the DP in this lane's shared-memory columns C and
// P (stride 32), then the rebuild.  The warp runs the DP variant of its largest treelet, at most
// NVMAX leaves.  Called by all 32 lanes together.
template <int NVMAX>
__device__ __forceinline__ void lane_dp(Node* nodes, const uint32_t* desc, uint32_t stride, uint32_t q, bool act,
                                        float* C, uint8_t* P) {
  const uint32_t w0 = act ? __ldcg(desc + q) : 0u;
  RegTreelet T;
  T.n = (int)(w0 & 255u);
  const int na = (int)(w0 >> 8);
#pragma unroll
  for (int i = 0; i < kTlMax; ++i) {
    T.id[i] = i < NVMAX && i < T.n ? (int32_t)__ldcg(desc + (size_t)(1 + i) * stride + q) : 0;
    T.b[i] = i < NVMAX && i < T.n ? ldcg_box(nodes, T.id[i]) : box_empty();
  }
  const int nv = (int)__reduce_max_sync(0xffffffffu, (uint32_t)T.n);
  if (nv < 2) return;
  reg_areas<NVMAX>(T, nv, C);
  reg_dp<NVMAX>(nv, C, P);
  if (T.n >= 2) {
    int avail[kTlMax];
#pragma unroll
    for (int i = 0; i < kTlMax - 1; ++i) avail[i] = (int)__ldcg(desc + (size_t)(8 + i) * stride + q);
    reg_build<32>(nodes, T, P, avail, na);
  }
}

// NVMAX < kTlMax: a DP for treelets of at most NVMAX leaves (heights where no more fit: height 2
// holds at most 4), compiled for fewer registers, so more warps share an SM.
template <int NVMAX>
__global__ void __launch_bounds__(kLvThreads) k_tl_dp(Node* __restrict__ nodes, const uint32_t* __restrict__ off,
                                                      const uint32_t* __restrict__ ctl,
                                                      const uint32_t* __restrict__ desc, uint32_t stride) {
  // per-lane columns of 2^NVMAX costs and partitions (the narrow path below uses 768 words)
  __shared__ float s_cost[std::max((1 << NVMAX) * 32, 1024)];
  __shared__ uint8_t s_part[(1 << NVMAX) * 32];
  if (__ldcg(ctl) != 0u) return;
  const uint32_t h = __ldcg(ctl + 2);
  const uint32_t b = __ldcg(off + h), e = __ldcg(off + h + 1);
  const int lane = threadIdx.x & 31;
  if (e - b <= 8u * gridDim.x) {
    // a narrow height: one treelet per warp with the warp-cooperative DP (shorter critical path)
    LaneTreelet& S = *reinterpret_cast<LaneTreelet*>(s_cost);
    float* cost = s_cost + 512;
    float* area = s_cost + 640;
    for (uint32_t k = b + blockIdx.x; k < e; k += gridDim.x) {
      const uint32_t q = k - b;
      const uint32_t w0 = __ldcg(desc + q);
      const int n = (int)(w0 & 255u);
      if (n < 2) continue;  // uniform over the warp
      if (lane < kTlMax) {
        const int32_t id = (int32_t)__ldcg(desc + (size_t)(1 + lane) * stride + q);
        S.act[lane] = id;
        const Box bx = lane < n ? ldcg_box(nodes, id) : box_empty();
        S.box[0][lane] = bx.lo.x; S.box[1][lane] = bx.lo.y; S.box[2][lane] = bx.lo.z;
        S.box[3][lane] = bx.hi.x; S.box[4][lane] = bx.hi.y; S.box[5][lane] = bx.hi.z;
      }
      if (lane == 0) S.n = n;
      __syncwarp();
      treelet_dp(S, cost, area);
      if (lane == 0) {
        RegTreelet T;
        T.n = n;
#pragma unroll
        for (int i = 0; i < kTlMax; ++i) {
          T.id[i] = S.act[i];
          T.b[i] = leaf_box(S, i);
        }
        int avail[kTlMax];
#pragma unroll
        for (int i = 0; i < kTlMax - 1; ++i) avail[i] = (int)__ldcg(desc + (size_t)(8 + i) * stride + q);
        reg_build<1>(nodes, T, S.part, avail, (int)(w0 >> 8));
      }
      __syncwarp();
    }
    return;
  }
  float* C = s_cost + lane;
  uint8_t* P = s_part + lane;
  // warp-uniform loop: the warp runs the DP variant of its largest treelet
  for (uint32_t kb = b + blockIdx.x * kLvThreads; kb < e; kb += gridDim.x * kLvThreads) {
    const uint32_t k = kb + lane;
    lane_dp<NVMAX>(nodes, desc, stride, k - b, k < e, C, P);
  }
}

// A height where treelet sizes are mixed (height 3: most treelets have 4 or 5 leaves, few 7):
// one kernel per size class, NV = 4 (3 or 4 leaves), 5, 6, 7, each running only the
// height's treelets of its class, so a warp runs the DP its own treelets need.  Each warp scans
// R rounds of 32 nodes, packs those of its class into a shared list (ballots) and runs them 32
// at a time; R shrinks with the height's node count so that every block gets a chunk.
template <int NV>
__global__ void __launch_bounds__(kLvThreads) k_tl_dpc(Node* __restrict__ nodes, const uint32_t* __restrict__ off,
                                                       const uint32_t* __restrict__ ctl,
                                                       const uint32_t* __restrict__ desc, uint32_t stride) {
  constexpr int R = 8;
  __shared__ float s_cost[(1 << NV) * 32];
  __shared__ uint8_t s_part[(1 << NV) * 32];
  __shared__ uint32_t s_list[32 * R];
  if (__ldcg(ctl) != 0u) return;
  const uint32_t h = __ldcg(ctl + 2);
  const uint32_t b = __ldcg(off + h), e = __ldcg(off + h + 1);
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  float* C = s_cost + lane;
  uint8_t* P = s_part + lane;
  const uint32_t rounds = max(1u, min((uint32_t)R, div_up(e - b, 32u * gridDim.x)));
  for (uint32_t chunk = b + blockIdx.x * (32u * rounds); chunk < e; chunk += gridDim.x * (32u * rounds)) {
    uint32_t cnt = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
      const uint32_t k = chunk + r * 32u + (uint32_t)lane;
      const int n = k < e ? (int)(__ldcg(desc + (k - b)) & 255u) : 0;
      const bool match = n >= 2 && (n <= 4 ? 4 : n) == NV;
      const uint32_t bal = __ballot_sync(0xffffffffu, match);
      if (match) s_list[cnt + __popc(bal & lt)] = k - b;
      cnt += (uint32_t)__popc(bal);
    }
    __syncwarp();
    for (uint32_t i = 0; i < cnt; i += 32) {
      const bool act = i + (uint32_t)lane < cnt;
      lane_dp<NV>(nodes, desc, stride, act ? s_list[i + lane] : 0u, act, C, P);
    }
    __syncwarp();  // the list is refilled by the next chunk
  }
}

// The narrow heights in one cooperative launch.  Once a height has few nodes, its two launches
// (growth, DP) cost mostly their latency; k_tl_narrow runs the remaining heights, from the current
// one (ctl[2]) to the largest (ctl[1]), with a grid barrier between heights (nodes of one height
// have disjoint subtrees, a height needs all lower ones done).  Per node, one warp: lane 0 refits
// the node and grows its treelet (as k_tl_grow), the warp runs the cooperative DP and lane 0
// rebuilds (as k_tl_dp's narrow path).  Same work and result as the per-height kernels.
constexpr int kNarrowThreads = 256;

struct NarrowWarp {
  LaneTreelet S;
  float cost[1 << kTlMax];
  float area[1 << kTlMax];
  int32_t avail[kTlMax];
  int32_t na;
};

__global__ void __launch_bounds__(kNarrowThreads) k_tl_narrow(Node* __restrict__ nodes, const uint32_t* __restrict__ list,
                                                              const uint32_t* __restrict__ off, uint32_t* __restrict__ ctl,
                                                              uint32_t* __restrict__ status) {
  __shared__ NarrowWarp s_warp[kNarrowThreads / 32];
  __shared__ uint32_t s_ok;
  // every block reads the same words (nothing writes them in this kernel)
  if (__ldcg(ctl) != 0u) return;  // too high: the fallback pass does the work
  const uint32_t h0 = __ldcg(ctl + 2), h1 = __ldcg(ctl + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  NarrowWarp& W = s_warp[w];
  const uint32_t gw = blockIdx.x * (kNarrowThreads / 32) + (uint32_t)w, nw = gridDim.x * (kNarrowThreads / 32);
  uint32_t nbar = 0;
  for (uint32_t h = h0; h <= h1; ++h) {
    const uint32_t b = __ldcg(off + h), e = __ldcg(off + h + 1);
    for (uint32_t k = b + gw; k < e; k += nw) {
      if (lane == 0) {
        const int32_t x = (int32_t)__ldcg(list + k);
        const int2 ch = ldcg_children(nodes, x);
        const Box box = box_union(ldcg_box(nodes, ch.x), ldcg_box(nodes, ch.y));
        float4* p = reinterpret_cast<float4*>(nodes + x);
        __stcg(p, box.lo);
        __stcg(p + 1, box.hi);
        GrowTreelet T;
        reg_grow(nodes, x, box, ch, T);
        W.S.n = T.n;
#pragma unroll
        for (int i = 0; i < kTlMax; ++i) W.S.act[i] = T.id[i];
        W.na = T.n >= 2 ? reg_avail(nodes, x, T, W.avail) : 0;
      }
      __syncwarp();
      const int n = W.S.n;
      if (n >= 2) {  // uniform over the warp
        if (lane < kTlMax) {
          const Box bx = lane < n ? ldcg_box(nodes, W.S.act[lane]) : box_empty();
          W.S.box[0][lane] = bx.lo.x; W.S.box[1][lane] = bx.lo.y; W.S.box[2][lane] = bx.lo.z;
          W.S.box[3][lane] = bx.hi.x; W.S.box[4][lane] = bx.hi.y; W.S.box[5][lane] = bx.hi.z;
        }
        __syncwarp();
        treelet_dp(W.S, W.cost, W.area);
        if (lane == 0) {
          RegTreelet T;
          T.n = n;
#pragma unroll
          for (int i = 0; i < kTlMax; ++i) {
            T.id[i] = W.S.act[i];
            T.b[i] = leaf_box(W.S, i);
          }
          reg_build<1>(nodes, T, W.S.part, W.avail, W.na);
        }
      }
      __syncwarp();
    }
    if (h < h1 && !grid_sync(ctl + 4, ++nbar * gridDim.x, status, &s_ok)) return;
  }
}

// End of a height: the next one, and whether the loop goes on (the graph's WHILE condition;
// the host-driven loop only advances the height).  The loop also stops at the first height of
// at most `narrow` nodes (0: never), from which k_tl_narrow goes on.
template <bool GRAPH>
__global__ void k_tl_step(uint32_t* __restrict__ ctl, const uint32_t* __restrict__ off, uint32_t narrow,
                          cudaGraphConditionalHandle handle) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t h = ctl[2] + 1;
  ctl[2] = h;
  bool go = ctl[0] == 0u && h <= ctl[1];
  if (go && narrow && off[h + 1] - off[h] <= narrow) go = false;
  if constexpr (GRAPH) cudaGraphSetConditional(handle, go ? 1u : 0u);
}

// The climb-ordered pass as a fallback for trees higher than kTlMaxHeight: persistent warps
// take groups of 32 leaves.  Launched every pass; returns at once unless flags[0] is set.
__global__ void __launch_bounds__(64) k_treelet_fallback(Node* __restrict__ nodes, unsigned long long* __restrict__ slots,
                                                         const uint32_t* epoch_word, uint32_t round, uint32_t n,
                                                         const uint32_t* __restrict__ flags) {
  __shared__ LaneTreelet S[64];
  __shared__ float s_cost[2][1 << kTlMax], s_area[2][1 << kTlMax];
  if (__ldcg(flags) == 0u) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned long long tag = (unsigned long long)(__ldcg(epoch_word) + 0x20u + round) << 32;
  LaneTreelet& mine = S[threadIdx.x];
  for (uint32_t base = (blockIdx.x * 2 + w) * 32u; base < n; base += gridDim.x * 64u) {
    const uint32_t i = base + lane;
    bool active = i < n;
    int32_t idx = (int32_t)(n - 1 + i);
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
            active = false;
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
      if (work) treelet_grow(nodes, idx, mine);
      __syncwarp();
      uint32_t ballot = __ballot_sync(0xffffffffu, work && mine.n >= 2);
      while (ballot) {
        const int src = __ffs(ballot) - 1;
        ballot &= ballot - 1;
        treelet_dp(S[w * 32 + src], s_cost[w], s_area[w]);
      }
      __syncwarp();
      if (work) treelet_rebuild(nodes, idx, mine);
      __threadfence();
    }
  }
}

static int g_dp_grid[64] = {};      // resident blocks of k_tl_dp per device
static int g_dp4_grid[64] = {};     // resident blocks of k_tl_dp<4> per device
static int g_dpc_grid[64][4] = {};  // resident blocks of k_tl_dpc<4..7> per device
static int g_narrow_grid[64] = {};  // resident blocks of k_tl_narrow per device (-1: no cooperative launch)

// The loop over heights as a graph: WHILE(cond) { grow; dp; step }.
static cudaError_t make_height_graph(Node* nodes, const uint32_t* list, const uint32_t* off, uint32_t* ctl,
                                     uint32_t* desc, uint32_t stride, uint32_t grow_grid, uint32_t dp_grid,
                                     uint32_t narrow, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaStream_t cs = nullptr;
  do {
    cudaGraphConditionalHandle handle;
    if ((e = cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp)) != cudaSuccess) break;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      break;
    k_tl_grow<<<grow_grid, kGrowThreads, 0, cs>>>(nodes, list, off, ctl, desc, stride);
    k_tl_dp<kTlMax><<<dp_grid, kLvThreads, 0, cs>>>(nodes, off, ctl, desc, stride);
    k_tl_step<true><<<1, 32, 0, cs>>>(ctl, off, narrow, handle);
    cudaGraph_t captured = nullptr;
    const cudaError_t e2 = cudaGetLastError();
    e = cudaStreamEndCapture(cs, &captured);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) break;
    e = cudaGraphInstantiate(out, g, 0);
  } while (false);
  if (cs) cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  return e;
}

cudaError_t treelet_rounds_run(Workspace& ws, uint32_t n, int rounds, cudaStream_t st, int fb, bool host_loop) {
  if (n < 2) return cudaSuccess;
  ScratchLayout L = scratch_layout(ws.cap_n);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if (!g_dp_grid[dev]) {
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tl_dp<kTlMax>, kLvThreads, 0)) != cudaSuccess)
      return e;
    g_dp_grid[dev] = std::max(1, per_sm * sms);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tl_dp<4>, kLvThreads, 0)) != cudaSuccess) return e;
    g_dp4_grid[dev] = std::max(1, per_sm * sms);
    const void* dpc[4] = {reinterpret_cast<const void*>(k_tl_dpc<4>), reinterpret_cast<const void*>(k_tl_dpc<5>),
                          reinterpret_cast<const void*>(k_tl_dpc<6>), reinterpret_cast<const void*>(k_tl_dpc<7>)};
    for (int c = 0; c < 4; ++c) {
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dpc[c], kLvThreads, 0)) != cudaSuccess) return e;
      g_dpc_grid[dev][c] = std::max(1, per_sm * sms);
    }
  }
  if (!g_narrow_grid[dev]) {
    int coop = 0, per_sm = 0;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tl_narrow, kNarrowThreads, 0)) != cudaSuccess)
      return e;
    g_narrow_grid[dev] = coop && per_sm > 0 ? per_sm * sms : -1;
  }
  // heights of at most `narrow` nodes (two per warp of the cooperative grid) run in k_tl_narrow
  const uint32_t narrow =
      !host_loop && g_narrow_grid[dev] > 0 ? 2u * (uint32_t)g_narrow_grid[dev] * (kNarrowThreads / 32) : 0u;
  // scratch: heights in the delta bytes (emission is done with them), the id list in the idle
  // value buffer, descriptors in the triangle boxes (32 B per triangle; a height has at most
  // n/2 nodes), counters / offsets / control words in the sort histogram words
  uint8_t* hgt = ws.delta;
  uint32_t* list = ws.vals[fb ^ 1];
  uint32_t* desc = reinterpret_cast<uint32_t*>(ws.boxes);
  const uint32_t stride = std::max<uint32_t>(n / 2, 1);
  uint32_t* cnt = ws.scratch + L.hist;       // 256
  uint32_t* off = cnt + 256;                 // 257
  uint32_t* cursor = off + 264;              // 256
  uint32_t* ctl = cursor + 256;              // [0] too high, [1] largest height, [2] current height
  static_assert(kTlCtlWord == 256 + 264 + 256, "control words of the treelet pass");
  static_assert(kTlCtlWord + 8 <= (size_t)kMaxPasses * 256, "treelet words fit the histogram area");
  const uint32_t* epoch = ws.scratch + L.epoch;
  const uint32_t grow_grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(stride, kGrowThreads), sms * 16));
  if (host_loop && !ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
  const bool same = host_loop || ws.tl_exec && ws.tl_key_n == n && ws.tl_key_nodes == ws.nodes && ws.tl_key_list == list &&
                    ws.tl_key_desc == desc && ws.tl_key_ctl == ctl;
  if (!same) {
    if (ws.tl_exec) cudaGraphExecDestroy(ws.tl_exec);
    ws.tl_exec = nullptr;
    if ((e = make_height_graph(ws.nodes, list, off, ctl, desc, stride, grow_grid, (uint32_t)g_dp_grid[dev], narrow,
                               &ws.tl_exec)) != cudaSuccess)
      return e;
    ws.tl_key_n = n;
    ws.tl_key_nodes = ws.nodes;
    ws.tl_key_list = list;
    ws.tl_key_desc = desc;
    ws.tl_key_ctl = ctl;
  }
  ws.tl_narrow = narrow != 0;
  for (int r = 0; r < rounds && r + 1 < 0x20; ++r) {
    if ((e = cudaMemsetAsync(cnt, 0, 256 * 4, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(ctl, 0, 8 * 4, st)) != cudaSuccess) return e;  // [4]: k_tl_narrow's barrier
    k_tl_heights<<<div_up(n, 256), 256, 0, st>>>(ws.nodes, ws.slots, epoch, (uint32_t)r, n, hgt, ctl);
    k_tl_count<<<std::max<uint32_t>(1, std::min<uint32_t>(div_up(n - 1, 256), sms * 8)), 256, 0, st>>>(hgt, n - 1, cnt);
    k_tl_offsets<<<1, 256, 0, st>>>(cnt, n - 1, off, cursor, ctl);
    k_tl_scatter<<<div_up(n - 1, 256), 256, 0, st>>>(hgt, n - 1, cursor, list);
    // heights 1 to 3 first: every height-1 treelet has two leaves and is finished by the growth
    // kernel; height 2 holds at most 4 leaves and takes the smaller DP; height 3 mixes treelet
    // sizes (mostly 4 and 5 leaves, few 7) and runs one DP per size class
    k_tl_grow<<<grow_grid, kGrowThreads, 0, st>>>(ws.nodes, list, off, ctl, desc, stride);
    k_tl_step<false><<<1, 32, 0, st>>>(ctl, off, 0u, cudaGraphConditionalHandle{});
    k_tl_grow<<<grow_grid, kGrowThreads, 0, st>>>(ws.nodes, list, off, ctl, desc, stride);
    k_tl_dp<4><<<g_dp4_grid[dev], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
    k_tl_step<false><<<1, 32, 0, st>>>(ctl, off, 0u, cudaGraphConditionalHandle{});
    k_tl_grow<<<grow_grid, kGrowThreads, 0, st>>>(ws.nodes, list, off, ctl, desc, stride);
    k_tl_dpc<4><<<g_dpc_grid[dev][0], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
    k_tl_dpc<5><<<g_dpc_grid[dev][1], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
    k_tl_dpc<6><<<g_dpc_grid[dev][2], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
    k_tl_dpc<7><<<g_dpc_grid[dev][3], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
    k_tl_step<false><<<1, 32, 0, st>>>(ctl, off, 0u, cudaGraphConditionalHandle{});
    if (host_loop) {
      // read the largest height (and the too-high flag) once, then one grow + dp per height
      if ((e = cudaMemcpyAsync(ws.ploc_host, ctl, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
      const uint32_t maxh = ws.ploc_host[0] ? 0u : ws.ploc_host[1];
      for (uint32_t h = 4; h <= maxh; ++h) {
        k_tl_grow<<<grow_grid, kGrowThreads, 0, st>>>(ws.nodes, list, off, ctl, desc, stride);
        k_tl_dp<kTlMax><<<g_dp_grid[dev], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
        k_tl_step<false><<<1, 32, 0, st>>>(ctl, off, 0u, cudaGraphConditionalHandle{});
      }
    } else {
      if ((e = cudaGraphLaunch(ws.tl_exec, st)) != cudaSuccess) return e;
      if (narrow) {  // the remaining heights, from where the graph's loop stopped
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((uint32_t)g_narrow_grid[dev]);
        cfg.blockDim = dim3(kNarrowThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = ws.no_cooperative ? cudaErrorNotSupported
                              : cudaLaunchKernelEx(&cfg, k_tl_narrow, ws.nodes, (const uint32_t*)list,
                                                   (const uint32_t*)off, ctl, ws.scratch + L.status);
        if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
          // no co-resident grid (a client limited to part of the GPU, or asked for): the
          // remaining heights as one grow + dp launch each, driven from the host
          (void)cudaGetLastError();
          ws.tl_narrow = false;
          if (!ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
          if ((e = cudaMemcpyAsync(ws.ploc_host, ctl, 12, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
              (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return e;
          if (!ws.ploc_host[0])
            for (uint32_t h = ws.ploc_host[2]; h <= ws.ploc_host[1]; ++h) {
              k_tl_grow<<<grow_grid, kGrowThreads, 0, st>>>(ws.nodes, list, off, ctl, desc, stride);
              k_tl_dp<kTlMax><<<g_dp_grid[dev], kLvThreads, 0, st>>>(ws.nodes, off, ctl, desc, stride);
              k_tl_step<false><<<1, 32, 0, st>>>(ctl, off, 0u, cudaGraphConditionalHandle{});
            }
        } else if (e != cudaSuccess) {
          return e;
        }
      }
    }
    k_treelet_fallback<<<sms * 8, 64, 0, st>>>(ws.nodes, ws.slots, epoch, (uint32_t)r, n, ctl);
  }
  return cudaGetLastError();
}

}  // namespace bvhgb
