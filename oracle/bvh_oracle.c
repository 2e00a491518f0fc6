/*
 * bvh_oracle.c -- CPU restatement of the reference BVH builders (TEST INFRASTRUCTURE).
 *
 * Used only as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg.  Compile with -ffp-contract=off so that every float operation rounds exactly as
 * written; FMA contractions that nvcc may apply to the reference's device code are
 * selected explicitly through orc_set_sa_form().
 *
 * Reference files cited below are paths inside the EdinHg/BVH project.
 */
#include "bvh_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_LEAF_BIT 0x80000000u

/* Form 3 is what nvcc emits for the reference's surfaceArea: measured bit-exact against the
 * reference PLOC nearest-neighbour kernel (kFindNearestNeighbors_ploc) on a GB300. */
static int g_sa_form = 3;
void orc_set_sa_form(int form) { g_sa_form = form; }
int orc_get_sa_form(void) { return g_sa_form; }

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* fminf/fmaxf as the GPU evaluates them (PTX min.f32/max.f32): a NaN operand is ignored,
 * and when both operands are zeros of different sign min gives -0 and max gives +0. */
float orc_fmin(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a == b) return signbit(a) ? a : b;
  return a < b ? a : b;
}
float orc_fmax(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a == b) return signbit(a) ? b : a;
  return a > b ? a : b;
}

static inline float sa_xyz(float x, float y, float z) {
  float s;
  switch (g_sa_form) {
    case 1: s = fmaf(z, x, (x * y) + (y * z)); break;
    case 2: s = fmaf(x, y, y * z) + (z * x); break;
    case 3: s = fmaf(z, x, fmaf(x, y, y * z)); break;
    case 4: s = fmaf(y, z, x * y) + (z * x); break;
    case 5: s = fmaf(z, x, fmaf(y, z, x * y)); break;
    case 6: s = fmaf(x, y, fmaf(y, z, z * x)); break;
    case 7: s = fmaf(y, z, fmaf(x, y, z * x)); break;
    default: s = ((x * y) + (y * z)) + (z * x); break;
  }
  return 2.0f * s;
}

/* AABB_cw::surfaceArea, include/common.h:41-44. */
float orc_sa(const orc_aabb* b) {
  return sa_xyz(b->mx[0] - b->mn[0], b->mx[1] - b->mn[1], b->mx[2] - b->mn[2]);
}
/* Host-compiled surfaceArea as the reference evaluator uses it (no contraction on x86-64). */
static inline float sa_plain(const orc_aabb* b) {
  float x = b->mx[0] - b->mn[0], y = b->mx[1] - b->mn[1], z = b->mx[2] - b->mn[2];
  return 2.0f * (((x * y) + (y * z)) + (z * x));
}

static inline void box_empty(orc_aabb* b) {
  b->mn[0] = b->mn[1] = b->mn[2] = FLT_MAX;
  b->mx[0] = b->mx[1] = b->mx[2] = -FLT_MAX;
  b->pad0 = b->pad1 = 0.0f;
}
/* AABB_cw::merge, include/common.h:46-64 (device branch: fminf/fmaxf, this first). */
static inline orc_aabb box_merge(const orc_aabb* a, const orc_aabb* b) {
  orc_aabb r;
  for (int k = 0; k < 3; ++k) {
    r.mn[k] = orc_fmin(a->mn[k], b->mn[k]);
    r.mx[k] = orc_fmax(a->mx[k], b->mx[k]);
  }
  r.pad0 = r.pad1 = 0.0f;
  return r;
}

/* kComputeBoundsAndCentroids_nt, src/cuda/lbvh_builder.cu:47-66 (identical in
 * lbvh_plus_builder.cu:255-274 and ploc_builder.cu:33-57). */
void orc_tri_bounds(const orc_mesh* m, orc_aabb* boxes, float* c4) {
  const int64_t n = m->n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    orc_aabb b;
    for (int k = 0; k < 3; ++k) {
      float a0 = m->v[k][i], a1 = m->v[3 + k][i], a2 = m->v[6 + k][i];
      b.mn[k] = orc_fmin(a0, orc_fmin(a1, a2));
      b.mx[k] = orc_fmax(a0, orc_fmax(a1, a2));
    }
    b.pad0 = b.pad1 = 0.0f;
    boxes[i] = b;
    if (c4) {
      for (int k = 0; k < 3; ++k) c4[4 * i + k] = (b.mn[k] + b.mx[k]) * 0.5f;
      c4[4 * i + 3] = 0.0f;
    }
  }
}

/* kReduceBounds_Step1_nt/Step2_nt, src/cuda/lbvh_builder.cu:73-165. */
void orc_scene_bounds(const orc_aabb* boxes, uint32_t n, orc_aabb* out) {
  orc_aabb acc;
  box_empty(&acc);
  for (uint32_t i = 0; i < n; ++i) acc = box_merge(&acc, &boxes[i]);
  *out = acc;
}

/* expandBits_nt, src/cuda/lbvh_builder.cu:11-17. */
static inline uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
/* expandBits_P, src/cuda/lbvh_plus_builder.cu:20-28. */
static inline uint64_t expand21(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

/* kComputeMortonCodes_nt (src/cuda/lbvh_builder.cu:167-181) with morton3D_nt (:19-27);
 * kComputeMortonCodes_P (src/cuda/lbvh_plus_builder.cu:276-290) with morton3D_P (:30-35). */
void orc_morton(const float* c4, uint32_t n, int bits, const orc_aabb* scene, uint64_t* codes) {
  float ext[3], mn[3];
  for (int k = 0; k < 3; ++k) {
    float e = scene->mx[k] - scene->mn[k];
    ext[k] = (e > 1e-6f) ? e : 1.0f;
    mn[k] = scene->mn[k];
  }
  const float scale = bits == 30 ? 1024.0f : (bits == 60 ? 1048576.0f : 2097152.0f);
  const float top = bits == 30 ? 1023.0f : (bits == 60 ? 1048575.0f : 2097151.0f);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    float q[3];
    for (int k = 0; k < 3; ++k) {
      float x = (c4[4 * i + k] - mn[k]) / ext[k];
      q[k] = orc_fmin(orc_fmax(x * scale, 0.0f), top);
    }
    if (bits == 30) {
      uint32_t xx = expand10((uint32_t)q[0]), yy = expand10((uint32_t)q[1]), zz = expand10((uint32_t)q[2]);
      codes[i] = (uint64_t)(uint32_t)(xx * 4 + yy * 2 + zz);
    } else {
      codes[i] = (expand21((uint64_t)q[2]) << 2) | (expand21((uint64_t)q[1]) << 1) | expand21((uint64_t)q[0]);
    }
  }
}

/* Stable LSD radix sort of (key, idx); the reference uses cub::DeviceRadixSort::SortPairs
 * (src/cuda/lbvh_builder.cu:421-429) and thrust::sort_by_key (lbvh_plus_builder.cu:465,
 * ploc_builder.cu:459-461), both stable, so ties keep ascending original index. */
void orc_sort_pairs(uint64_t* keys, uint32_t* idx, uint32_t n, int key_bits, int init_idx) {
  if (init_idx)
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
  if (n < 2) return;
  uint64_t* k2 = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
  uint32_t* i2 = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
  uint64_t *ks = keys, *kd = k2;
  uint32_t *is = idx, *id = i2;
  int nthreads = orc_threads();
  size_t* hist = (size_t*)malloc((size_t)nthreads * 256 * sizeof(size_t));
  int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    int sh = 8 * p;
    memset(hist, 0, (size_t)nthreads * 256 * sizeof(size_t));
#pragma omp parallel num_threads(nthreads)
    {
      int t = 0, nt = 1;
#ifdef _OPENMP
      t = omp_get_thread_num();
      nt = omp_get_num_threads();
#endif
      size_t lo = (size_t)n * t / nt, hi = (size_t)n * (t + 1) / nt;
      size_t* h = hist + (size_t)t * 256;
      for (size_t i = lo; i < hi; ++i) h[(ks[i] >> sh) & 255]++;
#pragma omp barrier
#pragma omp single
      {
        size_t run = 0;
        for (int d = 0; d < 256; ++d)
          for (int tt = 0; tt < nt; ++tt) {
            size_t c = hist[(size_t)tt * 256 + d];
            hist[(size_t)tt * 256 + d] = run;
            run += c;
          }
      }
      for (size_t i = lo; i < hi; ++i) {
        size_t o = h[(ks[i] >> sh) & 255]++;
        kd[o] = ks[i];
        id[o] = is[i];
      }
    }
    uint64_t* tk = ks; ks = kd; kd = tk;
    uint32_t* ti = is; is = id; id = ti;
  }
  if (ks != keys) {
    memcpy(keys, ks, (size_t)n * sizeof(uint64_t));
    memcpy(idx, is, (size_t)n * sizeof(uint32_t));
  }
  free(hist);
  free(k2);
  free(i2);
}

/* delta_nt (src/cuda/lbvh_builder.cu:33-43) and delta_P (lbvh_plus_builder.cu:41-47). */
static inline int karras_delta(const uint64_t* k, const uint32_t* id, int64_t n, int64_t i, int64_t j, int w) {
  if (j < 0 || j >= n) return -1;
  uint64_t a = k[i], b = k[j];
  if (a == b) {
    uint32_t x = id[i] ^ id[j];
    if (w == 32) return 32 + (x == 0 ? 32 : __builtin_clz(x));
    return 64 + (x == 0 ? 64 : __builtin_clzll((uint64_t)x));
  }
  if (w == 32) {
    uint32_t x = (uint32_t)a ^ (uint32_t)b;
    return x == 0 ? 32 : __builtin_clz(x);
  }
  return __builtin_clzll(a ^ b);
}

/* kBuildInternalNodes_nt, src/cuda/lbvh_builder.cu:183-229. */
void orc_karras(const uint64_t* keys, const uint32_t* idx, uint32_t n_, int w, orc_node* nodes) {
  const int64_t n = n_;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n - 1; ++i) {
    int d = (karras_delta(keys, idx, n, i, i + 1, w) - karras_delta(keys, idx, n, i, i - 1, w)) >= 0 ? 1 : -1;
    int min_delta = karras_delta(keys, idx, n, i, i - d, w);
    int64_t l_max = 2;
    while (karras_delta(keys, idx, n, i, i + l_max * d, w) > min_delta) l_max *= 2;
    int64_t l = 0;
    for (int64_t t = l_max / 2; t >= 1; t /= 2)
      if (karras_delta(keys, idx, n, i, i + (l + t) * d, w) > min_delta) l += t;
    int64_t j = i + l * d;
    int delta_node = karras_delta(keys, idx, n, i, j, w);
    int64_t first = d > 0 ? i : j, last = d > 0 ? j : i;
    int64_t s = 0, t = last - first;
    do {
      t = (t + 1) >> 1;
      if (karras_delta(keys, idx, n, first, first + s + t, w) > delta_node) s += t;
    } while (t > 1);
    int64_t split = first + s;
    nodes[i].left = (int32_t)(split == first ? (n - 1) + split : split);
    nodes[i].right = (int32_t)(split + 1 == last ? (n - 1) + split + 1 : split + 1);
    nodes[i].pad[0] = nodes[i].pad[1] = 0;
  }
}

/* kInitLeafNodes_nt, src/cuda/lbvh_builder.cu:231-241. */
void orc_init_leaves(const orc_aabb* tri_boxes, const uint32_t* idx, uint32_t n, orc_node* nodes) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    orc_node* nd = &nodes[(int64_t)n - 1 + i];
    nd->box = tri_boxes[idx[i]];
    nd->left = (int32_t)(idx[i] | ORC_LEAF_BIT);
    nd->right = -1;
    nd->pad[0] = nd->pad[1] = 0;
  }
}

static inline int is_leaf(const orc_node* nd) { return ((uint32_t)nd->left & ORC_LEAF_BIT) != 0; }

/* Post-order list of internal nodes reachable from the root (children before parents). */
static uint32_t post_order(const orc_node* nodes, uint32_t n_nodes, uint32_t* order) {
  if (n_nodes == 0 || is_leaf(&nodes[0])) return 0;
  uint32_t* stack = (uint32_t*)malloc((size_t)n_nodes * sizeof(uint32_t) * 2 + 16);
  int64_t sp = 0;
  uint32_t cnt = 0;
  stack[sp++] = 0;
  /* reverse of a (node, right, left) pre-order is a valid post-order */
  while (sp > 0) {
    uint32_t x = stack[--sp];
    order[cnt++] = x;
    const orc_node* nd = &nodes[x];
    if (!is_leaf(&nodes[nd->left])) stack[sp++] = (uint32_t)nd->left;
    if (!is_leaf(&nodes[nd->right])) stack[sp++] = (uint32_t)nd->right;
  }
  for (uint32_t a = 0, b = cnt ? cnt - 1 : 0; a < b; ++a, --b) {
    uint32_t t = order[a]; order[a] = order[b]; order[b] = t;
  }
  free(stack);
  return cnt;
}

/* kRefitHierarchy_nt, src/cuda/lbvh_builder.cu:243-274: parent box = union(left, right). */
void orc_refit(orc_node* nodes, uint32_t n_nodes) {
  uint32_t* order = (uint32_t*)malloc((size_t)n_nodes * sizeof(uint32_t) + 4);
  uint32_t cnt = post_order(nodes, n_nodes, order);
  for (uint32_t k = 0; k < cnt; ++k) {
    orc_node* nd = &nodes[order[k]];
    nd->box = box_merge(&nodes[nd->left].box, &nodes[nd->right].box);
  }
  free(order);
}

int orc_lbvh(const orc_mesh* m, int bits, orc_node* nodes, uint32_t* indices, uint64_t* sorted_keys) {
  if (bits != 30 && bits != 60 && bits != 63) return ORC_ERR_INVALID;
  const uint32_t n = m->n;
  if (n == 0) return ORC_OK;
  orc_aabb* boxes = (orc_aabb*)malloc((size_t)n * sizeof(orc_aabb));
  float* c4 = (float*)malloc((size_t)n * 4 * sizeof(float));
  uint64_t* keys = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
  orc_tri_bounds(m, boxes, c4);
  orc_aabb scene;
  orc_scene_bounds(boxes, n, &scene);
  orc_morton(c4, n, bits, &scene, keys);
  orc_sort_pairs(keys, indices, n, bits, 1);
  orc_karras(keys, indices, n, bits == 30 ? 32 : 64, nodes);
  orc_init_leaves(boxes, indices, n, nodes);
  orc_refit(nodes, 2 * n - 1);
  if (sorted_keys) memcpy(sorted_keys, keys, (size_t)n * sizeof(uint64_t));
  free(boxes);
  free(c4);
  free(keys);
  return ORC_OK;
}

/* optimizeTreeletSerial, src/cuda/lbvh_plus_builder.cu:71-247. */
#define TL_MAX 7
void orc_treelet(orc_node* nodes, uint32_t* parent, int root) {
  int act[TL_MAX];
  orc_aabb abox[TL_MAX];
  int cnt = 1;
  act[0] = root;
  abox[0] = nodes[root].box;
  /* grow: expand the internal treelet leaf of largest area, first index on ties (:82-114) */
  for (int step = 0; step < TL_MAX - 1; ++step) {
    int best = -1;
    float max_area = -1.0f;
    for (int i = 0; i < cnt; ++i) {
      if (!is_leaf(&nodes[act[i]])) {
        float a = orc_sa(&abox[i]);
        if (a > max_area) { max_area = a; best = i; }
      }
    }
    if (best == -1) break;
    int x = act[best];
    int l = nodes[x].left, r = nodes[x].right;
    act[best] = l;
    abox[best] = nodes[l].box;
    act[cnt] = r;
    abox[cnt] = nodes[r].box;
    cnt++;
  }
  const int n = cnt;
  if (n < 2) return;
  /* subset DP (:119-165) */
  float cost[1 << TL_MAX];
  uint8_t part[1 << TL_MAX];
  const int full = (1 << n) - 1;
  for (int s = 1; s <= full; ++s) cost[s] = __builtin_popcount((unsigned)s) == 1 ? 0.0f : 1e30f;
  for (int k = 2; k <= n; ++k) {
    for (int s = 1; s <= full; ++s) {
      if (__builtin_popcount((unsigned)s) != k) continue;
      orc_aabb b;
      box_empty(&b);
      for (int i = 0; i < n; ++i)
        if ((s >> i) & 1) b = box_merge(&b, &abox[i]);
      float area = orc_sa(&b);
      float min_cost = 1e30f;
      int best_p = -1;
      int delta = (s - 1) & s;
      int p = (-delta) & s;
      do {
        float c = cost[p] + cost[s ^ p];
        if (c < min_cost) { min_cost = c; best_p = p; }
        p = (p - delta) & s;
      } while (p != 0);
      cost[s] = min_cost + area; /* Ci = 1.0f, exact either contracted or not */
      part[s] = (uint8_t)best_p;
    }
  }
  /* internal node ids available for reuse, DFS popping the right child first (:167-191) */
  int avail[TL_MAX];
  int n_avail = 0;
  int stack[TL_MAX + 8];
  int top = 0;
  stack[top++] = root;
  while (top > 0) {
    int cur = stack[--top];
    int in_leaves = 0;
    for (int i = 0; i < n; ++i)
      if (act[i] == cur) { in_leaves = 1; break; }
    if (!in_leaves) {
      avail[n_avail++] = cur;
      stack[top++] = nodes[cur].left;
      stack[top++] = nodes[cur].right;
    }
  }
  /* breadth-first rebuild from the partition table (:194-246) */
  int qm[TL_MAX], qn[TL_MAX];
  int qh = 0, qt = 0, used = 1;
  qm[qt] = full;
  qn[qt++] = avail[0];
  while (qh < qt) {
    int mask = qm[qh], cur = qn[qh];
    qh++;
    int lm = part[mask], rm = mask ^ lm;
    int li, ri;
    if (__builtin_popcount((unsigned)lm) == 1) li = act[__builtin_ctz((unsigned)lm)];
    else { li = avail[used++]; qm[qt] = lm; qn[qt++] = li; }
    if (__builtin_popcount((unsigned)rm) == 1) ri = act[__builtin_ctz((unsigned)rm)];
    else { ri = avail[used++]; qm[qt] = rm; qn[qt++] = ri; }
    nodes[cur].left = li;
    nodes[cur].right = ri;
    orc_aabb b;
    box_empty(&b);
    for (int i = 0; i < n; ++i)
      if ((mask >> i) & 1) b = box_merge(&b, &abox[i]);
    nodes[cur].box = b;
    if (parent) { parent[li] = (uint32_t)cur; parent[ri] = (uint32_t)cur; }
  }
}

/* LBVHPlusBuilderCUDA::runCompute, src/cuda/lbvh_plus_builder.cu:441-508: bounds, Morton,
 * stable sort, Karras, leaves, refit, then refit+optimise passes (kRefitAndOptimize, :341-366).
 * A bottom-up pass visits each internal node after both children; any such order gives the
 * same tree because a treelet at X only touches X's subtree, so post-order is used here. */
int orc_lbvh_plus(const orc_mesh* m, int bits, int rounds, orc_node* nodes, uint32_t* indices) {
  const uint32_t n = m->n;
  int rc = orc_lbvh(m, bits, nodes, indices, NULL);
  if (rc != ORC_OK || n < 2) return rc;
  uint32_t nn = 2 * n - 1;
  uint32_t* parent = (uint32_t*)malloc((size_t)nn * sizeof(uint32_t));
  uint32_t* order = (uint32_t*)malloc((size_t)nn * sizeof(uint32_t));
  for (int r = 0; r < rounds; ++r) {
    uint32_t cnt = post_order(nodes, nn, order);
    for (uint32_t k = 0; k < cnt; ++k) {
      orc_node* nd = &nodes[order[k]];
      nd->box = box_merge(&nodes[nd->left].box, &nodes[nd->right].box);
      orc_treelet(nodes, parent, (int)order[k]);
    }
  }
  free(parent);
  free(order);
  return ORC_OK;
}

/* PLOCBuilderCUDA::build, src/cuda/ploc_builder.cu:403-586. */
int orc_ploc(const orc_mesh* m, int radius, int max_iter, orc_node* nodes, uint32_t* indices,
             uint32_t* n_nodes, int* iterations, uint64_t* cluster_sum) {
  const uint32_t n = m->n;
  *n_nodes = 0;
  if (iterations) *iterations = 0;
  if (cluster_sum) *cluster_sum = 0;
  if (n == 0) return ORC_OK;
  if (radius < 1) return ORC_ERR_INVALID;
  orc_aabb* boxes = (orc_aabb*)malloc((size_t)n * sizeof(orc_aabb));
  float* c4 = (float*)malloc((size_t)n * 4 * sizeof(float));
  uint64_t* keys = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
  orc_tri_bounds(m, boxes, c4);
  orc_aabb scene;
  orc_scene_bounds(boxes, n, &scene);
  orc_morton(c4, n, 30, &scene, keys); /* morton3D_ploc (:19-29) equals morton3D_nt */
  orc_sort_pairs(keys, indices, n, 30, 1);
  orc_aabb* cb = (orc_aabb*)malloc((size_t)n * sizeof(orc_aabb));
  orc_aabb* cb2 = (orc_aabb*)malloc((size_t)n * sizeof(orc_aabb));
  int32_t* cid = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  int32_t* cid2 = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  int32_t* nb = (int32_t*)malloc((size_t)n * sizeof(int32_t));
  uint8_t* valid = (uint8_t*)malloc((size_t)n);
  /* kGatherAABBs / kInitLeafNodes_ploc / kInitializeSequence (:143-171) */
  for (uint32_t i = 0; i < n; ++i) {
    cb[i] = boxes[indices[i]];
    nodes[i].box = cb[i];
    nodes[i].left = (int32_t)(indices[i] | ORC_LEAF_BIT);
    nodes[i].right = -1;
    nodes[i].pad[0] = nodes[i].pad[1] = 0;
    cid[i] = (int32_t)i;
  }
  uint32_t next = n, c = n;
  int it = 0, rc = ORC_OK;
  uint64_t csum = 0;
  while (c > 1) {
    if (max_iter > 0 && it >= max_iter) { rc = ORC_ERR_NO_PROGRESS; break; }
    csum += c;
    /* kFindNearestNeighbors_ploc (:173-209) */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)c; ++i) {
      float best = FLT_MAX;
      int64_t bj = -1;
      int64_t s = i - radius < 0 ? 0 : i - radius;
      int64_t e = i + radius > (int64_t)c - 1 ? (int64_t)c - 1 : i + radius;
      for (int64_t j = s; j <= e; ++j) {
        if (j == i) continue;
        orc_aabb u = box_merge(&cb[i], &cb[j]);
        float d = orc_sa(&u);
        if (d < best) { best = d; bj = j; }
        else if (d == best) { if (bj == -1 || j < bj) bj = j; }
      }
      nb[i] = (int32_t)bj;
    }
    /* kMergeClusters_ploc (:211-264), new node ids handed out in ascending i */
    for (uint32_t i = 0; i < c; ++i) {
      int32_t j = nb[i];
      if (j != -1 && nb[j] == (int32_t)i && (int32_t)i < j) {
        orc_aabb u = box_merge(&cb[i], &cb[j]);
        uint32_t id = next++;
        nodes[id].box = u;
        nodes[id].left = cid[i];
        nodes[id].right = cid[j];
        nodes[id].pad[0] = nodes[id].pad[1] = 0;
        cid[i] = (int32_t)id;
        cb[i] = u;
        valid[i] = 1;
      } else if (j != -1 && nb[j] == (int32_t)i && j < (int32_t)i) {
        valid[i] = 0;
      } else {
        valid[i] = 1;
      }
    }
    /* ExclusiveSum + kCompactIndices/kCompactAABBs (:267-293, 524-540) */
    uint32_t nc = 0;
    for (uint32_t i = 0; i < c; ++i)
      if (valid[i]) { cb2[nc] = cb[i]; cid2[nc] = cid[i]; nc++; }
    { orc_aabb* t = cb; cb = cb2; cb2 = t; }
    { int32_t* t = cid; cid = cid2; cid2 = t; }
    it++;
    if (nc == c) { rc = ORC_ERR_NO_PROGRESS; break; }
    c = nc;
  }
  if (rc == ORC_OK) {
    /* root (last allocated) moved to index 0 (:563-582) */
    uint32_t total = next;
    if (total > 1) {
      uint32_t root = total - 1;
      orc_node t = nodes[0]; nodes[0] = nodes[root]; nodes[root] = t;
      for (uint32_t k = 0; k < total; ++k) {
        orc_node* nd = &nodes[k];
        if (nd->left < 0) continue; /* BVHNode::isLeaf */
        if (nd->left == 0) nd->left = (int32_t)root; else if (nd->left == (int32_t)root) nd->left = 0;
        if (nd->right >= 0) {
          if (nd->right == 0) nd->right = (int32_t)root; else if (nd->right == (int32_t)root) nd->right = 0;
        }
      }
    }
    *n_nodes = total;
  }
  if (iterations) *iterations = it;
  if (cluster_sum) *cluster_sum = csum;
  free(boxes); free(c4); free(keys); free(cb); free(cb2); free(cid); free(cid2); free(nb); free(valid);
  return rc;
}

/* ---- traversal ----
 * Every operation rounds as nvcc evaluates the reference's expressions under its default
 * -fmad=true (pinned against the reference's own traverseBVH and generateRay on the GPU):
 *   a*b - c*d              -> fmaf(a, b, -(c*d))
 *   (a*x + b*y) + c*z      -> fmaf(c, z, fmaf(a, x, b*y))
 *   x + a*b                -> fmaf(a, b, x)
 * This file is compiled with -ffp-contract=off, so nothing else is fused. */
#define TR_EPS 1e-6f
#define TR_STACK 128

static inline float tr_dot(float a, float b, float c, float x, float y, float z) {
  return fmaf(c, z, fmaf(a, x, b * y));
}
static inline float tr_cross(float a, float b, float c, float d) { return fmaf(a, b, -(c * d)); }

/* intersectAABB, src/render_engine.cu:194-214 (nothing to contract). */
static inline int hit_box(const float o[3], const float inv[3], const orc_aabb* b, float tmax) {
  float t0[3], t1[3];
  for (int k = 0; k < 3; ++k) {
    float a = (b->mn[k] - o[k]) * inv[k];
    float c = (b->mx[k] - o[k]) * inv[k];
    t0[k] = orc_fmin(a, c);
    t1[k] = orc_fmax(a, c);
  }
  float tenter = orc_fmax(orc_fmax(t0[0], t0[1]), t0[2]);
  float texit = orc_fmin(orc_fmin(t1[0], t1[1]), t1[2]);
  return texit >= orc_fmax(tenter, 0.0f) && tenter < tmax;
}

/* intersectTriangle (Moller-Trumbore), src/render_engine.cu:220-273. */
static inline int hit_tri(const float o[3], const float d[3], const orc_mesh* m, uint32_t p, float* out_t) {
  float v0x = m->v[0][p], v0y = m->v[1][p], v0z = m->v[2][p];
  float e1x = m->v[3][p] - v0x, e1y = m->v[4][p] - v0y, e1z = m->v[5][p] - v0z;
  float e2x = m->v[6][p] - v0x, e2y = m->v[7][p] - v0y, e2z = m->v[8][p] - v0z;
  float px = tr_cross(d[1], e2z, d[2], e2y);
  float py = tr_cross(d[2], e2x, d[0], e2z);
  float pz = tr_cross(d[0], e2y, d[1], e2x);
  float det = tr_dot(e1x, e1y, e1z, px, py, pz);
  if (fabsf(det) < TR_EPS) return 0;
  float inv_det = 1.0f / det;
  float tx = o[0] - v0x, ty = o[1] - v0y, tz = o[2] - v0z;
  float u = tr_dot(tx, ty, tz, px, py, pz) * inv_det;
  if (u < -1e-5f || u > 1.00001f) return 0;
  float qx = tr_cross(ty, e1z, tz, e1y);
  float qy = tr_cross(tz, e1x, tx, e1z);
  float qz = tr_cross(tx, e1y, ty, e1x);
  float v = tr_dot(d[0], d[1], d[2], qx, qy, qz) * inv_det;
  if (v < -1e-5f || u + v > 1.00001f) return 0;
  float t = tr_dot(e2x, e2y, e2z, qx, qy, qz) * inv_det;
  if (t < TR_EPS) return 0;
  *out_t = t;
  return 1;
}

/* traverseBVH, src/render_engine.cu:289-356 (ray set-up as generateRay, :177-185). */
void orc_trace(const orc_node* nodes, uint32_t n_nodes, const orc_mesh* m, const float* ro, const float* rd,
               uint32_t nr, float* t_out, int32_t* prim_out, int32_t* vis_out, int32_t* aabb_out, int32_t* tri_out) {
  const int nn = (int)n_nodes;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t r = 0; r < (int64_t)nr; ++r) {
    float o[3] = {ro[3 * r], ro[3 * r + 1], ro[3 * r + 2]};
    float d[3] = {rd[3 * r], rd[3 * r + 1], rd[3 * r + 2]};
    float inv[3];
    for (int k = 0; k < 3; ++k) inv[k] = fabsf(d[k]) > TR_EPS ? 1.0f / d[k] : (d[k] >= 0 ? 1e30f : -1e30f);
    float best = 1e30f;
    int32_t prim = -1, vis = 0, at = 0, tt = 0;
    int stack[TR_STACK];
    int sp = 0;
    if (nn > 0) stack[sp++] = 0;
    while (sp > 0) {
      int x = stack[--sp];
      if (x < 0 || x >= nn) continue;
      const orc_node* nd = &nodes[x];
      vis++;
      at++;
      if (!hit_box(o, inv, &nd->box, best)) continue;
      if (nd->left < 0) { /* BVHNode::isLeaf */
        uint32_t p = (uint32_t)nd->left & 0x7FFFFFFFu;
        tt++;
        float t;
        if (p < m->n && hit_tri(o, d, m, p, &t)) {
          if (t < best) { best = t; prim = (int32_t)p; }
        }
      } else {
        if (nd->right >= 0 && nd->right < nn && sp < TR_STACK) stack[sp++] = nd->right;
        if (nd->left >= 0 && nd->left < nn && sp < TR_STACK) stack[sp++] = nd->left;
      }
    }
    t_out[r] = best;
    prim_out[r] = prim;
    vis_out[r] = vis;
    aabb_out[r] = at;
    tri_out[r] = tt;
  }
}

/* d_normalize, src/render_engine.cu:130-135. */
static void normalize3(float v[3]) {
  float len = sqrtf(tr_dot(v[0], v[1], v[2], v[0], v[1], v[2]));
  if (len < 1e-12f) { v[0] = v[1] = v[2] = 0.0f; return; }
  float inv = 1.0f / len;
  v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}
/* generateRay, src/render_engine.cu:155-188.  tan(fov/2) is the host's tanf, which may differ
 * from the device's tanf in the last place; tests that need the GPU's exact rays take them from
 * bvh_pinhole_rays, which is pinned bit for bit against the reference's generateRay. */
void orc_pinhole_rays(const float eye[3], const float look[3], const float up[3], float fovy, int w, int h,
                      float* ro, float* rd) {
  float f[3] = {look[0] - eye[0], look[1] - eye[1], look[2] - eye[2]};
  normalize3(f);
  float r[3] = {tr_cross(f[1], up[2], f[2], up[1]), tr_cross(f[2], up[0], f[0], up[2]),
                tr_cross(f[0], up[1], f[1], up[0])};
  normalize3(r);
  float u[3] = {tr_cross(r[1], f[2], r[2], f[1]), tr_cross(r[2], f[0], r[0], f[2]), tr_cross(r[0], f[1], r[1], f[0])};
  float half_h = tanf(fovy * 3.14159265358979f / 180.0f * 0.5f);
  float half_w = half_h * ((float)w / (float)h);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < (int64_t)w * h; ++p) {
    int x = (int)(p % w), y = (int)(p / w);
    float uu = (2.0f * ((float)x + 0.5f) / (float)w - 1.0f) * half_w;
    float vv = (2.0f * ((float)y + 0.5f) / (float)h - 1.0f) * half_h;
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = fmaf(-vv, u[k], fmaf(uu, r[k], f[k]));
    normalize3(d);
    for (int k = 0; k < 3; ++k) { ro[3 * p + k] = eye[k]; rd[3 * p + k] = d[k]; }
  }
}

/* kRenderKernel's shading of traced pixels, src/render_engine.cu:395-446: rd = each pixel's
 * ray direction, t / prim from the traversal; a miss gets the background (:33-36). */
void orc_shade(const orc_mesh* m, const float* rd, const float* t, const int32_t* prim, const int32_t* vis,
               uint32_t np, int mode, float diag, const float light[3], float* rgb) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)np; ++i) {
    float c[3];
    const int32_t p = prim[i];
    if (p < 0 || (uint32_t)p >= m->n) {
      c[0] = 0.15f; c[1] = 0.15f; c[2] = 0.18f;
    } else if (mode == 3) {
      c[0] = c[1] = c[2] = (float)vis[i];
    } else if (mode == 1) {
      float depth = orc_fmax(0.0f, orc_fmin(1.0f, t[i] / diag));
      c[0] = c[1] = c[2] = 1.0f - depth;
    } else if (mode == 0 || mode == 2) {
      /* geometric normal: normalise(e1 x e2), intersectTriangle :267-271 */
      float v0x = m->v[0][p], v0y = m->v[1][p], v0z = m->v[2][p];
      float e1x = m->v[3][p] - v0x, e1y = m->v[4][p] - v0y, e1z = m->v[5][p] - v0z;
      float e2x = m->v[6][p] - v0x, e2y = m->v[7][p] - v0y, e2z = m->v[8][p] - v0z;
      float n[3] = {tr_cross(e1y, e2z, e1z, e2y), tr_cross(e1z, e2x, e1x, e2z), tr_cross(e1x, e2y, e1y, e2x)};
      normalize3(n);
      if (mode == 0) {
        for (int k = 0; k < 3; ++k) c[k] = (n[k] + 1.0f) * 0.5f;
      } else {
        const float* d = rd + 3 * i;
        if (tr_dot(n[0], n[1], n[2], d[0], d[1], d[2]) > 0.0f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
        float diffuse = orc_fmax(0.0f, tr_dot(n[0], n[1], n[2], light[0], light[1], light[2]));
        float shade = orc_fmin(1.0f, fmaf(diffuse, 0.85f, 0.15f));
        for (int k = 0; k < 3; ++k) c[k] = shade * fmaf(0.3f, fabsf(n[k]), 0.7f);
      }
    } else {
      c[0] = 1.0f; c[1] = 0.0f; c[2] = 1.0f;
    }
    for (int k = 0; k < 3; ++k) rgb[3 * i + k] = c[k];
  }
}

static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* applyHeatmapColormap with getTurboColor, src/render_engine.cu:519-595, for a 256 x 3 colormap;
 * returns the normalisation used. */
float orc_heatmap(const int32_t* vis, uint32_t np, const float* lut, float fixed_max, float* rgb) {
  float mx = fixed_max;
  if (mx <= 0.0f) {
    size_t k = 0;
    int32_t* h = (int32_t*)malloc(sizeof(int32_t) * (np ? np : 1));
    for (uint32_t i = 0; i < np; ++i)
      if (vis[i] > 0) h[k++] = vis[i];
    mx = 128.0f;
    if (k) {
      qsort(h, k, sizeof(int32_t), cmp_i32);
      size_t q = (size_t)((double)k * 0.999);
      size_t idx = q < k - 1 ? q : k - 1;
      mx = orc_fmax(1.0f, (float)h[idx]);
    }
    free(h);
  }
  for (uint32_t i = 0; i < np; ++i) {
    if (vis[i] == 0) {
      rgb[3 * i] = 0.15f; rgb[3 * i + 1] = 0.15f; rgb[3 * i + 2] = 0.18f;
      continue;
    }
    float t = (float)vis[i] / mx;
    t = orc_fmax(0.0f, orc_fmin(1.0f, t));
    t = orc_fmax(0.0f, orc_fmin(1.0f, t));
    float scaled = t * 255.0f;
    int i0 = (int)scaled;
    int i1 = i0 + 1 < 255 ? i0 + 1 : 255;
    float frac = scaled - (float)i0;
    for (int c = 0; c < 3; ++c) rgb[3 * i + c] = lut[3 * i0 + c] * (1.0f - frac) + lut[3 * i1 + c] * frac;
  }
  return mx;
}

/* savePPM's conversion, src/render_engine.cu:502-507. */
void orc_rgb8(const float* rgb, uint32_t nv, uint8_t* out) {
  for (uint32_t i = 0; i < nv; ++i) {
    float v = orc_fmax(0.0f, orc_fmin(1.0f, rgb[i]));
    out[i] = (uint8_t)(v * 255.0f + 0.5f);
  }
}

/* BVHEvaluator::computeSAHRecursive, src/evaluator.cpp:54-88: DFS, float accumulation. */
static float sah_rec(const orc_node* nodes, int nn, int x, float root_area) {
  if (x < 0 || x >= nn) return 0.0f;
  const orc_node* nd = &nodes[x];
  float prob = sa_plain(&nd->box) / root_area;
  if (nd->left < 0) return prob * 2.0f * 1.0f;
  float cost = prob * 3.0f;
  if (nd->left >= 0 && nd->left < nn) cost += sah_rec(nodes, nn, nd->left, root_area);
  if (nd->right >= 0 && nd->right < nn) cost += sah_rec(nodes, nn, nd->right, root_area);
  return cost;
}
/* BVHEvaluator::computeSAH, src/evaluator.cpp:38-52. */
float orc_sah(const orc_node* nodes, uint32_t n_nodes) {
  if (n_nodes == 0) return 0.0f;
  float root_area = sa_plain(&nodes[0].box);
  if (root_area <= 0.0f) return 0.0f;
  return sah_rec(nodes, (int)n_nodes, 0, root_area);
}

/* BVHEvaluator::computeDepthStats, src/evaluator.cpp:90-113, and the float average of
 * evaluate() (:24-33), iteratively in the same visiting order. */
void orc_depth_stats(const orc_node* nodes, uint32_t n_nodes, int* max_depth, float* avg, uint32_t* leaf_count) {
  *max_depth = 0; *avg = 0.0f; *leaf_count = 0;
  if (n_nodes == 0) return;
  int64_t cap = (int64_t)n_nodes + 64;
  int* sx = (int*)malloc((size_t)cap * sizeof(int));
  int* sd = (int*)malloc((size_t)cap * sizeof(int));
  int64_t sp = 0;
  sx[sp] = 0; sd[sp] = 0; sp++;
  float sum = 0.0f;
  uint32_t leaves = 0;
  int md = 0;
  const int nn = (int)n_nodes;
  while (sp > 0) {
    --sp;
    int x = sx[sp], d = sd[sp];
    if (x < 0 || x >= nn) continue;
    if (d > md) md = d;
    const orc_node* nd = &nodes[x];
    if (nd->left < 0) { sum += (float)d; leaves++; continue; }
    if (sp + 2 > cap) break;
    /* push right first so that the left subtree is visited first, as the recursion does */
    if (nd->right >= 0 && nd->right < nn) { sx[sp] = nd->right; sd[sp] = d + 1; sp++; }
    if (nd->left >= 0 && nd->left < nn) { sx[sp] = nd->left; sd[sp] = d + 1; sp++; }
  }
  free(sx); free(sd);
  *max_depth = md;
  *leaf_count = leaves;
  *avg = leaves ? sum / (float)leaves : 0.0f;
}

static int canon_eq(const orc_node* a, int na, int xa, const orc_node* b, int nb, int xb) {
  /* explicit stack of pairs */
  int64_t cap = (int64_t)(na < nb ? na : nb) + 64;
  int* sa = (int*)malloc((size_t)cap * sizeof(int));
  int* sb = (int*)malloc((size_t)cap * sizeof(int));
  int64_t sp = 0;
  int ok = 1;
  sa[sp] = xa; sb[sp] = xb; sp++;
  while (sp > 0 && ok) {
    --sp;
    int x = sa[sp], y = sb[sp];
    if (x < 0 || x >= na || y < 0 || y >= nb) { ok = 0; break; }
    const orc_node* p = &a[x];
    const orc_node* q = &b[y];
    if (memcmp(&p->box.mn, &q->box.mn, 12) || memcmp(&p->box.mx, &q->box.mx, 12)) { ok = 0; break; }
    int lp = p->left < 0, lq = q->left < 0;
    if (lp != lq) { ok = 0; break; }
    if (lp) { if (p->left != q->left) ok = 0; continue; }
    if (sp + 2 > cap) { ok = 0; break; }
    sa[sp] = p->left; sb[sp] = q->left; sp++;
    sa[sp] = p->right; sb[sp] = q->right; sp++;
  }
  free(sa); free(sb);
  return ok;
}
int orc_tree_equal_canonical(const orc_node* a, uint32_t na, const orc_node* b, uint32_t nb) {
  if (na != nb) return 1;
  if (na == 0) return 0;
  return canon_eq(a, (int)na, 0, b, (int)nb, 0) ? 0 : 1;
}
