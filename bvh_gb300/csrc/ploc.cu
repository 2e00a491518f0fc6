// ploc.cu -- PLOC (parallel locally-ordered clustering) on sm_103a.
//
// Reference: PLOCBuilderCUDA::build, src/cuda/ploc_builder.cu:403-586.  Same Morton-30 order,
// same leaves (node i = sorted triangle i), same nearest-neighbour rule (smallest union area in
// the window [i-r, i+r], first j on ties, :173-209), same mutual-pair merge (:211-264) and
// order-preserving compaction (:267-293), same root move to index 0 (:563-582).
//
// Differences by design: new node ids are handed out in ascending cluster order through a
// scan (the reference uses atomicAdd, so its ids vary run to run); merge and compaction share
// one reduce-then-scan over 2048-cluster tiles; and the iteration loop runs on the device as a CUDA
// graph WHILE node (the reference synchronises with the host five times per iteration,
// :489-548): a one-thread step kernel swaps the cluster buffers, stops on convergence, on an
// iteration that merges nothing (NaN/Inf areas, where the reference loops forever) or at the
// iteration cap, and sets the loop condition.
#include <algorithm>

#include "lbvh.cuh"

namespace bvhgb {

constexpr int kPlocThreads = 256;
constexpr int kPlocIpt = 8;
constexpr int kPlocTile = kPlocThreads * kPlocIpt;

// control words (scratch + L.ploc):
//   [0] live clusters  [1] next node id  [2] count ticket  [3] buffer parity
//   [4] survivors (next iteration)  [5] next node id (next iteration)  [6] iterations  [7] cap
//   [8..9] sum of live clusters over iterations (64-bit)  [10] go on (host-driven loop)
//   [11] meshes (1 for a single build): the loop ends at one cluster per mesh
//   [12] hand-over size: the loop stops at this many live clusters and k_ploc_tail finishes
//        (0: no hand-over)
//   [13] single builds: the node that took node 0 (sorted triangle 0's leaf) as its left child,
//        for the root fix (cluster 0 stays at position 0 until it merges, always as the left)
//   [14] single builds: the loop also stops at this many live clusters and k_ploc_grid goes on
//        (0: no hand-over)  [15] k_ploc_grid's barrier counter
//   [16] iterations run by k_ploc_grid  [17] iterations run by k_ploc_tail
//   [18] k_ploc_grid was launched  [19] k_ploc_tail was launched (launch accounting)
struct PlocBufs {
  Box* cbox[2];
  int32_t* cid[2];
  int32_t* nbr;
  uint2* flags;  // per (tile, warp, round): the merge and survivor ballots of 32 clusters
  unsigned long long* desc;
  Node* nodes;
  uint32_t* ctrl;
  uint32_t* status;
};

// Batched builds: per-mesh loop state.  seg[par * count + m] = position of mesh m's first live
// cluster (a mesh's first cluster always survives: it is never the larger index of a pair);
// id_base[m] = the mesh-local id of this iteration's first new node minus the global merge
// rank of the mesh's first cluster, so a merge's local id is id_base[m] + its global rank.
struct PlocSeg {
  const uint32_t* offsets;  // count + 1 triangle offsets
  uint32_t* seg;            // 2 * count (ping-pong with the cluster buffers' parity)
  uint32_t* id_base;        // count
  uint32_t count;
};

__global__ void k_ploc_init(const uint32_t* __restrict__ sidx, const Box* __restrict__ tri_boxes, PlocBufs B, uint32_t n,
                            uint32_t cap, uint32_t tail, uint32_t grid_at) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    B.ctrl[0] = n;
    B.ctrl[1] = n;
    B.ctrl[2] = 0;
    B.ctrl[3] = 0;
    B.ctrl[6] = 0;
    B.ctrl[7] = cap;
    B.ctrl[8] = 0;
    B.ctrl[9] = 0;
    B.ctrl[11] = 1;
    B.ctrl[12] = tail;
    B.ctrl[13] = 0xffffffffu;
    B.ctrl[14] = grid_at;
#pragma unroll
    for (int k = 15; k < 20; ++k) B.ctrl[k] = 0;
  }
  if (i >= n) return;
  uint32_t prim = __ldg(sidx + i);
  const float4* bp = reinterpret_cast<const float4*>(tri_boxes + prim);
  float4 lo = __ldg(bp), hi = __ldg(bp + 1);
  reinterpret_cast<float4*>(B.cbox[0] + i)[0] = lo;
  reinterpret_cast<float4*>(B.cbox[0] + i)[1] = hi;
  B.cid[0][i] = (int32_t)i;
  float4* np = reinterpret_cast<float4*>(B.nodes + i);
  np[0] = lo;
  np[1] = hi;
  reinterpret_cast<int4*>(np + 2)[0] = make_int4((int32_t)(prim | kLeafBit), -1, 0, 0);
}

// Nearest neighbour in the +-r window (:173-209): the smallest union area, the smallest j on
// ties; areas that are NaN or infinite never win.  The area of a pair is symmetric (fminf/fmaxf
// commute), so each pair is evaluated once, by the thread of its earlier cluster x: it keeps x's
// forward best in registers and writes the area into a per-offset table D[k][j] for the later
// cluster j = x + k, which after a barrier reads its backward candidates from its column (the
// later offset, i.e. the smaller index, wins ties).  Offsets go in chunks of kNnKc to bound the
// table.  The r clusters before a tile ("halo") only fill the table; their pairs are spread over
// all warps.  Tiles of kNnTile clusters (kNnPer per thread, strided so lanes are consecutive),
// the window staged in shared memory.
constexpr int kNnPer = 4;
constexpr int kNnTile = kPlocThreads * kNnPer;
constexpr int kNnKc = 5;

__device__ __forceinline__ float pair_area(float4 xa, float4 xb, float4 ja, float4 jb) {
  return sa_xyz(__fsub_rn(fmaxf(xb.x, jb.x), fminf(xa.x, ja.x)), __fsub_rn(fmaxf(xb.y, jb.y), fminf(xa.y, ja.y)),
                __fsub_rn(fmaxf(xb.z, jb.z), fminf(xa.z, ja.z)));
}

// Batched builds keep each cluster's mesh in the w lane of its lo corner: a pair from two meshes
// has no area (+inf never wins), which clips every window at its mesh's boundary exactly as a
// single build's window ends at the ends of its cluster array.
template <bool SEG>
__device__ __forceinline__ float pair_d(float4 xa, float4 xb, float4 ja, float4 jb) {
  if (SEG && __float_as_int(xa.w) != __float_as_int(ja.w)) return __int_as_float(0x7f800000);
  return pair_area(xa, xb, ja, jb);
}

template <int PER, bool SEG>
__device__ __forceinline__ void nn_tiles(const PlocBufs& B, int r, uint32_t c, const Box* __restrict__ cbox,
                                         float4* sw) {
  constexpr int TILE = kPlocThreads * PER;
  // (TILE + 2r) boxes: all lo corners, then all hi corners (lanes read consecutive 16 bytes)
  float* sD = reinterpret_cast<float*>(sw + 2 * (TILE + 2 * r));  // [kNnKc][TILE]
  const int span = TILE + 2 * r;
  float4* s_lo = sw;
  float4* s_hi = sw + span;
  const int t = threadIdx.x;
  const float kInf = __int_as_float(0x7f800000);
  for (uint32_t base = blockIdx.x * (uint32_t)TILE; base < c; base += gridDim.x * (uint32_t)TILE) {
    const int lo = (int)base - r;  // window position 0; may be negative
    const int tile_n = (int)min((uint32_t)TILE, c - base);
    __syncthreads();  // previous tile's window no longer read
    for (int k = t; k < span; k += kPlocThreads) {
      const int j = lo + k;
      if (j >= 0 && j < (int)c) {
        const float4* bp = reinterpret_cast<const float4*>(cbox + j);
        s_lo[k] = __ldcg(bp);
        s_hi[k] = __ldcg(bp + 1);
      }
    }
    __syncthreads();
    float fd[PER], ed[PER];  // forward / backward best areas (+inf: none yet)
    int fj[PER], ej[PER];
    float4 xa[PER], xb[PER];
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      fd[m] = ed[m] = kInf;
      fj[m] = ej[m] = -1;
      const int xi = t + m * kPlocThreads;
      xa[m] = s_lo[min(xi + r, span - 1)];
      xb[m] = s_hi[min(xi + r, span - 1)];
    }
    // interior tile: every cluster has all r neighbours on both sides, so full offset chunks
    // take a path without bounds checks (fully unrolled)
    const bool interior = (int)base >= r && base + (uint32_t)TILE + (uint32_t)r <= c;
    for (int k0 = 1; k0 <= r; k0 += kNnKc) {
      const int kc = min(kNnKc, r - k0 + 1);
      const bool full = interior && kc == kNnKc;
      // pairs (x, x + k), k in [k0, k0 + kc): forward candidates of x, table entries for x + k
      if (full) {
#pragma unroll
        for (int m = 0; m < PER; ++m) {
          const int xi = t + m * kPlocThreads;
#pragma unroll
          for (int kk = 0; kk < kNnKc; ++kk) {
            const int jw = xi + r + k0 + kk;
            const float d = pair_d<SEG>(xa[m], xb[m], s_lo[jw], s_hi[jw]);
            if (d < fd[m]) {
              fd[m] = d;
              fj[m] = (int)base + xi + k0 + kk;
            }
            if (xi + k0 + kk < TILE) sD[kk * TILE + xi + k0 + kk] = d;
          }
        }
      } else {
#pragma unroll
        for (int m = 0; m < PER; ++m) {
          const int xi = t + m * kPlocThreads;
          if (xi < tile_n) {
            const int kmax = min(kc, (int)c - 1 - ((int)base + xi) - k0 + 1);  // j = base + xi + k < c
            for (int kk = 0; kk < kmax; ++kk) {
              const int jw = xi + r + k0 + kk;
              const float d = pair_d<SEG>(xa[m], xb[m], s_lo[jw], s_hi[jw]);
              if (d < fd[m]) {  // increasing j: the first of equal areas stays
                fd[m] = d;
                fj[m] = (int)base + xi + k0 + kk;
              }
              if (xi + k0 + kk < tile_n) sD[kk * TILE + xi + k0 + kk] = d;
            }
          }
        }
      }
      // halo pairs (h, jj) with jj < k: the table entries of the tile's first clusters
      for (int kk = 0; kk < kc; ++kk) {
        const int k = k0 + kk;
        const int rot = (k * 37) & (kPlocThreads - 1);  // spread each offset's pairs over the block
        for (int p = (t - rot) & (kPlocThreads - 1); p < k && p < tile_n; p += kPlocThreads) {
          const int h = (int)base + p - k;  // the halo cluster; p is the tile-relative target
          if (h >= 0) {
            const int hw = p - k + r;
            sD[kk * TILE + p] = pair_d<SEG>(s_lo[hw], s_hi[hw], s_lo[p + r], s_hi[p + r]);
          }
        }
      }
      __syncthreads();
      // backward candidates j - k of this thread's clusters
      if (full) {
#pragma unroll
        for (int m = 0; m < PER; ++m) {
          const int xi = t + m * kPlocThreads;
#pragma unroll
          for (int kk = 0; kk < kNnKc; ++kk) {
            const float d = sD[kk * TILE + xi];
            if (d < kInf && d <= ed[m]) {
              ed[m] = d;
              ej[m] = (int)base + xi - k0 - kk;
            }
          }
        }
      } else {
#pragma unroll
        for (int m = 0; m < PER; ++m) {
          const int xi = t + m * kPlocThreads;
          if (xi < tile_n) {
            for (int kk = 0; kk < kc; ++kk) {
              const int src = (int)base + xi - k0 - kk;
              if (src < 0) break;
              const float d = sD[kk * TILE + xi];
              if (d < kInf && d <= ed[m]) {  // later offset = smaller index: wins ties
                ed[m] = d;
                ej[m] = src;
              }
            }
          }
        }
      }
      __syncthreads();  // the table is refilled by the next chunk
    }
#pragma unroll
    for (int m = 0; m < PER; ++m) {
      const int xi = t + m * kPlocThreads;
      if (xi < tile_n) B.nbr[base + xi] = (ej[m] >= 0 && ed[m] <= fd[m]) ? ej[m] : fj[m];  // earlier index wins ties
    }
  }
}

// The large iterations take a second form of the same search (ploc_builder.cu:173-209), which
// moves about half the shared-memory bytes: thread t owns kNcP consecutive clusters x0 .. x0 + 3, so each window box
// it loads serves all four (r + 3 loads for 4r pairs instead of 4r), and the backward candidates
// a thread produces for one later cluster are reduced to one (area, index) entry before they go
// through the shared-memory table.  Both searches pick the smallest (area, index) pair in each
// direction, so they give the same neighbours.  The first H = ceil(r / kNcP) threads of a tile hold
// the r clusters before it: they only feed backward candidates.  Window box w is stored at
// w ^ ((w >> 3) & 3), which puts the 16-byte boxes that 8 lanes read -- every fourth box, or 8
// consecutive ones -- in distinct bank groups.
constexpr int kNcP = 4;      // consecutive clusters per thread
constexpr int kNcQ = 4;      // thread distances per table round
constexpr int kNcMaxR = 128;  // larger radii keep the strided form (a halo of 32 threads at 128)
__host__ __device__ constexpr int nc_swz(int w) { return w ^ ((w >> 3) & 3); }
// boxes staged: the halo, the tile, r past it, + kNcP read past the last pair; rounded to 8
__host__ __device__ constexpr int nc_span(int r) { return (kPlocThreads * kNcP + r + kNcP + 7) & ~7; }
static size_t nc_smem(int r) {
  const int h = (r + kNcP - 1) / kNcP;
  return 2 * 16 * (size_t)nc_span(r) + 8 * (size_t)kNcQ * kNcP * (kPlocThreads + h);
}

template <bool SEG, bool CHECK>
__device__ __forceinline__ void nc_pairs(int r, int c, int x0, int o, const float4 (&a)[kNcP], const float4 (&b)[kNcP],
                                         float4 jl, float4 jh, float (&fd)[kNcP], int (&fj)[kNcP], float& pa,
                                         int& ps) {
#pragma unroll
  for (int m = 0; m < kNcP; ++m) {
    if (m < o && o - m <= r) {
      float d = pair_d<SEG>(a[m], b[m], jl, jh);
      if (CHECK && !(x0 + m >= 0 && x0 + o < c)) d = __int_as_float(0x7f800000);
      if (d < fd[m]) {  // increasing o: the first of equal areas stays
        fd[m] = d;
        fj[m] = x0 + o;
      }
      if (d < pa) {  // increasing m: the smaller index stays
        pa = d;
        ps = x0 + m;
      }
    }
  }
}

template <bool SEG, bool CHECK>
__device__ __forceinline__ void nc_tile(const PlocBufs& B, int r, int c, int lo, int h, const float4* s_lo,
                                        const float4* s_hi, float2* sT) {
  constexpr int P = kNcP, Q = kNcQ;
  const int t = threadIdx.x, tw = kPlocThreads + h;
  const int x0 = lo + P * t;
  const float kInf = __int_as_float(0x7f800000);
  float4 a[P], b[P];
  float fd[P], ed[P];
  int fj[P], ej[P];
#pragma unroll
  for (int m = 0; m < P; ++m) {
    a[m] = s_lo[nc_swz(P * t + m)];
    b[m] = s_hi[nc_swz(P * t + m)];
    fd[m] = ed[m] = kInf;
    fj[m] = ej[m] = -1;
  }
  // pairs among the thread's own clusters
#pragma unroll
  for (int o = 1; o < P; ++o) {
    float pa = kInf;
    int ps = -1;
    nc_pairs<SEG, CHECK>(r, c, x0, o, a, b, a[o], b[o], fd, fj, pa, ps);
    if (pa < ed[o] || (pa == ed[o] && ps < ej[o])) {
      ed[o] = pa;
      ej[o] = ps;
    }
  }
  // pairs with the clusters of the threads q = 1 .. h further on, Q distances per table round
  for (int q0 = 1; q0 <= h; q0 += Q) {
    const int qn = min(Q, h - q0 + 1);
    for (int s = 0; s < qn; ++s) {
      const int q = q0 + s;
#pragma unroll
      for (int mp = 0; mp < P; ++mp) {
        const int o = P * q + mp;
        const int w = nc_swz(P * t + o);
        float pa = kInf;
        int ps = -1;
        nc_pairs<SEG, CHECK>(r, c, x0, o, a, b, s_lo[w], s_hi[w], fd, fj, pa, ps);
        sT[(s * P + mp) * tw + t + q] = make_float2(pa, __int_as_float(ps));
      }
    }
    __syncthreads();
    for (int s = 0; s < qn; ++s) {
#pragma unroll
      for (int mp = 0; mp < P; ++mp) {
        const float2 e = sT[(s * P + mp) * tw + t];
        const int es = __float_as_int(e.y);
        if (e.x < ed[mp] || (e.x == ed[mp] && es < ej[mp])) {  // the smaller index wins ties
          ed[mp] = e.x;
          ej[mp] = es;
        }
      }
    }
    __syncthreads();  // the table is refilled by the next round
  }
  if (t >= h) {
#pragma unroll
    for (int m = 0; m < P; ++m) {
      const int x = x0 + m;
      if (x < c) B.nbr[x] = (ej[m] >= 0 && ed[m] <= fd[m]) ? ej[m] : fj[m];  // earlier index wins ties
    }
  }
}

template <bool SEG>
__device__ __forceinline__ void nn_tiles_consec(const PlocBufs& B, int r, uint32_t c, const Box* __restrict__ cbox,
                                                float4* sw) {
  const int h = (r + kNcP - 1) / kNcP;            // halo threads = the largest thread distance of a pair
  const int out = (kPlocThreads - h) * kNcP;      // clusters a tile decides
  const int span = kPlocThreads * kNcP + r;       // boxes staged: the halo, the tile, r past it
  float4* s_lo = sw;
  float4* s_hi = sw + nc_span(r);
  float2* sT = reinterpret_cast<float2*>(s_hi + nc_span(r));  // [kNcQ][kNcP][threads + h]
  const int t = threadIdx.x;
  for (uint32_t tb = blockIdx.x * (uint32_t)out; tb < c; tb += gridDim.x * (uint32_t)out) {
    const int lo = (int)tb - kNcP * h;  // window position 0; may be negative
    __syncthreads();                    // previous tile's window no longer read
    for (int k = t; k < span; k += kPlocThreads) {
      const int j = lo + k;
      if (j >= 0 && j < (int)c) {
        const float4* bp = reinterpret_cast<const float4*>(cbox + j);
        s_lo[nc_swz(k)] = __ldcg(bp);
        s_hi[nc_swz(k)] = __ldcg(bp + 1);
      }
    }
    __syncthreads();
    if (lo >= 0 && lo + span <= (int)c) nc_tile<SEG, false>(B, r, (int)c, lo, h, s_lo, s_hi, sT);
    else nc_tile<SEG, true>(B, r, (int)c, lo, h, s_lo, s_hi, sT);
  }
}

template <bool SEG>
__global__ void __launch_bounds__(kPlocThreads) k_ploc_nn(PlocBufs B, int r) {
  extern __shared__ float4 sw[];
  const uint32_t c = __ldcg(B.ctrl + 0);
  const Box* __restrict__ cbox = (__ldcg(B.ctrl + 3) & 1u) ? B.cbox[1] : B.cbox[0];  // no stack copy of B
  // Once the live clusters no longer fill the grid with 4-per-thread tiles, an iteration lasts
  // one tile's latency: smaller tiles (2 or 1 clusters per thread) then spread it over more
  // blocks.  The result does not depend on the tiling.
  const uint32_t g = gridDim.x * (uint32_t)kPlocThreads;
  if (c > 2u * g && r <= kNcMaxR) nn_tiles_consec<SEG>(B, r, c, cbox, sw);
  else if (c > 2u * g) nn_tiles<kNnPer, SEG>(B, r, c, cbox, sw);
  else if (c > g) nn_tiles<2, SEG>(B, r, c, cbox, sw);
  else nn_tiles<1, SEG>(B, r, c, cbox, sw);
}

// Merge mutual pairs (i < j keeps position i, :211-264) and compact the survivors (:267-293),
// as reduce-then-scan: k_ploc_count totals each tile of 256 R clusters (R <= 8 rounds per warp)
// and stores its ballots, its last block scans the tile totals, k_ploc_scatter reads the ballots
// and writes, k_ploc_step ends the iteration.  Warp w of a tile takes its items w*32R + r*32 +
// lane in R rounds r of 32 consecutive clusters, so positions within the warp come from ballots
// and new node ids follow the cluster order whatever R is.  Counts are packed as
// merges << 31 | survivors.
constexpr int kPlocRounds = kPlocTile / kPlocThreads;  // 8

// Item i merges here (as the smaller index of a mutual pair) / survives, from its neighbour j
// and j's neighbour `back` (-1 where not loaded).
__device__ __forceinline__ void item_flags(uint32_t c, uint32_t i, int32_t j, int32_t back, bool& m, bool& v) {
  const bool mutual = i < c && j >= 0 && (uint32_t)j < c && back == (int32_t)i;
  m = mutual && (int32_t)i < j;
  v = i < c && !(mutual && j < (int32_t)i);
}

// End of one iteration: publish the survivors, swap buffers, decide whether to go on (the
// graph's WHILE condition, or ctrl[10] for the host-driven loop).
template <bool GRAPH>
__device__ __forceinline__ void ploc_step(PlocBufs B, cudaGraphConditionalHandle handle) {
  const uint32_t c = B.ctrl[0], nc = B.ctrl[4], it = B.ctrl[6] + 1, cap = B.ctrl[7];
  unsigned long long sum = ((unsigned long long)B.ctrl[9] << 32 | B.ctrl[8]) + c;
  B.ctrl[8] = (uint32_t)sum;
  B.ctrl[9] = (uint32_t)(sum >> 32);
  B.ctrl[6] = it;
  B.ctrl[0] = nc;
  B.ctrl[1] = B.ctrl[5];
  B.ctrl[3] ^= 1u;
  bool go = nc > B.ctrl[11];
  if (go && (nc >= c || it >= cap)) {  // no mutual pair anywhere, or the cap: stop and report
    atomicOr(B.status, kStatusNoProgress);
    go = false;
  } else if (go && (nc <= B.ctrl[12] || nc <= B.ctrl[14])) {  // k_ploc_grid / k_ploc_tail go on
    go = false;
  }
  if constexpr (GRAPH) cudaGraphSetConditional(handle, go ? 1u : 0u);
  else B.ctrl[10] = go ? 1u : 0u;
}

// Exclusive prefix of the tile totals (in place), the survivors and the next node id; run by
// the last block of k_ploc_count.
__device__ __forceinline__ void ploc_scan_tiles(PlocBufs B, uint32_t tiles, unsigned long long* s_w) {
  const uint32_t per = div_up(tiles, (uint32_t)kPlocThreads);
  const uint32_t t0 = threadIdx.x * per, t1 = min(t0 + per, tiles);
  unsigned long long sum = 0;
  for (uint32_t t = t0; t < t1; ++t) sum += __ldcg(B.desc + t);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[w] = x;
  __syncthreads();
  unsigned long long run = x - sum, total = 0;
#pragma unroll
  for (int k = 0; k < kPlocThreads / 32; ++k) {
    if (k < w) run += s_w[k];
    total += s_w[k];
  }
  for (uint32_t t = t0; t < t1; ++t) {
    const unsigned long long v = __ldcg(B.desc + t);
    B.desc[t] = run;
    run += v;
  }
  if (threadIdx.x == 0) {
    B.ctrl[4] = (uint32_t)(total & 0x7fffffffull);             // survivors
    B.ctrl[5] = __ldcg(B.ctrl + 1) + (uint32_t)(total >> 31);  // next node id
  }
}

// Rounds of 32 clusters per warp in a merge tile (8 at most, 2048 clusters per tile): the fewest
// whose tiles still fill the grid, so that late iterations (few clusters) spread over all blocks.
// k_ploc_count and k_ploc_scatter run on the same grid and agree on it.
__device__ __forceinline__ int ploc_rounds(uint32_t c, uint32_t grid) {
#pragma unroll
  for (int r = 1; r < kPlocRounds; r <<= 1)
    if (div_up(c, (uint32_t)(kPlocThreads * r)) <= grid) return r;
  return kPlocRounds;
}
__device__ __forceinline__ int ploc_rounds(uint32_t c) { return ploc_rounds(c, gridDim.x); }

template <int R>
__device__ __forceinline__ void count_tiles(const PlocBufs& B, uint32_t c, uint32_t tiles, unsigned long long* s_w) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t base = tile * (uint32_t)(kPlocThreads * R) + w * (32u * R);
    // all rounds' neighbours, then their neighbours, so that each load batch is in flight at once
    int32_t j[R], back[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint32_t i = base + r * 32 + lane;
      j[r] = i < c ? __ldcg(B.nbr + i) : -1;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) back[r] = (j[r] >= 0 && (uint32_t)j[r] < c) ? __ldcg(B.nbr + j[r]) : -1;
    uint32_t tm = 0, tv = 0;
    uint2 mine = make_uint2(0u, 0u);  // lane r keeps round r's ballots
#pragma unroll
    for (int r = 0; r < R; ++r) {
      bool m, v;
      item_flags(c, base + r * 32 + lane, j[r], back[r], m, v);
      const uint32_t mb = __ballot_sync(0xffffffffu, m), vb = __ballot_sync(0xffffffffu, v);
      if (lane == r) mine = make_uint2(mb, vb);
      tm += __popc(mb);
      tv += __popc(vb);
    }
    if (lane < R) B.flags[((size_t)tile * (kPlocThreads / 32) + w) * R + lane] = mine;
    if (lane == 0) s_w[w] = ((unsigned long long)tm << 31) | tv;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
#pragma unroll
      for (int k = 0; k < kPlocThreads / 32; ++k) t += s_w[k];
      B.desc[tile] = t;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kPlocThreads) k_ploc_count(PlocBufs B) {
  __shared__ unsigned long long s_w[kPlocThreads / 32];
  const uint32_t c = __ldcg(B.ctrl + 0);
  const int R = ploc_rounds(c);
  const uint32_t tiles = div_up(c, (uint32_t)(kPlocThreads * R));
  switch (R) {
    case 1: count_tiles<1>(B, c, tiles, s_w); break;
    case 2: count_tiles<2>(B, c, tiles, s_w); break;
    case 4: count_tiles<4>(B, c, tiles, s_w); break;
    default: count_tiles<kPlocRounds>(B, c, tiles, s_w); break;
  }
  // the last block to finish scans the tile totals (ticket in ctrl[2])
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(B.ctrl + 2, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  ploc_scan_tiles(B, tiles, s_w);
  if (threadIdx.x == 0) B.ctrl[2] = 0;
}

template <int R, bool SEG>
__device__ __forceinline__ void scatter_tiles(const PlocBufs& B, uint32_t c, uint32_t next, uint32_t tiles,
                                              const Box* __restrict__ cin, const int32_t* __restrict__ idin,
                                              Box* __restrict__ cout, int32_t* __restrict__ idout,
                                              Node* __restrict__ nodes, unsigned long long* s_w,
                                              const PlocSeg& S) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t base = tile * (uint32_t)(kPlocThreads * R) + w * (32u * R);
    uint32_t mb[R], vb[R];
    int32_t nj[R];
    uint32_t tm = 0, tv = 0;
    // the ballots k_ploc_count stored; the partner of each merging cluster
    const uint2* fl = B.flags + ((size_t)tile * (kPlocThreads / 32) + w) * R;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint2 f = __ldcg(fl + r);
      mb[r] = f.x;
      vb[r] = f.y;
      nj[r] = ((f.x >> lane) & 1u) ? __ldcg(B.nbr + base + r * 32 + lane) : -1;
      tm += __popc(mb[r]);
      tv += __popc(vb[r]);
    }
    if (lane == 0) s_w[w] = ((unsigned long long)tm << 31) | tv;
    __syncthreads();
    unsigned long long before = __ldcg(B.desc + tile);
#pragma unroll
    for (int k = 0; k < kPlocThreads / 32; ++k)
      if (k < w) before += s_w[k];
    __syncthreads();  // s_w is rewritten by the next tile
    uint32_t mpos = (uint32_t)(before >> 31), vpos = (uint32_t)(before & 0x7fffffffull);
    // two rounds at a time: both rounds' boxes and ids are loaded before either round stores
#pragma unroll
    for (int r0 = 0; r0 < R; r0 += 2) {
      float4 lo[2], hi[2], jlo[2], jhi[2];
      int32_t id[2], jid[2];
#pragma unroll
      for (int g = 0; g < 2 && r0 + g < R; ++g) {
        const int r = r0 + g;
        const uint32_t i = base + r * 32 + lane;
        const bool m = (mb[r] >> lane) & 1u, v = (vb[r] >> lane) & 1u;
        lo[g] = hi[g] = jlo[g] = jhi[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        id[g] = jid[g] = 0;
        if (m || v) {
          const float4* ip = reinterpret_cast<const float4*>(cin + i);
          lo[g] = __ldcg(ip);
          hi[g] = __ldcg(ip + 1);
          id[g] = __ldcg(idin + i);
        }
        if (m) {
          const float4* jp = reinterpret_cast<const float4*>(cin + nj[r]);
          jlo[g] = __ldcg(jp);
          jhi[g] = __ldcg(jp + 1);
          jid[g] = __ldcg(idin + nj[r]);
        }
      }
#pragma unroll
      for (int g = 0; g < 2 && r0 + g < R; ++g) {
        const int r = r0 + g;
        const bool m = (mb[r] >> lane) & 1u, v = (vb[r] >> lane) & 1u;
        float4 a = lo[g], b = hi[g];
        int32_t nid = id[g];
        if (m) {
          // a batched cluster keeps its mesh in lo.w; nodes get 0 there
          a = make_float4(fminf(a.x, jlo[g].x), fminf(a.y, jlo[g].y), fminf(a.z, jlo[g].z), SEG ? a.w : 0.f);
          b = make_float4(fmaxf(b.x, jhi[g].x), fmaxf(b.y, jhi[g].y), fmaxf(b.z, jhi[g].z), 0.f);
          float4* np;
          np = nullptr;
          if constexpr (SEG) {
            const uint32_t mesh = (uint32_t)__float_as_int(a.w);
            const uint32_t local = mesh < S.count ? __ldcg(S.id_base + mesh) + mpos + __popc(mb[r] & lt) : ~0u;
            nid = (int32_t)local;  // children and cluster ids are mesh-local
            if (mesh < S.count) {
              const uint32_t off = __ldg(S.offsets + mesh), nm = __ldg(S.offsets + mesh + 1) - off;
              if (local < 2 * nm - 1) np = reinterpret_cast<float4*>(nodes + (2 * (size_t)off - mesh) + local);
            }
            if (!np) atomicOr(B.status, kStatusBadInput);  // outside its mesh's range: skipped
          } else {
            nid = (int32_t)(next + mpos + __popc(mb[r] & lt));
            np = reinterpret_cast<float4*>(nodes + nid);
            if (id[g] == 0) B.ctrl[13] = (uint32_t)nid;  // node 0's parent, for the root fix
          }
          if (np) {
            np[0] = make_float4(a.x, a.y, a.z, 0.f);
            np[1] = b;
            reinterpret_cast<int4*>(np + 2)[0] = make_int4(id[g], jid[g], 0, 0);
          }
        }
        if (v) {
          const uint32_t o = vpos + __popc(vb[r] & lt);
          float4* op = reinterpret_cast<float4*>(cout + o);
          op[0] = a;
          op[1] = b;
          idout[o] = nid;
        }
        mpos += __popc(mb[r]);
        vpos += __popc(vb[r]);
      }
    }
  }
}

template <bool SEG>
__global__ void __launch_bounds__(kPlocThreads, 3) k_ploc_scatter(PlocBufs B, PlocSeg S) {
  __shared__ unsigned long long s_w[kPlocThreads / 32];
  const uint32_t c = __ldcg(B.ctrl + 0);
  const uint32_t next = __ldcg(B.ctrl + 1);
  const uint32_t par = __ldcg(B.ctrl + 3) & 1u;
  // selects, not an indexed parameter array (which would be copied to the stack)
  const Box* __restrict__ cin = par ? B.cbox[1] : B.cbox[0];
  const int32_t* __restrict__ idin = par ? B.cid[1] : B.cid[0];
  Box* __restrict__ cout = par ? B.cbox[0] : B.cbox[1];
  int32_t* __restrict__ idout = par ? B.cid[0] : B.cid[1];
  Node* __restrict__ nodes = B.nodes;
  const int R = ploc_rounds(c);
  const uint32_t tiles = div_up(c, (uint32_t)(kPlocThreads * R));
  switch (R) {
    case 1: scatter_tiles<1, SEG>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w, S); break;
    case 2: scatter_tiles<2, SEG>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w, S); break;
    case 4: scatter_tiles<4, SEG>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w, S); break;
    default: scatter_tiles<kPlocRounds, SEG>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w, S); break;
  }
}

// Batched builds, between k_ploc_count (whose last block has scanned the tile totals) and
// k_ploc_scatter: per mesh, the global merge and survivor ranks of its first live cluster, from
// its tile's prefix and the stored ballots before it in the tile (at most 64 words).  From them
// the mesh's id base (a merge's local id = id_base + its global rank) and the position of its
// first cluster after the compaction.  mg_grid = the grid of k_ploc_count / k_ploc_scatter,
// which fixes their tiling.
__global__ void __launch_bounds__(256) k_ploc_seg(PlocBufs B, PlocSeg S, uint32_t mg_grid) {
  const uint32_t c = __ldcg(B.ctrl + 0);
  const uint32_t par = __ldcg(B.ctrl + 3) & 1u;
  const int R = ploc_rounds(c, mg_grid);
  const uint32_t per_tile = (uint32_t)kPlocThreads * (uint32_t)R, per_warp = 32u * (uint32_t)R;
  const uint32_t* seg_in = S.seg + (size_t)par * S.count;
  uint32_t* seg_out = S.seg + (size_t)(par ^ 1u) * S.count;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < S.count; m += gridDim.x * blockDim.x) {
    const uint32_t p = seg_in[m];
    const uint32_t pe = m + 1 < S.count ? seg_in[m + 1] : c;
    if (p >= c || pe > c || pe <= p) {  // inconsistent loop state: no ranks for this mesh
      atomicOr(B.status, kStatusBadInput);
      S.id_base[m] = ~0u;
      seg_out[m] = p;
      continue;
    }
    const uint32_t nm = __ldg(S.offsets + m + 1) - __ldg(S.offsets + m);
    const uint32_t tile = p / per_tile, o = p - tile * per_tile;
    const uint32_t w = o / per_warp, rr = (o % per_warp) >> 5, lane = o & 31u;
    const uint2* fl = B.flags + (size_t)tile * (kPlocThreads / 32) * R;
    uint32_t mc = 0, vc = 0;
    for (uint32_t k = 0; k < w * (uint32_t)R + rr; ++k) {  // whole rounds before p's round
      const uint2 f = __ldcg(fl + k);
      mc += __popc(f.x);
      vc += __popc(f.y);
    }
    const uint2 f = __ldcg(fl + w * (uint32_t)R + rr);
    const uint32_t below = (1u << lane) - 1u;
    mc += __popc(f.x & below);
    vc += __popc(f.y & below);
    const unsigned long long pre = __ldcg(B.desc + tile);
    const uint32_t G = (uint32_t)(pre >> 31) + mc, V = (uint32_t)(pre & 0x7fffffffull) + vc;
    // local id of the next new node = n_m + merges so far = 2 n_m - live clusters
    S.id_base[m] = 2u * nm - (pe - p) - G;
    seg_out[m] = V;
  }
}

// Batched builds: leaves and clusters from the sorted order of all meshes (positions
// [offsets[m], offsets[m+1]) hold mesh m's triangles in its own Morton order).  Mesh m's tree
// starts at node 2 offsets[m] - m; its leaves are nodes 0 .. n_m - 1 of that range (mesh-local
// ids, as a single build numbers them); indices get mesh-local triangle numbers.
__global__ void __launch_bounds__(256) k_ploc_init_seg(const uint32_t* __restrict__ sidx,
                                                       const Box* __restrict__ tri_boxes, PlocBufs B, PlocSeg S,
                                                       const SegItem* __restrict__ items, uint32_t n_items,
                                                       uint32_t n, uint32_t cap, uint32_t* __restrict__ d_indices) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    B.ctrl[0] = n;
    B.ctrl[1] = n;
    B.ctrl[2] = 0;
    B.ctrl[3] = 0;
    B.ctrl[6] = 0;
    B.ctrl[7] = cap;
    B.ctrl[8] = 0;
    B.ctrl[9] = 0;
    B.ctrl[11] = S.count;
    B.ctrl[12] = 0;
#pragma unroll
    for (int k = 14; k < 20; ++k) B.ctrl[k] = 0;
  }
  for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const SegItem w = items[it];
    const uint32_t off = __ldg(S.offsets + w.mesh);
    const size_t base = 2 * (size_t)off - w.mesh;
    if (w.begin == off && threadIdx.x == 0) S.seg[w.mesh] = off;
    for (uint32_t p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
      const uint32_t prim = __ldg(sidx + p);
      const float4* bp = reinterpret_cast<const float4*>(tri_boxes + prim);
      const float4 lo = __ldg(bp), hi = __ldg(bp + 1);
      float4* cb = reinterpret_cast<float4*>(B.cbox[0] + p);
      cb[0] = make_float4(lo.x, lo.y, lo.z, __int_as_float((int)w.mesh));
      cb[1] = hi;
      B.cid[0][p] = (int32_t)(p - off);
      float4* np = reinterpret_cast<float4*>(B.nodes + base + (p - off));
      np[0] = make_float4(lo.x, lo.y, lo.z, 0.f);
      np[1] = hi;
      reinterpret_cast<int4*>(np + 2)[0] = make_int4((int32_t)((prim - off) | kLeafBit), -1, 0, 0);
      d_indices[p] = prim - off;
    }
  }
}

// End of an iteration, one thread.
template <bool GRAPH>
__global__ void k_ploc_step(PlocBufs B, cudaGraphConditionalHandle handle) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ploc_step<GRAPH>(B, handle);
}

// The last iterations in one block.  Once the live clusters fit in shared memory (at most
// kTailMax, and few enough that their 2r pairs per cluster are cheap), an iteration over many
// blocks costs mostly launch latency; this kernel runs the remaining iterations in one block of
// kTailThreads, with the same rules and results as the kernels above: neighbour = smallest union
// area in [x-r, x+r], smallest j on ties, +inf and NaN never winning; mutual pairs merge into
// the smaller index, new node ids in ascending cluster order, survivors compacted in order; the
// same stop (one cluster), no-progress and cap rules, iteration count and live-cluster sum.
constexpr int kTailThreads = 1024;
constexpr uint32_t kTailMax = 2048;

uint32_t ploc_tail_threshold(int radius, uint32_t pairs) {
  if (pairs == 0) return 0;
  const uint32_t t = pairs / (2u * (uint32_t)std::max(radius, 1));
  return std::min<uint32_t>(kTailMax, std::max<uint32_t>(t, 64));
}
static size_t tail_smem() { return (size_t)kTailMax * (4 * 16 + 3 * 4) + 2 * 32 * 4; }

__global__ void __launch_bounds__(kTailThreads, 1) k_ploc_tail(PlocBufs B, int r) {
  extern __shared__ float4 tsm[];
  float4* s_lo[2] = {tsm, tsm + 2 * kTailMax};
  float4* s_hi[2] = {tsm + kTailMax, tsm + 3 * kTailMax};
  int32_t* s_id[2] = {reinterpret_cast<int32_t*>(tsm + 4 * kTailMax),
                      reinterpret_cast<int32_t*>(tsm + 4 * kTailMax) + kTailMax};
  int32_t* s_nbr = s_id[1] + kTailMax;
  uint32_t* s_w = reinterpret_cast<uint32_t*>(s_nbr + kTailMax);  // 2 x 32 warp sums
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) B.ctrl[19] = 1;
  uint32_t c = __ldcg(B.ctrl + 0);
  // nothing left, or the loop stopped without handing over (too many clusters, an error)
  if (c <= 1 || c > kTailMax || (__ldcg(B.status) & kStatusNoProgress)) return;
  const uint32_t par = __ldcg(B.ctrl + 3) & 1u;
  const Box* cin = par ? B.cbox[1] : B.cbox[0];
  const int32_t* idin = par ? B.cid[1] : B.cid[0];
  for (uint32_t x = tid; x < c; x += kTailThreads) {
    const float4* bp = reinterpret_cast<const float4*>(cin + x);
    s_lo[0][x] = __ldcg(bp);
    s_hi[0][x] = __ldcg(bp + 1);
    s_id[0][x] = __ldcg(idin + x);
  }
  uint32_t next = __ldcg(B.ctrl + 1), it = __ldcg(B.ctrl + 6);
  const uint32_t it0 = it;
  const uint32_t cap = __ldcg(B.ctrl + 7);
  unsigned long long sum = (unsigned long long)__ldcg(B.ctrl + 9) << 32 | __ldcg(B.ctrl + 8);
  int cur = 0;
  bool no_progress = false;
  const float kInf = __int_as_float(0x7f800000);
  __syncthreads();
  while (true) {
    sum += c;
    ++it;
    const float4* lo = s_lo[cur];
    const float4* hi = s_hi[cur];
    // neighbours: ascending j with a strict < keeps the smallest j of equal areas
    for (uint32_t x = tid; x < c; x += kTailThreads) {
      const float4 xa = lo[x], xb = hi[x];
      const uint32_t j0 = x > (uint32_t)r ? x - (uint32_t)r : 0u, j1 = min(c - 1, x + (uint32_t)r);
      float best = kInf;
      int32_t bj = -1;
      for (uint32_t j = j0; j <= j1; ++j) {
        if (j == x) continue;
        const float d = pair_area(xa, xb, lo[j], hi[j]);
        if (d < best) {
          best = d;
          bj = (int32_t)j;
        }
      }
      s_nbr[x] = bj;
    }
    __syncthreads();
    // merge and survivor flags of this thread's clusters x = 2 tid, 2 tid + 1 (ascending)
    uint32_t mk = 0, vk = 0;
    bool m2[2], v2[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint32_t x = 2u * (uint32_t)tid + (uint32_t)q;
      bool mm = false, vv = false;
      if (x < c) {
        const int32_t j = s_nbr[x];
        const bool mutual = j >= 0 && s_nbr[j] == (int32_t)x;
        mm = mutual && (int32_t)x < j;
        vv = !(mutual && j < (int32_t)x);
      }
      m2[q] = mm;
      v2[q] = vv;
      mk += mm;
      vk += vv;
    }
    // block exclusive scan of (merges, survivors), packed 16 + 16 bits (c <= 2048)
    uint32_t packed = mk << 16 | vk, x = packed;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t t = s_w[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      s_w[32 + lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t before = (wid ? s_w[32 + wid - 1] : 0u) + x - packed;
    const uint32_t total = s_w[32 + 31];
    uint32_t mpos = before >> 16, vpos = before & 0xffffu;
    const int nb = cur ^ 1;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint32_t xi = 2u * (uint32_t)tid + (uint32_t)q;
      if (xi >= c) continue;
      float4 a = lo[xi], b = hi[xi];
      int32_t nid = s_id[cur][xi];
      if (m2[q]) {
        const int32_t j = s_nbr[xi];
        const float4 ja = lo[j], jb = hi[j];
        a = make_float4(fminf(a.x, ja.x), fminf(a.y, ja.y), fminf(a.z, ja.z), 0.f);
        b = make_float4(fmaxf(b.x, jb.x), fmaxf(b.y, jb.y), fmaxf(b.z, jb.z), 0.f);
        const int32_t id_new = (int32_t)(next + mpos);
        float4* np = reinterpret_cast<float4*>(B.nodes + id_new);
        np[0] = a;
        np[1] = b;
        reinterpret_cast<int4*>(np + 2)[0] = make_int4(nid, s_id[cur][j], 0, 0);
        if (nid == 0) B.ctrl[13] = (uint32_t)id_new;  // node 0's parent, for the root fix
        nid = id_new;
        ++mpos;
      }
      if (v2[q]) {
        s_lo[nb][vpos] = a;
        s_hi[nb][vpos] = b;
        s_id[nb][vpos] = nid;
        ++vpos;
      }
    }
    const uint32_t nc = total & 0xffffu, merges = total >> 16;
    next += merges;
    __syncthreads();  // the next buffer is complete; this iteration's buffers are free
    cur = nb;
    const uint32_t prev = c;
    c = nc;
    if (c <= 1) break;
    if (c >= prev || it >= cap) {  // no mutual pair anywhere, or the cap
      no_progress = true;
      break;
    }
  }
  if (tid == 0) {
    B.ctrl[0] = c;
    B.ctrl[1] = next;
    B.ctrl[6] = it;
    B.ctrl[8] = (uint32_t)sum;
    B.ctrl[9] = (uint32_t)(sum >> 32);
    B.ctrl[17] = it - it0;
    if (no_progress) atomicOr(B.status, kStatusNoProgress);
  }
}

// The middle iterations in one cooperative kernel.  Between the iterations over many clusters
// (one launch per phase over persistent grids) and k_ploc_tail (one block), an iteration costs
// mostly the latency of its four launches.  k_ploc_grid runs those iterations in one cooperative
// launch (every block resident): block b owns the contiguous chunk [b*ch, (b+1)*ch) of at most
// kGridPerBlock clusters and stages its window (the chunk and r clusters either side) in shared
// memory; grid barriers separate the neighbour search, the flag count and the merge + compaction.
// Same rules and results as the kernels above and k_ploc_tail (neighbour = smallest union area in
// [x-r, x+r], smallest j on ties, +inf and NaN never winning; mutual pairs merge into the smaller
// index; new ids in ascending cluster order; survivors compacted in order; the same stop rules,
// iteration count and live-cluster sum).  It runs while the live clusters number more than the
// tail hand-over (ctrl[12]) and at most kGridPerBlock per block.
constexpr int kGridThreads = 1024;
constexpr uint32_t kGridPerBlock = 2048;
constexpr int kGridPer = (int)kGridPerBlock / kGridThreads;  // consecutive clusters per thread
constexpr int kGridMaxR = 128;
// the window: the chunk and 2r clusters either side (the neighbours of the chunk and of r
// clusters either side of it, so the flag count needs no other block's neighbours)
constexpr uint32_t kGridWin = kGridPerBlock + 4 * kGridMaxR;
constexpr uint32_t kGridNbr = kGridPerBlock + 2 * kGridMaxR;
constexpr uint32_t kGridMaxBlocks = 1024;
static size_t grid_smem() { return (size_t)kGridWin * (2 * 16 + 4) + (size_t)kGridNbr * 4 + 64 * 8; }

// Exclusive block scan of one 64-bit value per thread (kGridThreads); *total gets the sum.
__device__ __forceinline__ unsigned long long grid_block_scan(unsigned long long v, unsigned long long* s_w,
                                                              unsigned long long* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned long long t = s_w[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    s_w[32 + lane] = t;  // inclusive warp totals
  }
  __syncthreads();
  const unsigned long long before = (wid ? s_w[32 + wid - 1] : 0ull) + x - v;
  *total = s_w[32 + 31];
  __syncthreads();  // s_w is reused by the next scan
  return before;
}

__global__ void __launch_bounds__(kGridThreads, 1) k_ploc_grid(PlocBufs B, int r) {
  extern __shared__ float4 gsm[];
  float4* s_lo = gsm;
  float4* s_hi = gsm + kGridWin;
  int32_t* s_id = reinterpret_cast<int32_t*>(gsm + 2 * kGridWin);
  int32_t* s_nbr = s_id + kGridWin;  // neighbours of [h0, h1)
  unsigned long long* s_w = reinterpret_cast<unsigned long long*>(s_nbr + kGridNbr);
  __shared__ uint32_t s_ok;
  const uint32_t G = gridDim.x, b = blockIdx.x;
  const int tid = threadIdx.x;
  if (b == 0 && tid == 0) B.ctrl[18] = 1;  // (no block reads it)
  // every block reads the same words (nothing writes them before the first barrier)
  uint32_t c = __ldcg(B.ctrl + 0);
  const uint32_t tail = __ldcg(B.ctrl + 12), cap = __ldcg(B.ctrl + 7);
  if (c <= 1 || c <= tail || c > G * kGridPerBlock || r > kGridMaxR || r < 1 ||
      (__ldcg(B.status) & kStatusNoProgress))
    return;
  uint32_t next = __ldcg(B.ctrl + 1), par = __ldcg(B.ctrl + 3) & 1u, it = __ldcg(B.ctrl + 6);
  const uint32_t it0 = it;
  unsigned long long sum = (unsigned long long)__ldcg(B.ctrl + 9) << 32 | __ldcg(B.ctrl + 8);
  uint32_t* bar = B.ctrl + 15;
  unsigned long long* totals = reinterpret_cast<unsigned long long*>(B.flags);  // one per block
  uint32_t nbar = 0;
  bool no_progress = false, ok = true;
  const float kInf = __int_as_float(0x7f800000);
  while (true) {
    const Box* cin = par ? B.cbox[1] : B.cbox[0];
    const int32_t* idin = par ? B.cid[1] : B.cid[0];
    Box* cout = par ? B.cbox[0] : B.cbox[1];
    int32_t* idout = par ? B.cid[0] : B.cid[1];
    const uint32_t ch = div_up(c, G);
    const uint32_t x0 = min(c, b * ch), x1 = min(c, x0 + ch);
    const uint32_t h0 = x0 > (uint32_t)r ? x0 - (uint32_t)r : 0u, h1 = min(c, x1 + (uint32_t)r);
    const uint32_t w0 = h0 > (uint32_t)r ? h0 - (uint32_t)r : 0u, w1 = min(c, h1 + (uint32_t)r);
    for (uint32_t x = w0 + tid; x < w1; x += kGridThreads) {
      const float4* bp = reinterpret_cast<const float4*>(cin + x);
      s_lo[x - w0] = __ldcg(bp);
      s_hi[x - w0] = __ldcg(bp + 1);
      s_id[x - w0] = __ldcg(idin + x);
    }
    __syncthreads();
    // neighbours of the chunk and r clusters either side: ascending j with a strict < keeps the
    // smallest j of equal areas
    for (uint32_t x = h0 + tid; x < h1; x += kGridThreads) {
      const float4 xa = s_lo[x - w0], xb = s_hi[x - w0];
      const uint32_t j0 = x > (uint32_t)r ? x - (uint32_t)r : 0u, j1 = min(c - 1, x + (uint32_t)r);
      float best = kInf;
      int32_t bj = -1;
      for (uint32_t j = j0; j <= j1; ++j) {
        if (j == x) continue;
        const float d = pair_area(xa, xb, s_lo[j - w0], s_hi[j - w0]);
        if (d < best) {
          best = d;
          bj = (int32_t)j;
        }
      }
      s_nbr[x - h0] = bj;
    }
    __syncthreads();
    // merge / survivor flags of this thread's clusters x0 + kGridPer tid + q (ascending); a
    // neighbour j lies within r of x, so both j and its neighbour are in s_nbr
    bool m2[kGridPer], v2[kGridPer];
    int32_t nj[kGridPer];
    uint32_t mk = 0, vk = 0;
#pragma unroll
    for (int q = 0; q < kGridPer; ++q) {
      const uint32_t x = x0 + (uint32_t)kGridPer * (uint32_t)tid + (uint32_t)q;
      m2[q] = v2[q] = false;
      nj[q] = -1;
      if (x < x1) {
        const int32_t j = s_nbr[x - h0];
        const int32_t back = j >= 0 ? s_nbr[(uint32_t)j - h0] : -1;
        const bool mutual = j >= 0 && back == (int32_t)x;
        m2[q] = mutual && (int32_t)x < j;
        v2[q] = !(mutual && j < (int32_t)x);
        nj[q] = j;
      }
      mk += m2[q];
      vk += v2[q];
    }
    unsigned long long btot;
    const unsigned long long before = grid_block_scan((unsigned long long)mk << 32 | vk, s_w, &btot);
    if (tid == 0) __stcg(totals + b, btot);
    if (!(ok = grid_sync(bar, ++nbar * G, B.status, &s_ok))) break;
    // this block's offset and the totals over all blocks
    unsigned long long mine = 0;
    for (uint32_t k = (uint32_t)tid; k < G; k += kGridThreads) mine += k < b ? __ldcg(totals + k) : 0ull;
    unsigned long long all = 0;
    for (uint32_t k = (uint32_t)tid; k < G; k += kGridThreads) all += __ldcg(totals + k);
    unsigned long long offs_b, grand_b;  // the block sums of `mine` and `all`
    grid_block_scan(mine, s_w, &offs_b);
    grid_block_scan(all, s_w, &grand_b);
    uint32_t mpos = (uint32_t)(offs_b >> 32) + (uint32_t)(before >> 32);
    uint32_t vpos = (uint32_t)offs_b + (uint32_t)before;
    const uint32_t M = (uint32_t)(grand_b >> 32), V = (uint32_t)grand_b;
#pragma unroll
    for (int q = 0; q < kGridPer; ++q) {
      const uint32_t xi = x0 + (uint32_t)kGridPer * (uint32_t)tid + (uint32_t)q;
      if (xi >= x1) continue;
      float4 a = s_lo[xi - w0], bb = s_hi[xi - w0];
      int32_t nid = s_id[xi - w0];
      if (m2[q]) {
        const uint32_t j = (uint32_t)nj[q];  // within [xi - r, xi + r], so inside the staged window
        const float4 ja = s_lo[j - w0], jb = s_hi[j - w0];
        a = make_float4(fminf(a.x, ja.x), fminf(a.y, ja.y), fminf(a.z, ja.z), 0.f);
        bb = make_float4(fmaxf(bb.x, jb.x), fmaxf(bb.y, jb.y), fmaxf(bb.z, jb.z), 0.f);
        const int32_t id_new = (int32_t)(next + mpos);
        float4* np = reinterpret_cast<float4*>(B.nodes + id_new);
        np[0] = a;
        np[1] = bb;
        reinterpret_cast<int4*>(np + 2)[0] = make_int4(nid, s_id[j - w0], 0, 0);
        if (nid == 0) B.ctrl[13] = (uint32_t)id_new;  // node 0's parent, for the root fix
        nid = id_new;
        ++mpos;
      }
      if (v2[q]) {
        float4* op = reinterpret_cast<float4*>(cout + vpos);
        op[0] = a;
        op[1] = bb;
        idout[vpos] = nid;
        ++vpos;
      }
    }
    sum += c;
    ++it;
    next += M;
    const uint32_t prev = c;
    c = V;
    par ^= 1u;
    if (c <= 1) break;
    if (c >= prev || it >= cap) {  // no mutual pair anywhere, or the cap
      no_progress = true;
      break;
    }
    if (c <= tail) break;
    if (!(ok = grid_sync(bar, ++nbar * G, B.status, &s_ok))) break;  // the next window reads the compacted buffer
  }
  if (ok && b == 0 && tid == 0) {
    B.ctrl[0] = c;
    B.ctrl[1] = next;
    B.ctrl[3] = par;
    B.ctrl[6] = it;
    B.ctrl[8] = (uint32_t)sum;
    B.ctrl[9] = (uint32_t)(sum >> 32);
    B.ctrl[16] = it - it0;
    if (no_progress) atomicOr(B.status, kStatusNoProgress);
  }
}

// Self-test of the grid barrier's bound: a cooperative launch whose blocks wait for one arrival
// more than there are blocks (a block that never comes), giving up after `limit` polls each.
// Words: [0] arrival counter, [1] status.
__device__ uint32_t g_grid_selftest[2];

__global__ void k_grid_selftest(uint32_t limit) {
  __shared__ uint32_t s_ok;
  grid_sync(g_grid_selftest, gridDim.x + 1, g_grid_selftest + 1, &s_ok, limit);
}

cudaError_t grid_wait_selftest(uint32_t limit, uint32_t* status_out) {
  int dev = 0, coop = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (e != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  cudaStream_t st = nullptr;
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return e;
  const uint32_t zero[2] = {0u, 0u};
  e = cudaMemcpyToSymbolAsync(g_grid_selftest, zero, sizeof(zero), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(4);
    cfg.blockDim = dim3(64);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_grid_selftest, limit);
  }
  if (e == cudaSuccess) e = cudaMemcpyFromSymbolAsync(status_out, g_grid_selftest, 4, 4, cudaMemcpyDeviceToHost, st);
  const cudaError_t e2 = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return e != cudaSuccess ? e : e2;
}

// Move the root (last node) to index 0 and swap every reference to 0 and the root
// (ploc_builder.cu:563-582); skipped when the loop did not converge.  The root has no parent and
// node 0 (a leaf) has one, recorded by the merge that made it (ctrl[13]), so three nodes change:
// 0, R and that parent.  Without a recorded parent every node is checked (one block).
__global__ void k_ploc_root(Node* __restrict__ nodes, uint32_t total, const uint32_t* __restrict__ ctrl) {
  if (__ldcg(ctrl + 0) != 1 || total < 2) return;
  const uint32_t R = total - 1;
  auto fix = [&](int32_t c) -> int32_t {
    if (c < 0) return c;
    if (c == 0) return (int32_t)R;
    if (c == (int32_t)R) return 0;
    return c;
  };
  const uint32_t p = __ldcg(ctrl + 13);
  const bool known = p > 0 && p < total;
  for (uint32_t k = threadIdx.x; k < total; k += blockDim.x) {
    if (known && k != 0) {  // only node 0's parent refers to 0 or R (R itself moves with k == 0)
      if (k == 1 && p != R) {
        int2 ch = *reinterpret_cast<int2*>(&nodes[p].left);
        *reinterpret_cast<int2*>(&nodes[p].left) = make_int2(fix(ch.x), fix(ch.y));
      }
      break;
    }
    if (k == 0) {
      Node a = nodes[0], b = nodes[R];
      if (b.left >= 0) { b.left = fix(b.left); b.right = fix(b.right); }
      if (a.left >= 0) { a.left = fix(a.left); a.right = fix(a.right); }
      nodes[0] = b;
      nodes[R] = a;
    } else if (k != R) {
      int2 ch = *reinterpret_cast<int2*>(&nodes[k].left);
      if (ch.x >= 0) {
        int2 nc = make_int2(fix(ch.x), fix(ch.y));
        if (nc.x != ch.x || nc.y != ch.y) *reinterpret_cast<int2*>(&nodes[k].left) = nc;
      }
    }
  }
}

// Batched builds: each mesh's root (its last node) moves to the start of its range, as in
// k_ploc_root; work items split the node ranges evenly.
__global__ void __launch_bounds__(256) k_ploc_root_seg(Node* __restrict__ nodes, const SegItem* __restrict__ items,
                                                       uint32_t n_items, PlocSeg S, const uint32_t* __restrict__ ctrl) {
  if (__ldcg(ctrl + 0) != S.count) return;
  for (uint32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const SegItem w = items[it];
    const uint32_t off = __ldg(S.offsets + w.mesh), nm = __ldg(S.offsets + w.mesh + 1) - off;
    Node* mn = nodes + (2 * (size_t)off - w.mesh);
    const uint32_t R = 2 * nm - 2;
    auto fix = [&](int32_t c) -> int32_t {
      if (c < 0) return c;
      if (c == 0) return (int32_t)R;
      if (c == (int32_t)R) return 0;
      return c;
    };
    const uint32_t k0 = 2 * (w.begin - off), k1 = min(2 * (w.end - off), 2 * nm - 1);
    for (uint32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      if (k == 0) {
        Node a = mn[0], b = mn[R];
        if (b.left >= 0) { b.left = fix(b.left); b.right = fix(b.right); }
        if (a.left >= 0) { a.left = fix(a.left); a.right = fix(a.right); }
        mn[0] = b;
        mn[R] = a;
      } else if (k != R) {
        int2 ch = *reinterpret_cast<int2*>(&mn[k].left);
        if (ch.x >= 0) {
          int2 nc = make_int2(fix(ch.x), fix(ch.y));
          if (nc.x != ch.x || nc.y != ch.y) *reinterpret_cast<int2*>(&mn[k].left) = nc;
        }
      }
    }
  }
}

cudaError_t workspace_reserve_ploc(Workspace& ws, uint32_t n) {
  if (!ws.aux_stream) {  // captures the batched loop body while a batch is being captured
    cudaError_t e = cudaStreamCreateWithFlags(&ws.aux_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
  }
  if (n <= ws.ploc_cap && ws.nbr) return cudaSuccess;
  uint32_t cap = std::max<uint32_t>(n, 1024);
  if (ws.ploc_exec) {
    cudaGraphExecDestroy(ws.ploc_exec);
    ws.ploc_exec = nullptr;
  }
  if (ws.ploc_seg_exec) {  // both loop graphs hold the cluster buffers' addresses
    cudaGraphExecDestroy(ws.ploc_seg_exec);
    ws.ploc_seg_exec = nullptr;
  }
  cudaFree(ws.cbox[0]); cudaFree(ws.cbox[1]); cudaFree(ws.cid[0]); cudaFree(ws.cid[1]); cudaFree(ws.nbr);
  ws.cbox[0] = ws.cbox[1] = nullptr; ws.cid[0] = ws.cid[1] = nullptr; ws.nbr = nullptr; ws.ploc_cap = 0;
  cudaError_t e;
  if ((e = cudaMalloc(&ws.cbox[0], (size_t)cap * sizeof(Box))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.cbox[1], (size_t)cap * sizeof(Box))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.cid[0], (size_t)cap * 4)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.cid[1], (size_t)cap * 4)) != cudaSuccess) return e;
  // neighbours (cap) + per-tile merge totals / prefixes (64-bit) share one allocation
  // ... and the per-round ballots (8 B per 32 clusters)
  size_t desc_words = div_up(cap, kPlocTile) + 8;
  // (smaller tiles in late iterations: at most one partial tile's worth more; never more tiles
  // than the grid, so desc_words holds their totals)
  size_t flag_words = (size_t)div_up(cap, kPlocTile) * (kPlocThreads / 32) * kPlocRounds +
                      (kPlocThreads / 32) * kPlocRounds;
  if ((e = cudaMalloc(&ws.nbr, (size_t)cap * 4 + desc_words * 8 + flag_words * 8 + 64)) != cudaSuccess) return e;
  ws.ploc_cap = cap;
  return cudaSuccess;
}

static size_t nn_smem(int radius) {
  const size_t strided = 32 * (kNnTile + 2 * (size_t)radius) + 4 * (size_t)kNnKc * kNnTile;
  return radius <= kNcMaxR ? std::max(strided, nc_smem(radius)) : strided;
}

// Persistent grids sized for n, capped at `bps` blocks per SM (the workspace's launch shapes).
struct PlocShape {
  int nn_bps, mg_bps;
  uint32_t key() const { return (uint32_t)nn_bps << 16 | (uint32_t)mg_bps; }
};
static PlocShape ploc_shape(const Workspace& ws) {
  return PlocShape{std::max(1, std::min(ws.ploc_nn_bps, 16)), std::max(1, std::min(ws.ploc_mg_bps, 32))};
}
static uint32_t nn_grid_for(uint32_t n, const PlocShape& sh) {
  return std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kNnTile), 152u * (uint32_t)sh.nn_bps));
}
static uint32_t mg_grid_for(uint32_t n, const PlocShape& sh) {
  return std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kPlocTile), 152u * (uint32_t)sh.mg_bps));
}

// One clustering iteration: neighbours, tile counts + scan, (batched: per-mesh ranks), merge +
// compaction, loop control.  Grids are persistent (sized for n); the kernels read the live
// cluster count from the control words.
template <bool SEG, bool GRAPH>
static void enqueue_iteration(const PlocBufs& B, const PlocSeg& S, uint32_t n, int radius, const PlocShape& sh,
                              cudaStream_t st, cudaGraphConditionalHandle handle) {
  const uint32_t mg_grid = mg_grid_for(n, sh);
  k_ploc_nn<SEG><<<nn_grid_for(n, sh), kPlocThreads, nn_smem(radius), st>>>(B, radius);
  k_ploc_count<<<mg_grid, kPlocThreads, 0, st>>>(B);
  if constexpr (SEG) k_ploc_seg<<<std::max<uint32_t>(1, std::min<uint32_t>(div_up(S.count, 256), 152 * 4)), 256, 0,
                                  st>>>(B, S, mg_grid);
  k_ploc_scatter<SEG><<<mg_grid, kPlocThreads, 0, st>>>(B, S);
  k_ploc_step<GRAPH><<<1, 32, 0, st>>>(B, handle);
}

// The loop as a graph: WHILE(cond) { one iteration }.
template <bool SEG>
static cudaError_t make_loop_graph(const PlocBufs& B, const PlocSeg& S, uint32_t n, int radius, const PlocShape& sh,
                                   cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle handle;
  cudaStream_t cs = nullptr;
  cudaGraphNode_t node;
  cudaGraphNodeParams cp = {};
  do {
    if ((e = cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if ((e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp)) != cudaSuccess) break;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
      break;
    enqueue_iteration<SEG, true>(B, S, n, radius, sh, cs, handle);
    cudaGraph_t captured = nullptr;
    cudaError_t e2 = cudaGetLastError();
    e = cudaStreamEndCapture(cs, &captured);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) break;
    e = cudaGraphInstantiate(out, g, 0);
  } while (false);
  if (cs) cudaStreamDestroy(cs);
  cudaGraphDestroy(g);
  return e;
}

static PlocBufs ploc_bufs(Workspace& ws, const ScratchLayout& L) {
  PlocBufs B;
  B.cbox[0] = ws.cbox[0];
  B.cbox[1] = ws.cbox[1];
  B.cid[0] = ws.cid[0];
  B.cid[1] = ws.cid[1];
  B.nbr = ws.nbr;
  B.desc = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(ws.nbr) +
                                                  (((size_t)ws.ploc_cap * 4 + 15) & ~size_t(15)));
  B.flags = reinterpret_cast<uint2*>(B.desc + div_up(ws.ploc_cap, kPlocTile) + 8);
  B.nodes = ws.nodes;
  B.ctrl = ws.scratch + L.ploc;
  B.status = ws.scratch + L.status;
  return B;
}

template <bool SEG>
static cudaError_t set_nn_smem(int radius) {
  if (nn_smem(radius) <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(k_ploc_nn<SEG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nn_smem(radius));
}

static cudaError_t set_tail_smem() {
  return cudaFuncSetAttribute(k_ploc_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tail_smem());
}

// Blocks of a k_ploc_grid launch on the current device: SMs x resident blocks per SM, or 0 where
// cooperative launches are not available.  Sets the kernel's shared-memory limit (so it is called
// before any capture, from ploc_prepare, and again by builds).
static uint32_t ploc_grid_blocks() {
  int dev = 0, coop = 0, sms = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaFuncSetAttribute(k_ploc_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grid_smem()) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_ploc_grid, kGridThreads, grid_smem()) != cudaSuccess)
    return 0;
  return (uint32_t)std::min<long long>((long long)sms * occ, kGridMaxBlocks);
}

cudaError_t ploc_prepare(int radius) {
  cudaError_t e = set_nn_smem<false>(radius);
  if (e == cudaSuccess) e = set_nn_smem<true>(radius);
  if (e == cudaSuccess) e = set_tail_smem();
  if (e == cudaSuccess) ploc_grid_blocks();
  return e;
}

cudaError_t ploc_build(Workspace& ws, const MeshPtrs& m, uint32_t n, int radius, int max_iter, cudaStream_t st,
                       StageEvents* evs, uint32_t** out_indices, bool host_loop) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  if ((e = workspace_reserve_ploc(ws, n)) != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  const PlocBufs B = ploc_bufs(ws, L);
  const PlocSeg none{};
  if ((e = set_nn_smem<false>(radius)) != cudaSuccess) return e;
  if ((e = set_tail_smem()) != cudaSuccess) return e;
  // every iteration that makes progress removes at least one cluster, so n bounds the loop
  const uint32_t cap = max_iter > 0 ? (uint32_t)max_iter : n;
  const uint32_t tail = ploc_tail_threshold(radius, ws.ploc_tail_pairs);
  // k_ploc_grid: from grid_at live clusters down to the tail hand-over (its per-block totals
  // live in the ballot words, which hold them from 65,536 triangles on)
  const uint32_t grid_blocks = ploc_grid_blocks();
  uint32_t grid_at = 0;
  if (grid_blocks && radius <= kGridMaxR && n >= 65536)
    grid_at = std::min<uint32_t>(ws.ploc_grid_max, grid_blocks * kGridPerBlock);
  if (grid_at <= tail) grid_at = 0;
  const bool loop = n > 1 && n > std::max(tail, grid_at);  // else the one-launch kernels do every iteration
  const PlocShape sh = ploc_shape(ws);
  if (host_loop && !ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
  if (loop && !host_loop) {
    const bool same = ws.ploc_exec && ws.ploc_key_n == n && ws.ploc_key_r == radius && ws.ploc_key_nodes == ws.nodes &&
                      ws.ploc_key_scratch == ws.scratch && ws.ploc_key_shape == sh.key();
    if (!same) {
      if (ws.ploc_exec) cudaGraphExecDestroy(ws.ploc_exec);
      ws.ploc_exec = nullptr;
      if ((e = make_loop_graph<false>(B, none, n, radius, sh, &ws.ploc_exec)) != cudaSuccess) return e;
      ws.ploc_key_n = n;
      ws.ploc_key_r = radius;
      ws.ploc_key_nodes = ws.nodes;
      ws.ploc_key_scratch = ws.scratch;
      ws.ploc_key_shape = sh.key();
    }
  }
  if (evs && evs->use) cudaEventRecord(evs->ev[0], st);
  uint32_t* sidx = nullptr;
  if ((e = prefix_sort30(ws, m, n, st, evs, &sidx)) != cudaSuccess) return e;
  *out_indices = sidx;
  k_ploc_init<<<div_up(n, 256), 256, 0, st>>>(sidx, ws.boxes, B, n, cap, tail, grid_at);
  if (evs && evs->use) cudaEventRecord(evs->ev[4], st);
  if (loop && host_loop) {
    for (uint32_t it = 0; it < cap; ++it) {
      enqueue_iteration<false, false>(B, none, n, radius, sh, st, cudaGraphConditionalHandle{});
      if ((e = cudaMemcpyAsync(ws.ploc_host, B.ctrl + 10, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
      if (!*ws.ploc_host) break;
    }
  } else if (loop) {
    if ((e = cudaGraphLaunch(ws.ploc_exec, st)) != cudaSuccess) return e;
  }
  if (n > 1) {
    if (grid_at) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid_blocks);
      cfg.blockDim = dim3(kGridThreads);
      cfg.dynamicSmemBytes = grid_smem();
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      e = ws.no_cooperative ? cudaErrorNotSupported : cudaLaunchKernelEx(&cfg, k_ploc_grid, B, radius);
      if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
        // no co-resident grid (a client limited to part of the GPU, or asked for): the same
        // iterations as one launch per kernel each, driven from the host, down to the tail
        // hand-over; the loop above stopped at grid_at live clusters or for good
        (void)cudaGetLastError();
        if (!ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(B.ctrl + 14, 0, 4, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(ws.ploc_host, B.ctrl, 8 * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
          return e;
        bool go = ws.ploc_host[0] > std::max<uint32_t>(tail, 1u) && ws.ploc_host[6] < ws.ploc_host[7];
        while (go) {
          enqueue_iteration<false, false>(B, none, n, radius, sh, st, cudaGraphConditionalHandle{});
          if ((e = cudaMemcpyAsync(ws.ploc_host, B.ctrl + 10, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
              (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return e;
          go = *ws.ploc_host != 0;
        }
      } else if (e != cudaSuccess) {
        return e;
      }
    }
    if (tail) k_ploc_tail<<<1, kTailThreads, tail_smem(), st>>>(B, radius);
    k_ploc_root<<<1, 256, 0, st>>>(ws.nodes, 2 * n - 1, B.ctrl);
  }
  if (evs && evs->use) cudaEventRecord(evs->ev[5], st);
  return cudaGetLastError();
}

// Batched PLOC: the batched prefix (per-mesh boxes and keys, one sort), then every mesh's
// clustering in the same iterations -- windows clipped at mesh boundaries, merges numbered per
// mesh -- until each mesh has one cluster, then each mesh's root fix.  Mesh m's result equals its
// single build: the same leaves, the same neighbours in every iteration, the same node ids
// relative to its range [2 offsets[m] - m, 2 offsets[m+1] - m - 1).  A mesh that has finished
// keeps its one cluster, which has no neighbour.  The loop is a CUDA graph WHILE node (or a
// host loop); the iteration count is the largest of the meshes' own.
cudaError_t batched_ploc_build(Workspace& ws, const MeshPtrs& m, uint32_t n, const uint32_t* d_offsets,
                               uint32_t count, const SegItem* d_items, uint32_t n_items, float* d_mbox,
                               uint32_t* d_indices, int radius, uint32_t max_iter, cudaStream_t st,
                               StageEvents* evs, bool host_loop) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  if ((e = workspace_reserve_ploc(ws, n)) != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  const PlocBufs B = ploc_bufs(ws, L);
  PlocSeg S;
  S.offsets = d_offsets;
  S.seg = reinterpret_cast<uint32_t*>(d_mbox);  // the mesh boxes are dead once the keys are made
  S.id_base = S.seg + 2 * (size_t)count;
  S.count = count;
  if ((e = set_nn_smem<true>(radius)) != cudaSuccess) return e;
  const uint32_t cap = max_iter > 0 ? max_iter : n;
  if (host_loop && !ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
  const bool loop = n > count;  // some mesh has two or more triangles
  const PlocShape sh = ploc_shape(ws);
  cudaStreamCaptureStatus cst0 = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(st, &cst0)) != cudaSuccess) return e;
  if (loop && !host_loop && cst0 == cudaStreamCaptureStatusNone) {
    const bool same = ws.ploc_seg_exec && ws.ploc_seg_key_n == n && ws.ploc_seg_key_count == count &&
                      ws.ploc_seg_key_r == radius && ws.ploc_seg_key[0] == ws.nodes &&
                      ws.ploc_seg_key[1] == ws.scratch && ws.ploc_seg_key[2] == d_offsets &&
                      ws.ploc_seg_key[3] == d_mbox && ws.ploc_seg_key_shape == sh.key();
    if (!same) {
      if (ws.ploc_seg_exec) cudaGraphExecDestroy(ws.ploc_seg_exec);
      ws.ploc_seg_exec = nullptr;
      if ((e = make_loop_graph<true>(B, S, n, radius, sh, &ws.ploc_seg_exec)) != cudaSuccess) return e;
      ws.ploc_seg_key_shape = sh.key();
      ws.ploc_seg_key_n = n;
      ws.ploc_seg_key_count = count;
      ws.ploc_seg_key_r = radius;
      ws.ploc_seg_key[0] = ws.nodes;
      ws.ploc_seg_key[1] = ws.scratch;
      ws.ploc_seg_key[2] = d_offsets;
      ws.ploc_seg_key[3] = d_mbox;
    }
  }
  BatchedSort bs;
  if ((e = batched_prefix(ws, m, n, count, d_items, n_items, d_mbox, st, evs, &bs)) != cudaSuccess) return e;
  const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(n_items, 152 * 8));
  k_ploc_init_seg<<<grid, 256, 0, st>>>(ws.vals[bs.fb], ws.boxes, B, S, d_items, n_items, n, cap, d_indices);
  if (evs && evs->use) cudaEventRecord(evs->ev[4], st);
  if (loop && host_loop) {
    for (uint32_t it = 0; it < cap; ++it) {
      enqueue_iteration<true, false>(B, S, n, radius, sh, st, cudaGraphConditionalHandle{});
      if ((e = cudaMemcpyAsync(ws.ploc_host, B.ctrl + 10, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
      if (!*ws.ploc_host) break;
    }
  } else if (loop) {
    cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edata = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(st, &cst, nullptr, &cg, &deps, &edata, &nd)) != cudaSuccess) return e;
    if (cst == cudaStreamCaptureStatusActive) {
      // the batch is being captured into one graph: the loop becomes a conditional node of it
      cudaGraphConditionalHandle h;
      if ((e = cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      if ((e = cudaGraphAddNode(&node, cg, deps, edata, nd, &cp)) != cudaSuccess) return e;
      cudaStream_t aux = ws.aux_stream;
      if (!aux) return cudaErrorInvalidResourceHandle;  // made by workspace_reserve_ploc, before any capture
      if ((e = cudaStreamBeginCaptureToGraph(aux, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return e;
      enqueue_iteration<true, true>(B, S, n, radius, sh, aux, h);
      cudaGraph_t body = nullptr;
      const cudaError_t e2 = cudaGetLastError();
      if ((e = cudaStreamEndCapture(aux, &body)) != cudaSuccess) return e;
      if (e2 != cudaSuccess) return e2;
      if ((e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
          cudaSuccess)
        return e;
    } else if ((e = cudaGraphLaunch(ws.ploc_seg_exec, st)) != cudaSuccess) {
      return e;
    }
  }
  if (loop) k_ploc_root_seg<<<grid, 256, 0, st>>>(ws.nodes, d_items, n_items, S, B.ctrl);
  if (evs && evs->use) cudaEventRecord(evs->ev[5], st);
  return cudaGetLastError();
}

// Order-independent hash of a tree's node fields: each node's (index, min, max, left, right)
// mixed to 64 bits (splitmix64 finaliser), XOR-combined per warp and then atomically.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) k_tree_hash(const Node* __restrict__ nodes, uint32_t n_nodes,
                                                   unsigned long long* __restrict__ out) {
  unsigned long long h = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += gridDim.x * blockDim.x) {
    const float4* p = reinterpret_cast<const float4*>(nodes + i);
    const float4 lo = __ldg(p), hi = __ldg(p + 1);
    const int2 ch = __ldg(reinterpret_cast<const int2*>(p + 2));
    unsigned long long z = mix64(i + 0x9e3779b97f4a7c15ull);
    z = mix64(z ^ ((unsigned long long)__float_as_uint(lo.x) << 32 | __float_as_uint(lo.y)));
    z = mix64(z ^ ((unsigned long long)__float_as_uint(lo.z) << 32 | __float_as_uint(hi.x)));
    z = mix64(z ^ ((unsigned long long)__float_as_uint(hi.y) << 32 | __float_as_uint(hi.z)));
    z = mix64(z ^ ((unsigned long long)(uint32_t)ch.x << 32 | (uint32_t)ch.y));
    h ^= z;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) h ^= __shfl_xor_sync(0xffffffffu, h, o);
  if ((threadIdx.x & 31) == 0 && h) atomicXor(out, h);
}

cudaError_t tree_hash(const Node* nodes, uint32_t n_nodes, unsigned long long* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, 8, st);
  if (e != cudaSuccess || n_nodes == 0) return e;
  k_tree_hash<<<std::min<uint32_t>(div_up(n_nodes, 256), 152 * 8), 256, 0, st>>>(nodes, n_nodes, out);
  return cudaGetLastError();
}

}  // namespace bvhgb
