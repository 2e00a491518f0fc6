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

__global__ void k_ploc_init(const uint32_t* __restrict__ sidx, const Box* __restrict__ tri_boxes, PlocBufs B, uint32_t n,
                            uint32_t cap) {
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

template <int PER>
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
            const float d = pair_area(xa[m], xb[m], s_lo[jw], s_hi[jw]);
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
              const float d = pair_area(xa[m], xb[m], s_lo[jw], s_hi[jw]);
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
            sD[kk * TILE + p] = pair_area(s_lo[hw], s_hi[hw], s_lo[p + r], s_hi[p + r]);
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

__global__ void __launch_bounds__(kPlocThreads) k_ploc_nn(PlocBufs B, int r) {
  extern __shared__ float4 sw[];
  const uint32_t c = __ldcg(B.ctrl + 0);
  const Box* __restrict__ cbox = (__ldcg(B.ctrl + 3) & 1u) ? B.cbox[1] : B.cbox[0];  // no stack copy of B
  // Once the live clusters no longer fill the grid with 4-per-thread tiles, an iteration lasts
  // one tile's latency: smaller tiles (2 or 1 clusters per thread) then spread it over more
  // blocks.  The result does not depend on the tiling.
  const uint32_t g = gridDim.x * (uint32_t)kPlocThreads;
  if (c > 2u * g) nn_tiles<kNnPer>(B, r, c, cbox, sw);
  else if (c > g) nn_tiles<2>(B, r, c, cbox, sw);
  else nn_tiles<1>(B, r, c, cbox, sw);
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
  bool go = nc > 1;
  if (go && (nc >= c || it >= cap)) {  // no mutual pair anywhere, or the cap: stop and report
    atomicOr(B.status, kStatusNoProgress);
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
__device__ __forceinline__ int ploc_rounds(uint32_t c) {
#pragma unroll
  for (int r = 1; r < kPlocRounds; r <<= 1)
    if (div_up(c, (uint32_t)(kPlocThreads * r)) <= gridDim.x) return r;
  return kPlocRounds;
}

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

template <int R>
__device__ __forceinline__ void scatter_tiles(const PlocBufs& B, uint32_t c, uint32_t next, uint32_t tiles,
                                              const Box* __restrict__ cin, const int32_t* __restrict__ idin,
                                              Box* __restrict__ cout, int32_t* __restrict__ idout,
                                              Node* __restrict__ nodes, unsigned long long* s_w) {
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
          a = make_float4(fminf(a.x, jlo[g].x), fminf(a.y, jlo[g].y), fminf(a.z, jlo[g].z), 0.f);
          b = make_float4(fmaxf(b.x, jhi[g].x), fmaxf(b.y, jhi[g].y), fmaxf(b.z, jhi[g].z), 0.f);
          nid = (int32_t)(next + mpos + __popc(mb[r] & lt));
          float4* np = reinterpret_cast<float4*>(nodes + nid);
          np[0] = a;
          np[1] = b;
          reinterpret_cast<int4*>(np + 2)[0] = make_int4(id[g], jid[g], 0, 0);
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

__global__ void __launch_bounds__(kPlocThreads, 3) k_ploc_scatter(PlocBufs B) {
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
    case 1: scatter_tiles<1>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w); break;
    case 2: scatter_tiles<2>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w); break;
    case 4: scatter_tiles<4>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w); break;
    default: scatter_tiles<kPlocRounds>(B, c, next, tiles, cin, idin, cout, idout, nodes, s_w); break;
  }
}

// End of an iteration, one thread.
template <bool GRAPH>
__global__ void k_ploc_step(PlocBufs B, cudaGraphConditionalHandle handle) {
  if (threadIdx.x == 0 && blockIdx.x == 0) ploc_step<GRAPH>(B, handle);
}

// Move the root (last node) to index 0 and swap every reference to 0 and the root
// (ploc_builder.cu:563-582); skipped when the loop did not converge.  Thread 0 owns 0 and R.
__global__ void k_ploc_root(Node* __restrict__ nodes, uint32_t total, const uint32_t* __restrict__ ctrl) {
  if (__ldcg(ctrl + 0) != 1) return;
  const uint32_t R = total - 1;
  auto fix = [&](int32_t c) -> int32_t {
    if (c < 0) return c;
    if (c == 0) return (int32_t)R;
    if (c == (int32_t)R) return 0;
    return c;
  };
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
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

cudaError_t workspace_reserve_ploc(Workspace& ws, uint32_t n) {
  if (n <= ws.ploc_cap && ws.nbr) return cudaSuccess;
  uint32_t cap = std::max<uint32_t>(n, 1024);
  if (ws.ploc_exec) {
    cudaGraphExecDestroy(ws.ploc_exec);
    ws.ploc_exec = nullptr;
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

static size_t nn_smem(int radius) { return 32 * (kNnTile + 2 * (size_t)radius) + 4 * (size_t)kNnKc * kNnTile; }

// The loop as a graph: WHILE(cond) { nn; merge; step }.  Grids are persistent (sized for n), the
// kernels read the live cluster count from the control words.
static cudaError_t make_loop_graph(Workspace& ws, const PlocBufs& B, uint32_t n, int radius, cudaGraphExec_t* out) {
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
    const uint32_t nn_grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kNnTile), 152 * 3));
    const uint32_t mg_grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kPlocTile), 152 * 8));
    k_ploc_nn<<<nn_grid, kPlocThreads, nn_smem(radius), cs>>>(B, radius);
    k_ploc_count<<<mg_grid, kPlocThreads, 0, cs>>>(B);
    k_ploc_scatter<<<mg_grid, kPlocThreads, 0, cs>>>(B);
    k_ploc_step<true><<<1, 32, 0, cs>>>(B, handle);
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

cudaError_t ploc_build(Workspace& ws, const MeshPtrs& m, uint32_t n, int radius, int max_iter, cudaStream_t st,
                       StageEvents* evs, uint32_t** out_indices, bool host_loop) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  if ((e = workspace_reserve_ploc(ws, n)) != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
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
  if (nn_smem(radius) > 48 * 1024) {
    if ((e = cudaFuncSetAttribute(k_ploc_nn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nn_smem(radius))) !=
        cudaSuccess)
      return e;
  }
  // every iteration that makes progress removes at least one cluster, so n bounds the loop
  const uint32_t cap = max_iter > 0 ? (uint32_t)max_iter : n;
  if (host_loop && !ws.ploc_host && (e = cudaMallocHost(&ws.ploc_host, 64)) != cudaSuccess) return e;
  if (n > 1 && !host_loop) {
    const bool same = ws.ploc_exec && ws.ploc_key_n == n && ws.ploc_key_r == radius && ws.ploc_key_nodes == ws.nodes &&
                      ws.ploc_key_scratch == ws.scratch;
    if (!same) {
      if (ws.ploc_exec) cudaGraphExecDestroy(ws.ploc_exec);
      ws.ploc_exec = nullptr;
      if ((e = make_loop_graph(ws, B, n, radius, &ws.ploc_exec)) != cudaSuccess) return e;
      ws.ploc_key_n = n;
      ws.ploc_key_r = radius;
      ws.ploc_key_nodes = ws.nodes;
      ws.ploc_key_scratch = ws.scratch;
    }
  }
  if (evs && evs->use) cudaEventRecord(evs->ev[0], st);
  uint32_t* sidx = nullptr;
  if ((e = prefix_sort30(ws, m, n, st, evs, &sidx)) != cudaSuccess) return e;
  *out_indices = sidx;
  k_ploc_init<<<div_up(n, 256), 256, 0, st>>>(sidx, ws.boxes, B, n, cap);
  if (evs && evs->use) cudaEventRecord(evs->ev[4], st);
  if (n > 1 && host_loop) {
    const uint32_t nn_grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kNnTile), 152 * 3));
    const uint32_t mg_grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(n, kPlocTile), 152 * 8));
    for (uint32_t it = 0; it < cap; ++it) {
      k_ploc_nn<<<nn_grid, kPlocThreads, nn_smem(radius), st>>>(B, radius);
      k_ploc_count<<<mg_grid, kPlocThreads, 0, st>>>(B);
      k_ploc_scatter<<<mg_grid, kPlocThreads, 0, st>>>(B);
      k_ploc_step<false><<<1, 32, 0, st>>>(B, cudaGraphConditionalHandle{});
      if ((e = cudaMemcpyAsync(ws.ploc_host, B.ctrl + 10, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
      if (!*ws.ploc_host) break;
    }
    k_ploc_root<<<std::min<uint32_t>(div_up(2 * n - 1, 256), 152 * 8), 256, 0, st>>>(ws.nodes, 2 * n - 1, B.ctrl);
  } else if (n > 1) {
    if ((e = cudaGraphLaunch(ws.ploc_exec, st)) != cudaSuccess) return e;
    k_ploc_root<<<std::min<uint32_t>(div_up(2 * n - 1, 256), 152 * 8), 256, 0, st>>>(ws.nodes, 2 * n - 1, B.ctrl);
  }
  if (evs && evs->use) cudaEventRecord(evs->ev[5], st);
  return cudaGetLastError();
}

}  // namespace bvhgb
