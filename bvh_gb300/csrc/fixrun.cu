// fixrun.cu -- finishes a 64-bit key sort whose radix passes covered only the high 32 bits.
//
// The LBVH with 60/63-bit Morton codes needs the (code, original index) order that a full
// 8-pass LSD radix sort produces (cub::DeviceRadixSort::SortPairs, lbvh_builder.cu:413-438;
// thrust::sort_by_key, lbvh_plus_builder.cu:465).  Here the onesweep passes sort only by
// H = code >> lbits (4 passes, lbits = 31 or 28); within each run of equal H the items are then
// still in original-index order (every pass is stable and the first one numbers the items), so
// ordering each run by (L = code & (2^lbits - 1), position) completes the sort.  On real meshes
// almost every run has length 1, so this costs one read of the keys instead of four more passes.
//
// k_fixrun: one block per tile of 1024 positions.  The block owns the runs that START in its
// tile.  Runs of up to kHalo items are ranked from shared memory (each item's rank is the count
// of smaller (L, position) pairs in its run) and permuted in place; longer runs are sorted by the
// owning block with a block-wide stable LSD over L, through the same positions of the other
// key/value buffer.  Blocks read positions owned by neighbours only for H, which a permutation
// within a run does not change, so the in-place writes cannot disturb them.
#include "lbvh.cuh"

namespace bvhgb {
namespace {

constexpr int kFixThreads = 256;
constexpr int kFixTile = 1024;
constexpr int kHalo = 64;  // runs up to this length are ranked in shared memory
constexpr uint32_t kNone = 0xffffffffu;
constexpr int kSpan = kFixTile + kHalo + 1;  // positions a-1 .. a+T+kHalo-1

// Exclusive prefix over the 256 threads' values (thread t = bin t); s_w holds 8 warp totals.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* s_w) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[w] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int k = 0; k < w; ++k) before += s_w[k];
  __syncthreads();
  return before + x - v;
}

// Stable LSD sort of keys[s, s+m) / vals[s, s+m) by the low `lbits` bits of the key, by the
// calling block alone, ping-ponging through tkeys/tvals at the same positions; an even number
// of 8-bit passes leaves the result in keys/vals.  Items are ranked in chunks of 2048 in their
// current order (warp w takes chunk items w*256 .. w*256+255), so equal digits keep their order
// (a warp's shared atomics execute in issue order).
__device__ void block_sort_run(unsigned long long* keys, uint32_t* vals, unsigned long long* tkeys,
                               uint32_t* tvals, uint32_t s, uint32_t m, int lbits, uint32_t* s_wh,
                               uint32_t* s_off, uint32_t* s_w) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  int passes = (lbits + 7) / 8;
  passes += passes & 1;
  const uint32_t lt = (1u << lane) - 1u;
  for (int p = 0; p < passes; ++p) {
    const unsigned long long* sk = (p & 1) ? tkeys : keys;
    const uint32_t* sv = (p & 1) ? tvals : vals;
    unsigned long long* dk = (p & 1) ? keys : tkeys;
    uint32_t* dv = (p & 1) ? vals : tvals;
    const int sh = 8 * p;
    // digit histogram of the whole run -> global start of each bin
    s_wh[t] = 0;
    __syncthreads();
    for (uint32_t q = t; q < m; q += kFixThreads) atomicAdd(&s_wh[(uint32_t)(sk[s + q] >> sh) & 255u], 1u);
    __syncthreads();
    const uint32_t c0 = s_wh[t];
    __syncthreads();
    s_off[t] = block_excl_scan256(c0, s_w);
    __syncthreads();
    for (uint32_t base = 0; base < m; base += 8 * 256) {
      for (int b = t; b < 8 * 256; b += kFixThreads) s_wh[b] = 0;
      __syncthreads();
      unsigned long long key[8];
      uint32_t val[8], rnk[8], dig[8];
      uint32_t* wh = s_wh + w * 256;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint32_t i = base + (uint32_t)w * 256u + (uint32_t)k * 32u + lane;
        const bool ok = i < m;
        key[k] = ok ? sk[s + i] : 0ull;
        val[k] = ok ? sv[s + i] : 0u;
        dig[k] = ok ? (uint32_t)(key[k] >> sh) & 255u : 256u;
        const uint32_t peers = warp_match_bits<9>(dig[k]);
        const uint32_t leader = 31u - __clz(peers);
        uint32_t old = 0;
        if (lane == leader && dig[k] < 256u) old = atomicAdd(wh + dig[k], (uint32_t)__popc(peers));
        rnk[k] = __shfl_sync(0xffffffffu, old, leader) + __popc(peers & lt);
      }
      __syncthreads();
      // per bin: exclusive prefix over the warps, chunk count
      uint32_t c = 0;
#pragma unroll
      for (int ww = 0; ww < 8; ++ww) {
        const uint32_t x = s_wh[ww * 256 + t];
        s_wh[ww * 256 + t] = c;
        c += x;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (dig[k] < 256u) {
          const uint32_t dst = s_off[dig[k]] + s_wh[w * 256 + dig[k]] + rnk[k];
          dk[s + dst] = key[k];
          dv[s + dst] = val[k];
        }
      }
      __syncthreads();
      s_off[t] += c;
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kFixThreads, 5) k_fixrun(unsigned long long* __restrict__ keys,
                                                        uint32_t* __restrict__ vals,
                                                        unsigned long long* __restrict__ tkeys,
                                                        uint32_t* __restrict__ tvals, uint32_t n, int lbits) {
  constexpr int kPer = (kSpan + kFixThreads - 1) / kFixThreads;  // positions per thread
  __shared__ uint32_t s_h[kSpan];    // H of position q at q - a + 1
  __shared__ uint32_t s_l[kSpan];    // L
  __shared__ uint32_t s_wh[8 * 256];
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_long[kFixTile / kHalo];
  __shared__ uint32_t s_nlong, s_e;

  const int t = threadIdx.x;
  const uint32_t a = blockIdx.x * kFixTile;
  const uint32_t lo = a == 0 ? 0 : a - 1;
  const uint32_t hi = min(n, a + (uint32_t)kFixTile + (uint32_t)kHalo);
  const uint32_t tile_end = min(n, a + (uint32_t)kFixTile);
  const unsigned long long lmask = (1ull << lbits) - 1ull;
  if (t == 0) s_nlong = 0;
  {
    // all of this thread's loads first, then the stores
    unsigned long long k[kPer];
#pragma unroll
    for (int r = 0; r < kPer; ++r) {
      const uint32_t q = lo + t + (uint32_t)r * kFixThreads;
      k[r] = q < hi ? keys[q] : 0ull;
    }
#pragma unroll
    for (int r = 0; r < kPer; ++r) {
      const uint32_t q = lo + t + (uint32_t)r * kFixThreads;
      if (q < hi) {
        s_h[q - a + 1] = (uint32_t)(k[r] >> lbits);
        s_l[q - a + 1] = (uint32_t)(k[r] & lmask);
      }
    }
  }
  __syncthreads();
#define H(q) s_h[(q) - a + 1]
#define L(q) s_l[(q) - a + 1]
  // this thread's positions a + t + 256 r: new position of a moved item (or kNone) and its value
  uint32_t dst[kPer], mv[kPer];
#pragma unroll
  for (int r = 0; r < kPer; ++r) {
    dst[r] = kNone;
    mv[r] = 0;
    const uint32_t q = a + t + (uint32_t)r * kFixThreads;
    if (q >= hi) continue;
    const uint32_t h = H(q);
    const bool prev_same = q > 0 && H(q - 1) == h;
    const bool next_same = q + 1 < hi && H(q + 1) == h;
    // a run of more than kHalo items that starts in this tile goes to the block-wide path
    if (!prev_same && q < tile_end && q + kHalo < n && H(q + kHalo) == h) {
      const uint32_t slot = atomicAdd(&s_nlong, 1u);
      s_long[slot] = q;
      continue;
    }
    if (!prev_same && !next_same) continue;  // a run of one
    // start of q's run, within kHalo steps
    uint32_t s = q;
    while (s > lo && q - s < (uint32_t)kHalo && H(s - 1) == h) --s;
    if (q - s == (uint32_t)kHalo) continue;  // more than kHalo equal items: a long run
    if (s < a || s >= tile_end) continue;    // started in another tile: not ours
    if (s + kHalo < n && H(s + kHalo) == h) continue;  // long run (sorted by the block-wide path)
    uint32_t e = q + 1;
    while (e < hi && H(e) == h) ++e;
    // rank by (L, position) within [s, e)
    const uint32_t l = L(q);
    uint32_t rank = 0;
    for (uint32_t j = s; j < e; ++j) {
      const uint32_t lj = L(j);
      rank += (lj < l) || (lj == l && j < q);
    }
    if (s + rank != q) {
      dst[r] = s + rank;
      mv[r] = vals[q];
    }
  }
  __syncthreads();  // every item of the block's runs has been read
#pragma unroll
  for (int r = 0; r < kPer; ++r) {
    if (dst[r] != kNone) {
      const uint32_t q = a + t + (uint32_t)r * kFixThreads;
      keys[dst[r]] = ((unsigned long long)H(q) << lbits) | L(q);
      vals[dst[r]] = mv[r];
    }
  }
  __syncthreads();
  // long runs starting in this tile, one at a time by the whole block
  const uint32_t nlong = s_nlong;
  for (uint32_t li = 0; li < nlong; ++li) {
    const uint32_t s = s_long[li];
    const uint32_t h = H(s);
    if (t == 0) s_e = n;
    __syncthreads();
    for (uint32_t base = s + kHalo + 1; base < n; base += kFixThreads) {
      const uint32_t q = base + t;
      if (q < n && (uint32_t)(keys[q] >> lbits) != h) atomicMin(&s_e, q);
      __syncthreads();
      const bool found = s_e != n;
      __syncthreads();
      if (found) break;
    }
    block_sort_run(keys, vals, tkeys, tvals, s, s_e - s, lbits, s_wh, s_off, s_w);
    __syncthreads();
  }
#undef H
#undef L
}

}  // namespace

cudaError_t sort_fix_runs(unsigned long long* keys, uint32_t* vals, unsigned long long* tkeys, uint32_t* tvals,
                          uint32_t n, int lbits, cudaStream_t st) {
  if (n < 2) return cudaSuccess;
  k_fixrun<<<div_up(n, (uint32_t)kFixTile), kFixThreads, 0, st>>>(keys, vals, tkeys, tvals, n, lbits);
  return cudaGetLastError();
}

}  // namespace bvhgb
