// fixrun.cu -- finishes a sort of 60/63-bit codes (and of the batched path's mesh-prefixed
// keys) whose radix passes covered only the high 32 bits.
//
// The LBVH with 60/63-bit Morton codes needs the (code, original index) order that a full
// 8-pass LSD radix sort produces (cub::DeviceRadixSort::SortPairs, lbvh_builder.cu:413-438;
// thrust::sort_by_key, lbvh_plus_builder.cu:465).  Here the codes are held split: the onesweep
// passes sort (H = code >> lbits, original index) pairs, and L = code & (2^lbits - 1) stays in
// input order.  Within each run of equal H the items are then still in original-index order
// (every pass is stable and the first one numbers the items), so ordering each run by
// (L, position) completes the sort.  On real meshes most runs have length 1 or 2, so this costs
// one read of the sorted halves instead of four more passes.
//
// k_fixrun_split_short: one thread per 4 consecutive positions, with the next thread's 4 (from
// the adjacent lane) as an 8-position window.  A thread owns the runs that START in its 4
// positions (a run's first position differs from its predecessor).  A run that ends inside the
// window is ordered in registers by (L, position) -- a pair by one compare, a longer run by an
// 8-input sorting network -- and only its values move; a longer one is appended to a list, which
// k_fixrun_split_long ranks by counting in shared memory (up to 1024 items) or sorts with a
// block-wide stable LSD over L through idle buffers.  Other threads read positions of a run only
// for H, which a permutation within the run does not change.
#include "lbvh.cuh"

namespace bvhgb {
namespace {

constexpr int kFixThreads = 256;
constexpr int kRankMax = 1024;  // listed runs up to this length are ranked by counting

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

// Ascending sort of 8 (key, value) pairs in registers: Batcher's odd-even merge network,
// 19 compare-exchanges.
__device__ __forceinline__ void cx(unsigned long long& ka, uint32_t& va, unsigned long long& kb, uint32_t& vb) {
  const bool sw = ka > kb;
  const unsigned long long k0 = sw ? kb : ka, k1 = sw ? ka : kb;
  const uint32_t v0 = sw ? vb : va, v1 = sw ? va : vb;
  ka = k0;
  kb = k1;
  va = v0;
  vb = v1;
}
__device__ __forceinline__ void sort8(unsigned long long (&k)[8], uint32_t (&v)[8]) {
  cx(k[0], v[0], k[1], v[1]); cx(k[2], v[2], k[3], v[3]); cx(k[4], v[4], k[5], v[5]); cx(k[6], v[6], k[7], v[7]);
  cx(k[0], v[0], k[2], v[2]); cx(k[1], v[1], k[3], v[3]); cx(k[4], v[4], k[6], v[6]); cx(k[5], v[5], k[7], v[7]);
  cx(k[1], v[1], k[2], v[2]); cx(k[5], v[5], k[6], v[6]);
  cx(k[0], v[0], k[4], v[4]); cx(k[1], v[1], k[5], v[5]); cx(k[2], v[2], k[6], v[6]); cx(k[3], v[3], k[7], v[7]);
  cx(k[2], v[2], k[4], v[4]); cx(k[3], v[3], k[5], v[5]);
  cx(k[1], v[1], k[2], v[2]); cx(k[3], v[3], k[4], v[4]); cx(k[5], v[5], k[6], v[6]);
}

// delta(k, k+1) + 1 of codes held split (the value of the delta pass on whole 64-bit codes:
// clz of their XOR, or 64 + clz of the 64-bit XOR of the indices for equal codes): neighbours
// whose high halves differ, and neighbours inside a run (equal high halves).
__device__ __forceinline__ uint8_t delta_hi(uint32_t a, uint32_t b, int lbits) {
  return (uint8_t)(__clz(a ^ b) + 32 - lbits + 1);
}
__device__ __forceinline__ uint8_t delta_lo(uint32_t la, uint32_t lb, uint32_t va, uint32_t vb) {
  return (uint8_t)((la != lb ? 32 + __clz(la ^ lb) : 96 + __clz(va ^ vb)) + 1);
}

// H = hkeys[position] (sorted), L = lows[original index]; only the values of a run move.  With
// DELTA the kernel also writes D[k] = delta(k, k+1) + 1 (of the final order) for every k whose
// high half differs from the next one's, and for the inner positions of the runs it orders.
template <bool DELTA>
__global__ void __launch_bounds__(256, 4) k_fixrun_split_short(const uint32_t* __restrict__ hkeys,
                                                            uint32_t* __restrict__ vals,
                                                            const uint32_t* __restrict__ lows, uint32_t n, int lbits,
                                                            uint8_t* __restrict__ D, uint32_t* __restrict__ long_list,
                                                            uint32_t* __restrict__ long_count) {
  constexpr unsigned long long kNoH = ~0ull;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t p0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4u;
  unsigned long long hw[8];
  uint32_t v[8];
  // one round trip: this thread's 4 keys and values; lane 31 also the next thread's 4 (the
  // window's other half comes from the next lane), lane 0 the key before
  unsigned long long edge_h[4] = {kNoH, kNoH, kNoH, kNoH};
  uint32_t edge_v[4] = {0u, 0u, 0u, 0u};
  unsigned long long hprev = kNoH;
  if (lane == 31) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (p0 + 4 + j < n) {
        edge_h[j] = hkeys[p0 + 4 + j];
        edge_v[j] = vals[p0 + 4 + j];
      }
  }
  if (lane == 0 && p0 > 0 && p0 - 1 < n) hprev = hkeys[p0 - 1];
  if (p0 + 4 <= n) {
    const uint4 a = *reinterpret_cast<const uint4*>(hkeys + p0);
    const uint4 c = *reinterpret_cast<const uint4*>(vals + p0);
    hw[0] = a.x;
    hw[1] = a.y;
    hw[2] = a.z;
    hw[3] = a.w;
    v[0] = c.x;
    v[1] = c.y;
    v[2] = c.z;
    v[3] = c.w;
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      hw[j] = p0 + j < n ? (unsigned long long)hkeys[p0 + j] : kNoH;
      v[j] = p0 + j < n ? vals[p0 + j] : 0u;
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    hw[4 + j] = __shfl_down_sync(0xffffffffu, hw[j], 1);
    v[4 + j] = __shfl_down_sync(0xffffffffu, v[j], 1);
  }
  if (lane == 31) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      hw[4 + j] = edge_h[j];
      v[4 + j] = edge_v[j];
    }
  }
  {
    const unsigned long long up = __shfl_up_sync(0xffffffffu, hw[3], 1);
    if (lane != 0) hprev = up;
  }
  if (DELTA) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (p0 + j + 1 < n && hw[j] != hw[j + 1]) D[p0 + j] = delta_hi((uint32_t)hw[j], (uint32_t)hw[j + 1], lbits);
  }
  // runs of 2+ equal high halves that start in this thread's positions: their lengths in the
  // window (a run reaching the window's end may be longer: checked against position p0 + 8)
  int rlen[4];
  uint32_t need = 0;  // window slots whose low halves the runs read
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const unsigned long long hp = j == 0 ? hprev : hw[j - 1];
    rlen[j] = 0;
    if (hw[j] == kNoH || hw[j] == hp || hw[j] != hw[j + 1]) continue;  // not the start of a run of 2+
    int m = 2;
#pragma unroll
    for (int q = j + 2; q < 8; ++q) m += (m == q - j && hw[q] == hw[j]) ? 1 : 0;
    rlen[j] = m;
    need |= ((1u << m) - 1u) << j;
  }
  const bool at_end = ((need >> 7) & 1u) && p0 + 8 < n;
  const unsigned long long h8 = at_end ? (unsigned long long)hkeys[p0 + 8] : kNoH;
  // all needed low halves in one batch, before any store of this thread
  uint32_t lw[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) lw[i] = ((need >> i) & 1u) ? __ldg(lows + v[i]) : 0u;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int m = rlen[j];
    if (m == 0) continue;
    const uint32_t s = p0 + j;
    if (j + m == 8 && p0 + 8 < n && h8 == hw[j]) {
      long_list[atomicAdd(long_count, 1u)] = s;
      continue;
    }
    if (m == 2) {  // the common case: swap when out of order
      const uint32_t la = lw[j], lb = lw[j + 1];
      if (la > lb) {
        vals[s] = v[j + 1];
        vals[s + 1] = v[j];
      }
      if (DELTA) D[s] = delta_lo(la, lb, v[j], v[j + 1]);
      continue;
    }
    // a run of 3 or more inside the window: an 8-input sorting network over (L, slot) puts its
    // items in order (slots outside the run sort last); position j + r takes the r-th item
    unsigned long long sk[8];
    uint32_t sv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      sk[i] = (i >= j && i < j + m) ? ((unsigned long long)lw[i] << 3) | (unsigned)i : ~0ull;
      sv[i] = v[i];
    }
    sort8(sk, sv);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (r < m) {
        if ((int)(sk[r] & 7ull) != j + r) vals[p0 + j + r] = sv[r];
        if (DELTA && r + 1 < m)
          D[p0 + j + r] = delta_lo((uint32_t)(sk[r] >> 3), (uint32_t)(sk[r + 1] >> 3), sv[r], sv[r + 1]);
      }
    }
  }
}

// One block per listed run of split codes: find its end; up to kRankMax items are ranked by
// counting, longer runs are sorted block-wide with their low bits staged in scratch_a.
template <bool DELTA>
__global__ void __launch_bounds__(kFixThreads) k_fixrun_split_long(const uint32_t* __restrict__ hkeys,
                                                               uint32_t* __restrict__ vals,
                                                               const uint32_t* __restrict__ lows, uint32_t n,
                                                               int lbits, unsigned long long* __restrict__ scratch_a,
                                                               unsigned long long* __restrict__ scratch_b,
                                                               uint32_t* __restrict__ tvals, uint8_t* __restrict__ D,
                                                               const uint32_t* __restrict__ long_list,
                                                               const uint32_t* __restrict__ long_count) {
  static_assert(kRankMax <= 1024, "sorted low bits share s_wh with the unsorted ones");
  __shared__ uint32_t s_wh[8 * 256];  // [0, kRankMax): L in run order; [1024, 1024 + kRankMax): L by rank
  __shared__ uint32_t s_sv[kRankMax];  // values by rank
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_w[8];
  __shared__ uint32_t s_e;
  const uint32_t count = __ldcg(long_count);
  const int t = threadIdx.x;
  for (uint32_t li = blockIdx.x; li < count; li += gridDim.x) {
    const uint32_t s = __ldcg(long_list + li);
    const uint32_t h = hkeys[s];
    if (t == 0) s_e = n;
    __syncthreads();
    for (uint32_t base = s + 1; base < n; base += kFixThreads) {
      const uint32_t q = base + t;
      if (q < n && hkeys[q] != h) atomicMin(&s_e, q);
      __syncthreads();
      const bool found = s_e != n;
      __syncthreads();
      if (found) break;
    }
    const uint32_t m = s_e - s;
    if (m <= kRankMax) {
      for (uint32_t q = t; q < m; q += kFixThreads) s_wh[q] = __ldg(lows + vals[s + q]);
      __syncthreads();
      uint32_t vq[kRankMax / kFixThreads], rq[kRankMax / kFixThreads];
#pragma unroll
      for (int r = 0; r < kRankMax / kFixThreads; ++r) {
        const uint32_t q = t + (uint32_t)r * kFixThreads;
        if (q < m) {
          const uint32_t lq = s_wh[q];
          uint32_t rank = 0;
          for (uint32_t x = 0; x < m; ++x) {
            const uint32_t lx = s_wh[x];
            rank += (lx < lq) || (lx == lq && x < q);
          }
          vq[r] = vals[s + q];
          rq[r] = rank;
        }
      }
      __syncthreads();  // every value of the run is read before any is written
#pragma unroll
      for (int r = 0; r < kRankMax / kFixThreads; ++r) {
        const uint32_t q = t + (uint32_t)r * kFixThreads;
        if (q < m) {
          if (rq[r] != q) vals[s + rq[r]] = vq[r];
          if (DELTA) {
            s_wh[1024 + rq[r]] = s_wh[q];
            s_sv[rq[r]] = vq[r];
          }
        }
      }
      if (DELTA) {
        __syncthreads();
        for (uint32_t q = t; q + 1 < m; q += kFixThreads)
          D[s + q] = delta_lo(s_wh[1024 + q], s_wh[1024 + q + 1], s_sv[q], s_sv[q + 1]);
      }
    } else {
      for (uint32_t q = t; q < m; q += kFixThreads) scratch_a[s + q] = __ldg(lows + vals[s + q]);
      block_sort_run(scratch_a, vals, scratch_b, tvals, s, m, lbits, s_wh, s_off, s_w);
      if (DELTA) {
        for (uint32_t q = t; q + 1 < m; q += kFixThreads)
          D[s + q] = delta_lo((uint32_t)scratch_a[s + q], (uint32_t)scratch_a[s + q + 1], vals[s + q], vals[s + q + 1]);
      }
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t sort_fix_runs_split(const uint32_t* hkeys, uint32_t* vals, const uint32_t* lows, uint32_t n, int lbits,
                                unsigned long long* scratch_a, unsigned long long* scratch_b, uint32_t* tvals,
                                uint32_t* long_list, uint32_t* long_count, uint8_t* D, cudaStream_t st) {
  if (n < 2) return cudaSuccess;
  const uint32_t grid = div_up(div_up(n, 4u), 256u);
  if (D) {
    k_fixrun_split_short<true><<<grid, 256, 0, st>>>(hkeys, vals, lows, n, lbits, D, long_list, long_count);
    k_fixrun_split_long<true><<<152, kFixThreads, 0, st>>>(hkeys, vals, lows, n, lbits, scratch_a, scratch_b, tvals,
                                                           D, long_list, long_count);
  } else {
    k_fixrun_split_short<false><<<grid, 256, 0, st>>>(hkeys, vals, lows, n, lbits, D, long_list, long_count);
    k_fixrun_split_long<false><<<152, kFixThreads, 0, st>>>(hkeys, vals, lows, n, lbits, scratch_a, scratch_b, tvals,
                                                            D, long_list, long_count);
  }
  return cudaGetLastError();
}

}  // namespace bvhgb
