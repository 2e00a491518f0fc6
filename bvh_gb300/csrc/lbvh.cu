// lbvh.cu -- LBVH construction on sm_103a.
//
// Pipeline (one stream, no host synchronisation):
//   k_bounds      scene AABB of all triangles (reference: kComputeBoundsAndCentroids_nt +
//                 kReduceBounds_Step1/2_nt, src/cuda/lbvh_builder.cu:47-165), also zeroes the
//                 sort scratch the current build uses.
//   k_morton      per-triangle AABB (kept for the leaves), centroid, Morton code
//                 (kComputeMortonCodes_nt :167-181 / kComputeMortonCodes_P, lbvh_plus_builder.cu:276-290)
//                 and the digit histograms of every radix pass.
//   k_onesweep    one kernel per 8-bit digit: stable LSD radix sort with decoupled look-back
//                 (replaces cub::DeviceRadixSort::SortPairs, lbvh_builder.cu:413-438, and
//                 thrust::sort_by_key, lbvh_plus_builder.cu:465).
//   k_emit        bottom-up construction of the Karras tree with boxes in one pass: every
//                 node is completed by the second child to arrive, which also unions the
//                 boxes (reference: kBuildInternalNodes_nt :183-229 + kInitLeafNodes_nt :231-241
//                 + kRefitHierarchy_nt :243-274).  The node ids are exactly Karras's.
#include <algorithm>
#include <cstdio>

#include "emit.cuh"
#include "lbvh.cuh"

namespace bvhgb {

// ---------------------------------------------------------------------------------------
// scratch
// ---------------------------------------------------------------------------------------
int sort_tile() { return kSortThreads * 8; }  // smallest variant tile (8 keys per thread)

ScratchLayout scratch_layout(uint32_t n) {
  ScratchLayout L;
  size_t o = 0;
  L.status = o; o += 1;
  L.ticket = o; o += 1;
  L.epoch = o; o += 1;
  o = (o + 3) & ~size_t(3);
  L.scene = o; o += 8;
  L.ploc = o; o += 20;
  L.partials = o; o += (size_t)kBoundsBlocks * 8;
  o = (o + 3) & ~size_t(3);
  L.zero_begin = o;
  L.counters = o; o += 16;
  L.hist = o; o += (size_t)kMaxPasses * 256;
  L.desc = o;
  // the smallest variant tile gives the most tiles
  size_t tiles = div_up(std::max<uint32_t>(n, 1), (uint32_t)sort_tile());
  o += (size_t)kMaxPasses * tiles * 256;
  L.zero_end = o;
  L.total = o;
  return L;
}

// ---------------------------------------------------------------------------------------
// k_bounds: scene AABB (+ zeroing of the per-build scratch)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void warp_reduce_box(float& a, float& b, float& c, float& d, float& e, float& f) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fminf(b, __shfl_xor_sync(0xffffffffu, b, o));
    c = fminf(c, __shfl_xor_sync(0xffffffffu, c, o));
    d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
    e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    f = fmaxf(f, __shfl_xor_sync(0xffffffffu, f, o));
  }
}

__device__ __forceinline__ void tri_box_acc(float a0, float a1, float a2, float& mn, float& mx) {
  mn = fminf(mn, fminf(a0, fminf(a1, a2)));
  mx = fmaxf(mx, fmaxf(a0, fmaxf(a1, a2)));
}

__global__ void __launch_bounds__(256) k_bounds(MeshPtrs m, uint32_t n, int vec4, uint32_t* __restrict__ scratch,
                                                ScratchLayout L) {
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t gsz = gridDim.x * blockDim.x;
  // zero the current build's histograms, tile counters and look-back descriptors
  {
    uint4* z = reinterpret_cast<uint4*>(scratch + L.zero_begin);
    size_t words4 = (L.zero_end - L.zero_begin) / 4;
    for (size_t w = gtid; w < words4; w += gsz) z[w] = make_uint4(0, 0, 0, 0);
    for (size_t w = L.zero_begin + words4 * 4 + gtid; w < L.zero_end; w += gsz) scratch[w] = 0;
    if (gtid == 0) {
      scratch[L.status] = 0;
      uint32_t e = scratch[L.epoch] + kEpochStride;
      scratch[L.epoch] = e < kEpochStride ? kEpochStride : e;
    }
  }
  float mnx = FLT_MAX, mny = FLT_MAX, mnz = FLT_MAX, mxx = -FLT_MAX, mxy = -FLT_MAX, mxz = -FLT_MAX;
  uint32_t done = 0;
  if (vec4) {
    const uint32_t n4 = n >> 2;
    const float4* p[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k] = reinterpret_cast<const float4*>(m.v[k]);
    for (uint32_t q = gtid; q < n4; q += gsz) {
      float4 x0 = __ldcs(p[0] + q), y0 = __ldcs(p[1] + q), z0 = __ldcs(p[2] + q);
      float4 x1 = __ldcs(p[3] + q), y1 = __ldcs(p[4] + q), z1 = __ldcs(p[5] + q);
      float4 x2 = __ldcs(p[6] + q), y2 = __ldcs(p[7] + q), z2 = __ldcs(p[8] + q);
      tri_box_acc(x0.x, x1.x, x2.x, mnx, mxx); tri_box_acc(x0.y, x1.y, x2.y, mnx, mxx);
      tri_box_acc(x0.z, x1.z, x2.z, mnx, mxx); tri_box_acc(x0.w, x1.w, x2.w, mnx, mxx);
      tri_box_acc(y0.x, y1.x, y2.x, mny, mxy); tri_box_acc(y0.y, y1.y, y2.y, mny, mxy);
      tri_box_acc(y0.z, y1.z, y2.z, mny, mxy); tri_box_acc(y0.w, y1.w, y2.w, mny, mxy);
      tri_box_acc(z0.x, z1.x, z2.x, mnz, mxz); tri_box_acc(z0.y, z1.y, z2.y, mnz, mxz);
      tri_box_acc(z0.z, z1.z, z2.z, mnz, mxz); tri_box_acc(z0.w, z1.w, z2.w, mnz, mxz);
    }
    done = n4 << 2;
  }
  for (uint32_t i = done + gtid; i < n; i += gsz) {
    tri_box_acc(m.v[0][i], m.v[3][i], m.v[6][i], mnx, mxx);
    tri_box_acc(m.v[1][i], m.v[4][i], m.v[7][i], mny, mxy);
    tri_box_acc(m.v[2][i], m.v[5][i], m.v[8][i], mnz, mxz);
  }
  warp_reduce_box(mnx, mny, mnz, mxx, mxy, mxz);
  __shared__ float s_red[8][6];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    s_red[w][0] = mnx; s_red[w][1] = mny; s_red[w][2] = mnz;
    s_red[w][3] = mxx; s_red[w][4] = mxy; s_red[w][5] = mxz;
  }
  __syncthreads();
  float* part = reinterpret_cast<float*>(scratch + L.partials);
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      mnx = fminf(mnx, s_red[k][0]); mny = fminf(mny, s_red[k][1]); mnz = fminf(mnz, s_red[k][2]);
      mxx = fmaxf(mxx, s_red[k][3]); mxy = fmaxf(mxy, s_red[k][4]); mxz = fmaxf(mxz, s_red[k][5]);
    }
    float* pb = part + (size_t)blockIdx.x * 8;
    pb[0] = mnx; pb[1] = mny; pb[2] = mnz; pb[3] = mxx; pb[4] = mxy; pb[5] = mxz;
    __threadfence();
    uint32_t t = atomicAdd(scratch + L.ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  // last block: reduce the partials
  __threadfence();
  mnx = mny = mnz = FLT_MAX;
  mxx = mxy = mxz = -FLT_MAX;
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    const float* pb = part + (size_t)b * 8;
    mnx = fminf(mnx, __ldcg(pb + 0)); mny = fminf(mny, __ldcg(pb + 1)); mnz = fminf(mnz, __ldcg(pb + 2));
    mxx = fmaxf(mxx, __ldcg(pb + 3)); mxy = fmaxf(mxy, __ldcg(pb + 4)); mxz = fmaxf(mxz, __ldcg(pb + 5));
  }
  warp_reduce_box(mnx, mny, mnz, mxx, mxy, mxz);
  __syncthreads();
  if (lane == 0) {
    s_red[w][0] = mnx; s_red[w][1] = mny; s_red[w][2] = mnz;
    s_red[w][3] = mxx; s_red[w][4] = mxy; s_red[w][5] = mxz;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      mnx = fminf(mnx, s_red[k][0]); mny = fminf(mny, s_red[k][1]); mnz = fminf(mnz, s_red[k][2]);
      mxx = fmaxf(mxx, s_red[k][3]); mxy = fmaxf(mxy, s_red[k][4]); mxz = fmaxf(mxz, s_red[k][5]);
    }
    SceneParams* sp = reinterpret_cast<SceneParams*>(scratch + L.scene);
    float ex = mxx - mnx, ey = mxy - mny, ez = mxz - mnz;
    sp->mn[0] = mnx; sp->mn[1] = mny; sp->mn[2] = mnz; sp->mn[3] = 0.f;
    sp->ext[0] = (ex > 1e-6f) ? ex : 1.0f;
    sp->ext[1] = (ey > 1e-6f) ? ey : 1.0f;
    sp->ext[2] = (ez > 1e-6f) ? ez : 1.0f;
    sp->ext[3] = 0.f;
    scratch[L.ticket] = 0;  // ready for the next build
  }
}

// ---------------------------------------------------------------------------------------
// k_morton: AABB + centroid + Morton code + digit histograms of the 4 sort passes
// (32-bit keys: bits 0..31; 64-bit keys: the high 32 bits, from bit BITS-32)
// ---------------------------------------------------------------------------------------
template <int BITS, typename K>
__device__ __forceinline__ K tri_code(float x0, float y0, float z0, float x1, float y1, float z1, float x2,
                                      float y2, float z2, const float* smn, const float* sext, Box& box) {
  float lx = fminf(x0, fminf(x1, x2)), ly = fminf(y0, fminf(y1, y2)), lz = fminf(z0, fminf(z1, z2));
  float hx = fmaxf(x0, fmaxf(x1, x2)), hy = fmaxf(y0, fmaxf(y1, y2)), hz = fmaxf(z0, fmaxf(z1, z2));
  box.lo = make_float4(lx, ly, lz, 0.f);
  box.hi = make_float4(hx, hy, hz, 0.f);
  // centroid = (min + max) * 0.5 (lbvh_builder.cu:65), normalised with IEEE division (:175-177)
  float cx = __fmul_rn(__fadd_rn(lx, hx), 0.5f), cy = __fmul_rn(__fadd_rn(ly, hy), 0.5f),
        cz = __fmul_rn(__fadd_rn(lz, hz), 0.5f);
  float nx = __fdiv_rn(__fsub_rn(cx, smn[0]), sext[0]);
  float ny = __fdiv_rn(__fsub_rn(cy, smn[1]), sext[1]);
  float nz = __fdiv_rn(__fsub_rn(cz, smn[2]), sext[2]);
  return (K)morton_code<BITS>(nx, ny, nz);
}

// Codes of more than 32 bits are written split: keys = the high 32 bits (code >> (BITS - 32)),
// which the radix passes sort, and lows = the rest, in input order.
template <int BITS, typename K>
__global__ void __launch_bounds__(256) k_morton(MeshPtrs m, uint32_t n, int vec4, uint32_t* __restrict__ keys,
                                                uint32_t* __restrict__ lows, Box* __restrict__ boxes,
                                                uint32_t* __restrict__ scratch, ScratchLayout L) {
  constexpr int P = 4;                                   // 8-bit digit passes
  constexpr int S0 = sizeof(K) == 8 ? BITS - 32 : 0;     // first sorted bit
  constexpr unsigned long long kLowMask = (1ull << S0) - 1ull;
  __shared__ uint32_t s_hist[P][256];
  for (int i = threadIdx.x; i < P * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0;
  __shared__ float s_scene[8];
  if (threadIdx.x < 8) s_scene[threadIdx.x] = __ldcg(reinterpret_cast<const float*>(scratch + L.scene) + threadIdx.x);
  __syncthreads();
  const float* smn = s_scene;
  const float* sext = s_scene + 4;
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t gsz = gridDim.x * blockDim.x;
  uint32_t done = 0;
  if (vec4) {
    const uint32_t n4 = n >> 2;
    const float4* p[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k] = reinterpret_cast<const float4*>(m.v[k]);
    for (uint32_t q = gtid; q < n4; q += gsz) {
      float4 x0 = __ldcs(p[0] + q), y0 = __ldcs(p[1] + q), z0 = __ldcs(p[2] + q);
      float4 x1 = __ldcs(p[3] + q), y1 = __ldcs(p[4] + q), z1 = __ldcs(p[5] + q);
      float4 x2 = __ldcs(p[6] + q), y2 = __ldcs(p[7] + q), z2 = __ldcs(p[8] + q);
      Box b[4];
      K c[4];
      c[0] = tri_code<BITS, K>(x0.x, y0.x, z0.x, x1.x, y1.x, z1.x, x2.x, y2.x, z2.x, smn, sext, b[0]);
      c[1] = tri_code<BITS, K>(x0.y, y0.y, z0.y, x1.y, y1.y, z1.y, x2.y, y2.y, z2.y, smn, sext, b[1]);
      c[2] = tri_code<BITS, K>(x0.z, y0.z, z0.z, x1.z, y1.z, z1.z, x2.z, y2.z, z2.z, smn, sext, b[2]);
      c[3] = tri_code<BITS, K>(x0.w, y0.w, z0.w, x1.w, y1.w, z1.w, x2.w, y2.w, z2.w, smn, sext, b[3]);
      reinterpret_cast<uint4*>(keys)[q] = make_uint4((uint32_t)(c[0] >> S0), (uint32_t)(c[1] >> S0),
                                                     (uint32_t)(c[2] >> S0), (uint32_t)(c[3] >> S0));
      if constexpr (sizeof(K) == 8)
        reinterpret_cast<uint4*>(lows)[q] = make_uint4((uint32_t)(c[0] & kLowMask), (uint32_t)(c[1] & kLowMask),
                                                       (uint32_t)(c[2] & kLowMask), (uint32_t)(c[3] & kLowMask));
      float4* bp = reinterpret_cast<float4*>(boxes + 4 * (size_t)q);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        bp[2 * e] = b[e].lo;
        bp[2 * e + 1] = b[e].hi;
#pragma unroll
        for (int p2 = 0; p2 < P; ++p2) atomicAdd(&s_hist[p2][(uint32_t)(c[e] >> (S0 + 8 * p2)) & 255u], 1u);
      }
    }
    done = n4 << 2;
  }
  for (uint32_t i = done + gtid; i < n; i += gsz) {
    Box b;
    K c = tri_code<BITS, K>(m.v[0][i], m.v[1][i], m.v[2][i], m.v[3][i], m.v[4][i], m.v[5][i], m.v[6][i],
                            m.v[7][i], m.v[8][i], smn, sext, b);
    keys[i] = (uint32_t)(c >> S0);
    if constexpr (sizeof(K) == 8) lows[i] = (uint32_t)(c & kLowMask);
    boxes[i] = b;
#pragma unroll
    for (int p2 = 0; p2 < P; ++p2) atomicAdd(&s_hist[p2][(uint32_t)(c >> (S0 + 8 * p2)) & 255u], 1u);
  }
  __syncthreads();
  uint32_t* gh = scratch + L.hist;
  for (int i = threadIdx.x; i < P * 256; i += blockDim.x) {
    uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(gh + i, c);
  }
}

// ---------------------------------------------------------------------------------------
// k_onesweep: one stable LSD pass over an 8-bit digit with decoupled look-back
// ---------------------------------------------------------------------------------------
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr int kMatchWords = 260;  // a warp's peer-mask words: 256 digits, items past n, padding
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValMask = (1u << 30) - 1;

template <int THREADS>
__device__ __forceinline__ unsigned long long block_exclusive_scan_u64(unsigned long long v,
                                                                      unsigned long long* s_warp) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned long long t = lane < THREADS / 32 ? s_warp[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < THREADS / 32) s_warp[lane] = t;  // inclusive warp totals
  }
  __syncthreads();
  unsigned long long before = w ? s_warp[w - 1] : 0ull;
  return before + x - v;
}

// Stable warp-local ranking of the warp's 32 x IPT items (item k of lane l is the warp's item
// 32k + l, so (k, lane) order is input order).  The lanes holding one digit find each other
// through the warp's peer-mask word for that digit: each ORs its lane bit in, and after the
// warp's shared-memory writes are visible each reads the mask (one atomic and one load per
// item, where a ballot per digit bit costs 8 votes and their masking).  Items past n (PARTIAL
// tiles) use a word of their own and are never counted.  The leader of each group (its highest
// lane) clears the word and reserves the group's slots with one shared atomic; the atomics of
// one warp execute in issue order, so earlier items of a digit always get the lower ranks.
template <bool PARTIAL, typename K, int IPT>
__device__ __forceinline__ void warp_rank(const K (&key)[IPT], uint32_t (&rnk)[IPT], int shift, uint32_t wbase,
                                          uint32_t n, uint32_t* wh, uint32_t* wm, uint32_t lane) {
  const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const uint32_t d = (uint32_t)(key[k] >> shift) & 255u;
    const bool valid = !PARTIAL || wbase + (uint32_t)k * 32u + lane < n;
    const uint32_t slot = valid ? d : 256u;
    atomicOr(wm + slot, 1u << lane);
    __syncwarp();
    const uint32_t peers = wm[slot];
    const uint32_t leader = 31u - __clz(peers);
    __syncwarp();  // every lane has read its mask before the leaders clear them
    uint32_t old = 0;
    if (lane == leader) {
      wm[slot] = 0u;
      if (valid) old = atomicAdd(wh + d, (uint32_t)__popc(peers));
    }
    __syncwarp();  // the words are clear before the next item marks them
    rnk[k] = __shfl_sync(0xffffffffu, old, leader) + __popc(peers & lt);
  }
}

template <typename K, int THREADS, int IPT, int W, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_onesweep(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                      K* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                                      int pass, uint32_t* __restrict__ scratch, ScratchLayout L,
                                                      uint32_t tiles) {
  constexpr int BINS = 256, NW = THREADS / 32, TILE = THREADS * IPT;
  static_assert(THREADS == BINS, "one thread per bin");
  extern __shared__ __align__(16) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
  uint32_t* s_whist = s_vals + TILE;          // NW x BINS: warp counts, then each warp's tile offset per bin
  uint32_t* s_gdelta = s_whist + NW * BINS;   // BINS: output position of tile item i is s_gdelta[digit] + i
  unsigned long long* s_scan = reinterpret_cast<unsigned long long*>(s_gdelta + 2 * BINS);  // 32
  uint32_t* s_tile = reinterpret_cast<uint32_t*>(s_scan + 32);
  uint32_t* s_match = s_tile + 4;             // NW x kMatchWords: peer masks per digit (+ items past n)

  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int shift = 8 * pass;  // digit `pass` of the key
  if (tid == 0) *s_tile = atomicAdd(scratch + L.counters + pass, 1u);
  for (int b = tid; b < NW * BINS; b += THREADS) s_whist[b] = 0;
  for (int b = tid; b < NW * kMatchWords; b += THREADS) s_match[b] = 0;
  __syncthreads();
  const uint32_t tile = *s_tile;
  const uint32_t base = tile * (uint32_t)TILE;

  K key[IPT];
  uint32_t val[IPT];
  uint32_t rnk[IPT];
  const uint32_t wbase = base + (uint32_t)w * 32u * IPT;
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    uint32_t idx = wbase + (uint32_t)k * 32u + lane;
    bool ok = idx < n;
    key[k] = ok ? __ldcs(kin + idx) : K(0);
    val[k] = ok ? (vin ? __ldcs(vin + idx) : idx) : 0u;
  }
  uint32_t* wh = s_whist + w * BINS;
  uint32_t* wm = s_match + w * kMatchWords;
  if (base + (uint32_t)TILE <= n) warp_rank<false>(key, rnk, shift, wbase, n, wh, wm, (uint32_t)lane);
  else warp_rank<true>(key, rnk, shift, wbase, n, wh, wm, (uint32_t)lane);
  __syncthreads();
  // per bin: the tile count, its exclusive scan over bins, and each warp's offset in tile order
  const int b = tid;
  uint32_t wc[NW];
  uint32_t cnt = 0;
#pragma unroll
  for (int ww = 0; ww < NW; ++ww) {
    wc[ww] = s_whist[ww * BINS + b];
    cnt += wc[ww];
  }
  const uint32_t ghist = __ldcg(scratch + L.hist + pass * BINS + b);
  unsigned long long packed = ((unsigned long long)ghist << 32) | cnt;
  unsigned long long ex = block_exclusive_scan_u64<THREADS>(packed, s_scan);
  const uint32_t binstart = (uint32_t)ex;         // tile-local start of bin b
  const uint32_t binbase = (uint32_t)(ex >> 32);  // global start of bin b
  // publish this tile's count first so that successors can proceed
  uint32_t* desc = scratch + L.desc + ((size_t)pass * tiles) * BINS;
  st_relaxed(desc + (size_t)tile * BINS + b, (tile == 0 ? kFlagInc : kFlagAgg) | cnt);
  {
    uint32_t run = binstart;
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) {
      s_whist[ww * BINS + b] = run;
      run += wc[ww];
    }
  }
  __syncthreads();  // warp offsets complete
  // local scatter into tile order (independent of the global offsets); frees the key registers
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    uint32_t idx = wbase + (uint32_t)k * 32u + lane;
    if (idx < n) {
      uint32_t d = (uint32_t)(key[k] >> shift) & 255u;
      uint32_t pos = wh[d] + rnk[k];
      s_keys[pos] = key[k];
      s_vals[pos] = val[k];
    }
  }
  // decoupled look-back on bin b, W predecessors per round
  uint32_t excl = 0;
  if (tile != 0) {
    excl = lookback<W, uint32_t>(desc + b, BINS, (int64_t)tile, ~kValMask, kFlagInc, scratch + L.status,
                                 kStatusSortTimeout);
    st_relaxed(desc + (size_t)tile * BINS + b, kFlagInc | (excl + cnt));
  }
  s_gdelta[b] = binbase + excl - binstart;
  __syncthreads();
  const uint32_t len = min((uint32_t)TILE, n - base);
  for (uint32_t i = tid; i < len; i += THREADS) {
    K kk = s_keys[i];
    uint32_t d = (uint32_t)(kk >> shift) & 255u;
    uint32_t dst = s_gdelta[d] + i;
    if (dst < n) {  // always true unless a look-back wait gave up (status already set)
      kout[dst] = kk;
      vout[dst] = s_vals[i];
    }
  }
}

// Onesweep variants (items per thread, look-back window, minimum blocks per SM); the autotuner
// (bvh_autotune) times them and each context keeps the fastest per key width.
struct SortVariant {
  const void* fn;
  int ipt, window, minb;
  size_t smem;
};

template <typename K, int IPT, int W, int MINB>
constexpr SortVariant make_variant() {
  return SortVariant{reinterpret_cast<const void*>(&k_onesweep<K, kSortThreads, IPT, W, MINB>), IPT, W, MINB,
                     (size_t)kSortThreads * IPT * sizeof(K) + (size_t)kSortThreads * IPT * 4 +
                         (size_t)(kSortThreads / 32) * 256 * 4 + 2 * 256 * 4 + 32 * 8 + 16 +
                         (size_t)(kSortThreads / 32) * kMatchWords * 4};
}

static const SortVariant kVariants[] = {
    make_variant<uint32_t, 16, 32, 2>(), make_variant<uint32_t, 16, 16, 3>(), make_variant<uint32_t, 24, 16, 2>(),
    make_variant<uint32_t, 8, 32, 4>(),  make_variant<uint32_t, 24, 32, 2>(),
};
constexpr int kNumVariants = 5;

static const SortVariant& variant(int v) { return kVariants[v < 0 || v >= kNumVariants ? 0 : v]; }

int sort_variant_count() { return kNumVariants; }
int sort_variant_tile(int v) { return kSortThreads * variant(v).ipt; }
// The variant a build uses where nothing chose one, by key count (clustered meshes, GB300): small
// tiles fill the GPU below ~600k keys (8 keys per thread), 16 keys per thread win around 1M, and
// 24 keys with the 16-wide window from ~2M (10M LBVH-63 sort 0.334 vs 0.371 ms with 16 keys).
int default_sort_variant(uint32_t n) { return n < 600000u ? 3 : n < 2000000u ? 0 : 2; }
void sort_variant_describe(int v, int* ipt, int* window, int* minb) {
  const SortVariant& sv = variant(v);
  *ipt = sv.ipt;
  *window = sv.window;
  *minb = sv.minb;
}

// Kernel attributes set once per device, outside any stream capture.
cudaError_t prepare_kernels() {
  for (int v = 0; v < kNumVariants; ++v) {
    const SortVariant& sv = variant(v);
    cudaError_t e = cudaFuncSetAttribute(sv.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sv.smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// `passes` stable 8-bit passes over the 32-bit keys in ws.keys[0] (values: the original index).
static cudaError_t run_sort(Workspace& ws, uint32_t n, int passes, cudaStream_t st, const ScratchLayout& L,
                            int* final_buf) {
  using K = uint32_t;
  const SortVariant& sv = variant(ws.sort_variant);
  const uint32_t tile = (uint32_t)kSortThreads * sv.ipt;
  uint32_t tiles = div_up(n, tile);
  int cur = 0;
  for (int p = 0; p < passes; ++p) {
    const K* kin = reinterpret_cast<const K*>(ws.keys[cur]);
    const uint32_t* vin = p == 0 ? nullptr : ws.vals[cur];
    K* kout = reinterpret_cast<K*>(ws.keys[cur ^ 1]);
    uint32_t* vout = ws.vals[cur ^ 1];
    uint32_t* scratch = ws.scratch;
    ScratchLayout Lc = L;
    void* args[] = {(void*)&kin, (void*)&vin, (void*)&kout, (void*)&vout, (void*)&n, (void*)&p, (void*)&scratch,
                    (void*)&Lc, (void*)&tiles};
    cudaError_t e = cudaLaunchKernel(sv.fn, dim3(tiles), dim3(kSortThreads), args, sv.smem, st);
    if (e != cudaSuccess) return e;
    cur ^= 1;
  }
  *final_buf = cur;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------------------
// autotuning of the sort
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Pseudo-random 32-bit keys with the radix histograms of the 4 passes.
__global__ void __launch_bounds__(256) k_tune_keys(uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist) {
  constexpr int P = 4;
  __shared__ uint32_t s_hist[P][256];
  for (int k = threadIdx.x; k < P * 256; k += blockDim.x) (&s_hist[0][0])[k] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t k = (uint32_t)(mix64(i) >> 32);
    keys[i] = k;
#pragma unroll
    for (int p = 0; p < P; ++p) atomicAdd(&s_hist[p][(k >> (8 * p)) & 255u], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P * 256; k += blockDim.x)
    if ((&s_hist[0][0])[k]) atomicAdd(hist + k, (&s_hist[0][0])[k]);
}

cudaError_t autotune_sort(Workspace& ws, uint32_t n, cudaStream_t st, float* ms) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  if ((e = cudaMemsetAsync(ws.scratch + L.zero_begin, 0, (L.zero_end - L.zero_begin) * 4, st)) != cudaSuccess)
    return e;
  k_tune_keys<<<152 * 8, 256, 0, st>>>(reinterpret_cast<uint32_t*>(ws.keys[0]), n, ws.scratch + L.hist);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = 0;
  for (int v = 0; v < kNumVariants; ++v) {
    ws.sort_variant = v;
    float vbest = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      // tile counters and look-back words start at zero; the histograms stay valid (the keys
      // are a permutation of the same multiset after an even number of passes)
      cudaMemsetAsync(ws.scratch + L.counters, 0, 16 * 4, st);
      cudaMemsetAsync(ws.scratch + L.desc, 0, (L.zero_end - L.desc) * 4, st);
      int fb = 0;
      cudaEventRecord(e0, st);
      e = run_sort(ws, n, 4, st, L, &fb);
      cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) break;
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0 && t < vbest) vbest = t;  // first run warms up
    }
    if (e != cudaSuccess) break;
    ms[v] = vbest;
    if (vbest < ms[best]) best = v;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ws.sort_variant = best;
  return e;
}

// ---------------------------------------------------------------------------------------
// self-test of the bounded device wait
// ---------------------------------------------------------------------------------------
// The sort's look-back waits only on tiles that started before its own, so in a build it always
// ends.  To show that the bound works, one thread of tile 1 looks back at a tile 0 whose
// descriptor is never published, with a short poll limit: it must give up, set the timeout bit
// and return.  Words 0-31: descriptors (zero = unpublished); word 32: the status word.
__device__ uint32_t g_wait_selftest[64];

__global__ void k_wait_selftest(uint32_t limit) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int k = 0; k < 64; ++k) g_wait_selftest[k] = 0;
  __threadfence();
  lookback<1, uint32_t>(g_wait_selftest, 1, 1, ~kValMask, kFlagInc, g_wait_selftest + 32, kStatusSortTimeout, limit);
}

cudaError_t wait_selftest(uint32_t limit, uint32_t* status_out) {
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  k_wait_selftest<<<1, 32, 0, st>>>(limit);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyFromSymbolAsync(status_out, g_wait_selftest, 4, 32 * 4, cudaMemcpyDeviceToHost, st);
  const cudaError_t e2 = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return e != cudaSuccess ? e : e2;
}

// ---------------------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------------------
void workspace_free(Workspace& ws) {
  cudaFree(ws.keys[0]); cudaFree(ws.keys[1]);
  cudaFree(ws.vals[0]); cudaFree(ws.vals[1]);
  cudaFree(ws.boxes); cudaFree(ws.nodes); cudaFree(ws.slots); cudaFree(ws.scratch); cudaFree(ws.delta);
  if (ws.ploc_exec) cudaGraphExecDestroy(ws.ploc_exec);
  if (ws.ploc_seg_exec) cudaGraphExecDestroy(ws.ploc_seg_exec);
  if (ws.aux_stream) cudaStreamDestroy(ws.aux_stream);
  if (ws.ploc_host) cudaFreeHost(ws.ploc_host);
  if (ws.tl_exec) cudaGraphExecDestroy(ws.tl_exec);
  cudaFree(ws.cbox[0]); cudaFree(ws.cbox[1]); cudaFree(ws.cid[0]); cudaFree(ws.cid[1]); cudaFree(ws.nbr);
  cudaFree(ws.mesh_dev);
  cudaFree(ws.bat_offsets); cudaFreeHost(ws.bat_offsets_h); cudaFree(ws.bat_mbox); cudaFree(ws.bat_indices);
  ws = Workspace();
}

// Grows the build buffers to n triangles.  The first-use zeroing (rendezvous slots, scratch) is
// enqueued on `st`, the stream the next build runs on, so that it is ordered before that build's
// kernels even when `st` is a non-blocking stream (a synchronous cudaMemset would run on the
// legacy stream, unordered with respect to non-blocking streams).
cudaError_t epoch_tick(Workspace& ws, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cs);
  if (e != cudaSuccess || cs != cudaStreamCaptureStatusNone) return e;
  if (ws.epoch_builds > 0 && ws.epoch_builds % kEpochCycle == 0 && ws.slots && ws.cap_n)
    e = cudaMemsetAsync(ws.slots, 0, (size_t)ws.cap_n * 8, st);  // no stale tag can match again
  ws.epoch_builds++;
  return e;
}

cudaError_t workspace_reserve(Workspace& ws, uint32_t n, cudaStream_t st) {
  if (n <= ws.cap_n && ws.scratch) return cudaSuccess;
  uint32_t cap = std::max<uint32_t>(n, 1024);
  cudaFree(ws.keys[0]); cudaFree(ws.keys[1]); cudaFree(ws.vals[0]); cudaFree(ws.vals[1]);
  cudaFree(ws.boxes); cudaFree(ws.nodes); cudaFree(ws.slots); cudaFree(ws.scratch); cudaFree(ws.delta);
  ws.keys[0] = ws.keys[1] = nullptr; ws.vals[0] = ws.vals[1] = nullptr;
  ws.boxes = nullptr; ws.nodes = nullptr; ws.slots = nullptr; ws.scratch = nullptr; ws.delta = nullptr;
  ws.cap_n = 0;
  cudaError_t e;
  if ((e = cudaMalloc(&ws.keys[0], (size_t)cap * 8)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.keys[1], (size_t)cap * 8)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.vals[0], (size_t)cap * 4)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.vals[1], (size_t)cap * 4)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.boxes, (size_t)cap * sizeof(Box))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.nodes, (2 * (size_t)cap) * sizeof(Node))) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.slots, (size_t)cap * 8)) != cudaSuccess) return e;
  if ((e = cudaMalloc(&ws.delta, (size_t)cap + 16)) != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(cap);
  if ((e = cudaMalloc(&ws.scratch, L.total * 4)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(ws.slots, 0, (size_t)cap * 8, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(ws.scratch, 0, L.total * 4, st)) != cudaSuccess) return e;
  ws.scratch_words = L.total;
  ws.cap_n = cap;
  return cudaSuccess;
}

static inline bool all_aligned16(const MeshPtrs& m) {
  for (int k = 0; k < 9; ++k)
    if (reinterpret_cast<uintptr_t>(m.v[k]) & 15) return false;
  return true;
}

static inline void rec(StageEvents* evs, int k, cudaStream_t st) {
  if (evs && evs->use) cudaEventRecord(evs->ev[k], st);
}

// Split codes keep their low bits in the node buffer, which emission writes only after the run
// fix-up: [lows by original index: 4n B][64-bit run scratch: 8n B][long-run list: n/6 words],
// 16-byte aligned; at most 13n + 48 bytes of the 96n - 48 the nodes take.
static inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
static inline uint32_t* split_lows(const Workspace& ws) { return reinterpret_cast<uint32_t*>(ws.nodes); }
static inline unsigned long long* split_run_scratch(const Workspace& ws, uint32_t n) {
  return reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(ws.nodes) + align16((size_t)n * 4));
}
static inline uint32_t* split_long_list(const Workspace& ws, uint32_t n) {
  return reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(ws.nodes) + align16((size_t)n * 4) +
                                     align16((size_t)n * 8));
}

template <int BITS, typename K>
static cudaError_t lbvh_prefix(Workspace& ws, const MeshPtrs& m, uint32_t n, cudaStream_t st, StageEvents* evs,
                               const ScratchLayout& L, int* final_buf) {
  uint32_t* lows = sizeof(K) == 8 ? split_lows(ws) : nullptr;
  const int vec4 = all_aligned16(m) && (reinterpret_cast<uintptr_t>(lows) & 15) == 0 ? 1 : 0;
  // zero only the descriptors the current build's passes use (the passes sort 32-bit keys)
  ScratchLayout Lz = L;
  Lz.zero_end = L.desc + (size_t)4 * div_up(std::max<uint32_t>(n, 1),
                                             (uint32_t)sort_variant_tile(ws.sort_variant)) * 256;
  cudaError_t et = epoch_tick(ws, st);
  if (et != cudaSuccess) return et;
  k_bounds<<<kBoundsBlocks, 256, 0, st>>>(m, n, vec4, ws.scratch, Lz);
  rec(evs, 1, st);
  const uint32_t work = vec4 ? div_up(n, 4) : n;
  const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(div_up(work, 256), 152 * 8));
  k_morton<BITS, K><<<grid, 256, 0, st>>>(m, n, vec4, reinterpret_cast<uint32_t*>(ws.keys[0]), lows, ws.boxes,
                                          ws.scratch, L);
  rec(evs, 2, st);
  // 4 passes sort the 32-bit keys: the whole 30-bit code, or the high 32 bits of a 60/63-bit
  // code; then each run of equal high halves is ordered by its low bits.
  cudaError_t e = run_sort(ws, n, 4, st, L, final_buf);
  if (e == cudaSuccess && sizeof(K) == 8) {
    const int fb = *final_buf;
    // the fix-up also writes the delta bytes of the final order
    e = sort_fix_runs_split(reinterpret_cast<const uint32_t*>(ws.keys[fb]), ws.vals[fb], lows, n, BITS - 32,
                            reinterpret_cast<unsigned long long*>(ws.keys[fb ^ 1]), split_run_scratch(ws, n),
                            ws.vals[fb ^ 1], split_long_list(ws, n), ws.scratch + L.counters + kLongRunCounter,
                            ws.delta, st);
  }
  rec(evs, 3, st);
  return e;
}

cudaError_t prefix_sort30(Workspace& ws, const MeshPtrs& m, uint32_t n, cudaStream_t st, StageEvents* evs,
                          uint32_t** sorted_idx) {
  ScratchLayout L = scratch_layout(ws.cap_n);
  int fb = 0;
  cudaError_t e = lbvh_prefix<30, uint32_t>(ws, m, n, st, evs, L, &fb);
  *sorted_idx = ws.vals[fb];
  return e;
}

template <int BITS, bool PARENTS>
static void launch_emit(Workspace& ws, int fb, uint32_t n, const ScratchLayout& L, cudaStream_t st) {
  const uint32_t* keys = reinterpret_cast<const uint32_t*>(ws.keys[fb]);
  const uint32_t* epoch = ws.scratch + L.epoch;
  uint32_t* fcount = ws.scratch + L.counters + kFrontierCounter;
  uint2* frontier = reinterpret_cast<uint2*>(ws.keys[fb ^ 1]);  // the sort's other key buffer, 8 B per position
  // delta bytes: computed by k_emit from the 30-bit keys, written by the run fix-up for 60/63 bits
  k_emit<SegSingle, PARENTS, kEmitTile, BITS == 30><<<div_up(n, kEmitTile), kEmitTile, 0, st>>>(
      ws.delta, keys, ws.vals[fb], ws.boxes, ws.nodes, n, SegSingle{n}, nullptr, frontier, fcount, kEmitMaxSteps);
  if (ws.leaves_ready && !PARENTS) cudaEventRecord(ws.leaves_ready, st);
  k_emit_climb<SegSingle, PARENTS><<<std::min<uint32_t>(div_up(n, 256), 152 * 16), 256, 0, st>>>(
      ws.delta, ws.nodes, ws.slots, epoch, n, SegSingle{n}, frontier, fcount);
}

cudaError_t run_sort_u32(Workspace& ws, uint32_t n, int passes, cudaStream_t st, const ScratchLayout& L,
                         int* final_buf) {
  return run_sort(ws, n, passes, st, L, final_buf);
}

cudaError_t lbvh_build(Workspace& ws, const MeshPtrs& m, uint32_t n, int bits, int treelet_rounds, cudaStream_t st,
                       StageEvents* evs, uint32_t** out_indices, bool host_loops) {
  cudaError_t e = workspace_reserve(ws, n, st);
  if (e != cudaSuccess) return e;
  ScratchLayout L = scratch_layout(ws.cap_n);
  rec(evs, 0, st);
  int fb = 0;
  const bool parents = treelet_rounds > 0;
  if (bits == 30) {
    e = lbvh_prefix<30, uint32_t>(ws, m, n, st, evs, L, &fb);
    if (e != cudaSuccess) return e;
    if (parents) launch_emit<30, true>(ws, fb, n, L, st);
    else launch_emit<30, false>(ws, fb, n, L, st);
  } else if (bits == 60) {
    e = lbvh_prefix<60, unsigned long long>(ws, m, n, st, evs, L, &fb);
    if (e != cudaSuccess) return e;
    if (parents) launch_emit<60, true>(ws, fb, n, L, st);
    else launch_emit<60, false>(ws, fb, n, L, st);
  } else {
    e = lbvh_prefix<63, unsigned long long>(ws, m, n, st, evs, L, &fb);
    if (e != cudaSuccess) return e;
    if (parents) launch_emit<63, true>(ws, fb, n, L, st);
    else launch_emit<63, false>(ws, fb, n, L, st);
  }
  rec(evs, 4, st);
  if (treelet_rounds > 0 && n >= 2) {
    e = treelet_rounds_run(ws, n, treelet_rounds, st, fb, host_loops);
    if (e != cudaSuccess) return e;
  }
  rec(evs, 5, st);
  *out_indices = ws.vals[fb];
  return cudaGetLastError();
}

}  // namespace bvhgb
