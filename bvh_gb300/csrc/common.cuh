// common.cuh -- device types and helpers shared by every kernel of the library.
//
// Layouts match the reference's data model bit for bit:
//   AABB_cw  (include/common.h:29-65)  -> Box  : two 16-byte float4, xyz used, w = 0
//   BVHNode  (include/bvh_node.h:8-31) -> Node : Box + int32 left/right + 8 bytes (aux)
// A leaf has bit 31 of `left` set (primitive index in the low 31 bits) and right = -1.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cfloat>

namespace bvhgb {

struct __align__(16) Box {
  float4 lo;  // min.xyz, w = 0
  float4 hi;  // max.xyz, w = 0
};

struct __align__(16) Node {
  float4 lo;
  float4 hi;
  int32_t left;
  int32_t right;
  int32_t aux0;  // parent index while building (unspecified for users of BVHNode)
  int32_t aux1;
};
static_assert(sizeof(Box) == 32, "AABB_cw is 32 bytes");
static_assert(sizeof(Node) == 48, "BVHNode is 48 bytes");

constexpr uint32_t kLeafBit = 0x80000000u;

// Device status word bits (set by kernels, read by the host after a build).
enum : uint32_t {
  kStatusSortTimeout = 1u << 0,     // onesweep look-back spin gave up
  kStatusClimbTimeout = 1u << 1,    // reserved: bounded waits in bottom-up passes
  kStatusNoProgress = 1u << 2,      // PLOC iteration merged nothing
  kStatusBadInput = 1u << 3,        // index outside its buffer was seen and skipped
  kStatusGridTimeout = 1u << 4,     // a grid-wide barrier of a cooperative kernel gave up
};

// Spin limit for every device-side wait: ~1e7 polls of an L2 line (well over 100 ms),
// after which the waiter records a status bit and carries on instead of hanging.
constexpr uint32_t kSpinLimit = 1u << 24;

__device__ __forceinline__ float fmin_dev(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float fmax_dev(float a, float b) { return fmaxf(a, b); }

__device__ __forceinline__ Box box_empty() {
  Box b;
  b.lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
  b.hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
  return b;
}

// AABB_cw::merge (include/common.h:46-64), device branch: fminf/fmaxf, `a` first.
__device__ __forceinline__ Box box_union(const Box& a, const Box& b) {
  Box r;
  r.lo = make_float4(fminf(a.lo.x, b.lo.x), fminf(a.lo.y, b.lo.y), fminf(a.lo.z, b.lo.z), 0.f);
  r.hi = make_float4(fmaxf(a.hi.x, b.hi.x), fmaxf(a.hi.y, b.hi.y), fmaxf(a.hi.z, b.hi.z), 0.f);
  return r;
}

// AABB_cw::surfaceArea (include/common.h:41-44) exactly as nvcc evaluates the reference's
// expression 2*(dx*dy + dy*dz + dz*dx): 2 * fma(dz, dx, fma(dx, dy, dy*dz)).  Pinned by
// comparing against the reference's own PLOC nearest-neighbour kernel on a GB300.
__device__ __forceinline__ float sa_xyz(float x, float y, float z) {
  return __fmul_rn(2.0f, __fmaf_rn(z, x, __fmaf_rn(x, y, __fmul_rn(y, z))));
}
__device__ __forceinline__ float box_area(const Box& b) {
  return sa_xyz(__fsub_rn(b.hi.x, b.lo.x), __fsub_rn(b.hi.y, b.lo.y), __fsub_rn(b.hi.z, b.lo.z));
}

// expandBits_nt (src/cuda/lbvh_builder.cu:11-17): 10 bits -> every third bit of 30.
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
// expandBits_P (src/cuda/lbvh_plus_builder.cu:20-28): 21 bits -> every third bit of 63.
__device__ __forceinline__ uint64_t expand21(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

// Morton code of a centroid already normalised to the scene box.
//  30 bits: morton3D_nt (src/cuda/lbvh_builder.cu:19-27), x in the most significant slot.
//  60 bits: morton3D_P  (src/cuda/lbvh_plus_builder.cu:30-35), z in the most significant slot.
//  63 bits: the 60-bit layout with 21 bits per axis.
template <int BITS>
__device__ __forceinline__ uint64_t morton_code(float x, float y, float z) {
  if constexpr (BITS == 30) {
    x = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
    y = fminf(fmaxf(y * 1024.0f, 0.0f), 1023.0f);
    z = fminf(fmaxf(z * 1024.0f, 0.0f), 1023.0f);
    return (uint64_t)(expand10((uint32_t)x) * 4u + expand10((uint32_t)y) * 2u + expand10((uint32_t)z));
  } else {
    constexpr float kScale = BITS == 60 ? 1048576.0f : 2097152.0f;
    constexpr float kTop = BITS == 60 ? 1048575.0f : 2097151.0f;
    x = fminf(fmaxf(x * kScale, 0.0f), kTop);
    y = fminf(fmaxf(y * kScale, 0.0f), kTop);
    z = fminf(fmaxf(z * kScale, 0.0f), kTop);
    return (expand21((uint64_t)z) << 2) | (expand21((uint64_t)y) << 1) | expand21((uint64_t)x);
  }
}

// Scene parameters handed from the bounds pass to the Morton pass (device resident).
struct SceneParams {
  float mn[4];
  float ext[4];  // extent, or 1 where the extent is <= 1e-6 (lbvh_builder.cu:175-177)
};

// L2-coherent loads/stores for data exchanged between thread blocks inside one kernel.
__device__ __forceinline__ float4 ld_cg(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ int ld_cg(const int* p) { return __ldcg(p); }
__device__ __forceinline__ void st_cg(float4* p, float4 v) { __stcg(p, v); }
__device__ __forceinline__ void st_cg(int* p, int v) { __stcg(p, v); }

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Lanes of the (full) warp whose low NB bits of d equal this lane's: one ballot per bit, a cost
// independent of how many distinct values the warp holds (match.any's grows with it).
template <int NB>
__device__ __forceinline__ uint32_t warp_match_bits(uint32_t d) {
  uint32_t m = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const uint32_t s = 0u - ((d >> b) & 1u);  // all ones where this lane's bit is set
    const uint32_t bal = __ballot_sync(0xffffffffu, s != 0u);
    m &= ~(bal ^ s);  // the lanes whose bit equals this lane's
  }
  return m;
}

// Decoupled look-back over tiles (Merrill & Garland): descriptor words hold a 2-bit flag and the
// value in one word, so relaxed loads suffice.  Predecessors are read W at a time to shorten the
// dependent chain; an unpublished word (flag 0) is polled again, at most `limit` times.
template <int W, typename T>
__device__ __forceinline__ T lookback(const T* desc, size_t stride, int64_t tile, T flag_mask, T flag_inc,
                                      uint32_t* status, uint32_t status_bit, uint32_t limit = kSpinLimit) {
  T excl = 0;
  int64_t j = tile - 1;
  uint32_t spins = 0;
  while (j >= 0) {
    T v[W];
#pragma unroll
    for (int k = 0; k < W; ++k) v[k] = (j - k >= 0) ? ld_relaxed(desc + (size_t)(j - k) * stride) : flag_inc;
    int k = 0;
    bool done = false;
#pragma unroll
    for (; k < W; ++k) {
      const T fl = v[k] & flag_mask;
      if (fl == 0) break;  // not yet published: poll again from here
      excl += v[k] & ~flag_mask;
      if (fl == flag_inc) { done = true; break; }
    }
    if (done) break;
    if (k < W) {
      j -= k;
      if (++spins > limit) {
        atomicOr(status, status_bit);
        break;
      }
      continue;
    }
    j -= W;
  }
  return excl;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch: arrivals count up in *bar, and the k-th barrier of
// the kernel waits until k * gridDim.x blocks have arrived.  Bounded: past kSpinLimit polls the
// block records kStatusGridTimeout and returns false (every other block then gives up at its
// next wait).  The counter is zeroed before the launch.
__device__ __forceinline__ bool grid_sync(uint32_t* bar, uint32_t target, uint32_t* status, uint32_t* s_ok,
                                          uint32_t limit = kSpinLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    uint32_t ok = 1, spins = 0;
    while (ld_acquire(bar) < target) {
      if (++spins > limit) {
        atomicOr(status, kStatusGridTimeout);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

__host__ __device__ inline uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace bvhgb
