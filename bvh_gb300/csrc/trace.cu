// trace.cu -- closest-hit ray traversal used to measure tree quality.
//
// Reference: traverseBVH (src/render_engine.cu:289-356) with intersectAABB (:194-214),
// intersectTriangle (:220-273) and generateRay (:155-188).  Same visiting order (left child
// first, 128-entry stack that silently drops pushes when full), same counters (a node counts as
// visited before its box test), same closest-hit rule (strict <).
//
// Rounding: every float operation is an explicitly rounded intrinsic, in the form nvcc gives the
// reference's expressions under its default -fmad=true.  A two-product difference a*b - c*d is
// fma(a, b, -(c*d)); a three-term dot product (a.x*b.x + a.y*b.y) + a.z*b.z is
// fma(a.z, b.z, fma(a.x, b.x, a.y*b.y)); x + a*b is fma(a, b, x).  (The left product of a sum is
// fused first, and a sum whose left operand is already fused takes the right product into a second
// fma.)  Expressions with a division or subtraction between the multiply and the add
// ((lo - o) * inv, (2(x + 0.5)/w - 1) * half_w) have nothing to contract.  The forms are pinned
// against the reference's own traverseBVH and generateRay on the same rays.  The CPU oracle uses
// the same forms (C fmaf), so it reproduces t, hit ids and counters bit for bit.
#include <algorithm>

#include "lbvh.cuh"
#include "trace.cuh"

namespace bvhgb {

constexpr int kStack = 128;
constexpr float kEps = 1e-6f;

__device__ __forceinline__ bool hit_box(const float3 o, const float3 inv, const float4 lo, const float4 hi, float tmax) {
  float ax = __fmul_rn(__fsub_rn(lo.x, o.x), inv.x), bx = __fmul_rn(__fsub_rn(hi.x, o.x), inv.x);
  float ay = __fmul_rn(__fsub_rn(lo.y, o.y), inv.y), by = __fmul_rn(__fsub_rn(hi.y, o.y), inv.y);
  float az = __fmul_rn(__fsub_rn(lo.z, o.z), inv.z), bz = __fmul_rn(__fsub_rn(hi.z, o.z), inv.z);
  float tenter = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
  float texit = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
  return texit >= fmaxf(tenter, 0.0f) && tenter < tmax;
}

// d_dot (:122-124): (a*x + b*y) + c*z, contracted.
__device__ __forceinline__ float dot3(float a, float b, float c, float x, float y, float z) {
  return __fmaf_rn(c, z, __fmaf_rn(a, x, __fmul_rn(b, y)));
}
// a*b - c*d, contracted (d_cross :114-120 and the edge products of intersectTriangle).
__device__ __forceinline__ float cross_c(float a, float b, float c, float d) {
  return __fmaf_rn(a, b, -__fmul_rn(c, d));
}

__device__ __forceinline__ bool hit_tri(const float3 o, const float3 d, const MeshPtrs& m, uint32_t p, float& t_out) {
  const float v0x = __ldg(m.v[0] + p), v0y = __ldg(m.v[1] + p), v0z = __ldg(m.v[2] + p);
  const float e1x = __fsub_rn(__ldg(m.v[3] + p), v0x), e1y = __fsub_rn(__ldg(m.v[4] + p), v0y),
              e1z = __fsub_rn(__ldg(m.v[5] + p), v0z);
  const float e2x = __fsub_rn(__ldg(m.v[6] + p), v0x), e2y = __fsub_rn(__ldg(m.v[7] + p), v0y),
              e2z = __fsub_rn(__ldg(m.v[8] + p), v0z);
  const float px = cross_c(d.y, e2z, d.z, e2y), py = cross_c(d.z, e2x, d.x, e2z), pz = cross_c(d.x, e2y, d.y, e2x);
  const float det = dot3(e1x, e1y, e1z, px, py, pz);
  if (fabsf(det) < kEps) return false;
  const float inv_det = __fdiv_rn(1.0f, det);
  const float tx = __fsub_rn(o.x, v0x), ty = __fsub_rn(o.y, v0y), tz = __fsub_rn(o.z, v0z);
  const float u = __fmul_rn(dot3(tx, ty, tz, px, py, pz), inv_det);
  if (u < -1e-5f || u > 1.00001f) return false;
  const float qx = cross_c(ty, e1z, tz, e1y), qy = cross_c(tz, e1x, tx, e1z), qz = cross_c(tx, e1y, ty, e1x);
  const float v = __fmul_rn(dot3(d.x, d.y, d.z, qx, qy, qz), inv_det);
  if (v < -1e-5f || __fadd_rn(u, v) > 1.00001f) return false;
  const float t = __fmul_rn(dot3(e2x, e2y, e2z, qx, qy, qz), inv_det);
  if (t < kEps) return false;
  t_out = t;
  return true;
}

__device__ __forceinline__ float inv_dir(float d) {
  return fabsf(d) > kEps ? __fdiv_rn(1.0f, d) : (d >= 0.0f ? 1e30f : -1e30f);
}

__device__ void trace_one(const float3 o, const float3 d, const Node* __restrict__ nodes, int n_nodes,
                          const MeshPtrs& m, uint32_t n_tris, uint32_t r, const HitOut& out) {
  const float3 inv = make_float3(inv_dir(d.x), inv_dir(d.y), inv_dir(d.z));
  float best = 1e30f;
  int32_t prim = -1, vis = 0, at = 0, tt = 0;
  int stack[kStack];
  int sp = 0;
  if (n_nodes > 0) stack[sp++] = 0;
  while (sp > 0) {
    const int x = stack[--sp];
    if (x < 0 || x >= n_nodes) continue;
    const float4* np = reinterpret_cast<const float4*>(nodes + x);
    const float4 lo = __ldg(np), hi = __ldg(np + 1);
    vis++;
    at++;
    if (!hit_box(o, inv, lo, hi, best)) continue;
    const int2 ch = __ldg(reinterpret_cast<const int2*>(np + 2));
    if (ch.x < 0) {
      const uint32_t p = (uint32_t)ch.x & 0x7FFFFFFFu;
      tt++;
      float t;
      if (p < n_tris && hit_tri(o, d, m, p, t)) {
        if (t < best) {
          best = t;
          prim = (int32_t)p;
        }
      }
    } else {
      if (ch.y >= 0 && ch.y < n_nodes && sp < kStack) stack[sp++] = ch.y;
      if (ch.x >= 0 && ch.x < n_nodes && sp < kStack) stack[sp++] = ch.x;
    }
  }
  out.t[r] = best;
  out.prim[r] = prim;
  out.vis[r] = vis;
  out.aabb[r] = at;
  out.tri[r] = tt;
}

__global__ void __launch_bounds__(128) k_trace(const Node* __restrict__ nodes, int n_nodes, MeshPtrs m, uint32_t n_tris,
                                               RayPtrs rays, uint32_t nr, HitOut out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  const float3 o = make_float3(__ldg(rays.o[0] + r), __ldg(rays.o[1] + r), __ldg(rays.o[2] + r));
  const float3 d = make_float3(__ldg(rays.d[0] + r), __ldg(rays.d[1] + r), __ldg(rays.d[2] + r));
  trace_one(o, d, nodes, n_nodes, m, n_tris, r, out);
}

// d_normalize (:130-135): zero below length 1e-12, else each component times 1 / length.
__device__ __forceinline__ float3 normalize3(float x, float y, float z) {
  const float len = __fsqrt_rn(dot3(x, y, z, x, y, z));
  if (len < 1e-12f) return make_float3(0.f, 0.f, 0.f);
  const float inv = __fdiv_rn(1.0f, len);
  return make_float3(__fmul_rn(x, inv), __fmul_rn(y, inv), __fmul_rn(z, inv));
}

// generateRay (:155-188) for pixel (x, y): the camera basis and tan(fov/2) are computed per ray,
// as the reference does, with the device's own tanf.
__device__ __forceinline__ float3 pinhole_dir(const PinholeCam& c, int x, int y) {
  const float3 f = normalize3(__fsub_rn(c.look[0], c.eye[0]), __fsub_rn(c.look[1], c.eye[1]),
                              __fsub_rn(c.look[2], c.eye[2]));
  const float3 rt = normalize3(cross_c(f.y, c.up[2], f.z, c.up[1]), cross_c(f.z, c.up[0], f.x, c.up[2]),
                               cross_c(f.x, c.up[1], f.y, c.up[0]));
  const float3 up = make_float3(cross_c(rt.y, f.z, rt.z, f.y), cross_c(rt.z, f.x, rt.x, f.z),
                                cross_c(rt.x, f.y, rt.y, f.x));
  const float fov = __fdiv_rn(__fmul_rn(c.fov_deg, 3.14159265358979f), 180.0f);
  const float half_h = tanf(__fmul_rn(fov, 0.5f));
  const float half_w = __fmul_rn(half_h, __fdiv_rn((float)c.width, (float)c.height));
  const float uu = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)x, 0.5f)), (float)c.width), 1.0f), half_w);
  const float vv = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)y, 0.5f)), (float)c.height), 1.0f), half_h);
  // forward + u*right - v*up, contracted: fma(-v, up, fma(u, right, forward))
  return normalize3(__fmaf_rn(-vv, up.x, __fmaf_rn(uu, rt.x, f.x)), __fmaf_rn(-vv, up.y, __fmaf_rn(uu, rt.y, f.y)),
                    __fmaf_rn(-vv, up.z, __fmaf_rn(uu, rt.z, f.z)));
}

__global__ void __launch_bounds__(128) k_trace_pinhole(const Node* __restrict__ nodes, int n_nodes, MeshPtrs m,
                                                       uint32_t n_tris, PinholeCam cam, HitOut out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (r >= total) return;
  const int x = (int)(r % (uint32_t)cam.width), y = (int)(r / (uint32_t)cam.width);
  const float3 o = make_float3(cam.eye[0], cam.eye[1], cam.eye[2]);
  trace_one(o, pinhole_dir(cam, x, y), nodes, n_nodes, m, n_tris, r, out);
}

__global__ void k_pinhole_rays(PinholeCam cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (r >= total) return;
  const float3 d = pinhole_dir(cam, (int)(r % (uint32_t)cam.width), (int)(r / (uint32_t)cam.width));
  ox[r] = cam.eye[0]; oy[r] = cam.eye[1]; oz[r] = cam.eye[2];
  dx[r] = d.x; dy[r] = d.y; dz[r] = d.z;
}

// ---------------------------------------------------------------------------------------
// Shading and the traversal-cost heatmap: kRenderKernel's shading (src/render_engine.cu:395-446)
// and the host post-processing of renderImage -- applyHeatmapColormap (:541-595) with
// getTurboColor (:519-535), and savePPM's float-to-byte conversion (:502-507) -- on the device,
// with the same explicitly rounded operations as the traversal above.
// ---------------------------------------------------------------------------------------
constexpr float kBgR = 0.15f, kBgG = 0.15f, kBgB = 0.18f;  // a pixel without a hit (BG_R/G/B)

// Geometric normal of triangle p (intersectTriangle, :267-271): normalise(e1 x e2).
__device__ __forceinline__ float3 tri_normal(const MeshPtrs& m, uint32_t p) {
  const float v0x = __ldg(m.v[0] + p), v0y = __ldg(m.v[1] + p), v0z = __ldg(m.v[2] + p);
  const float e1x = __fsub_rn(__ldg(m.v[3] + p), v0x), e1y = __fsub_rn(__ldg(m.v[4] + p), v0y),
              e1z = __fsub_rn(__ldg(m.v[5] + p), v0z);
  const float e2x = __fsub_rn(__ldg(m.v[6] + p), v0x), e2y = __fsub_rn(__ldg(m.v[7] + p), v0y),
              e2z = __fsub_rn(__ldg(m.v[8] + p), v0z);
  return normalize3(cross_c(e1y, e2z, e1z, e2y), cross_c(e1z, e2x, e1x, e2z), cross_c(e1x, e2y, e1y, e2x));
}

__global__ void __launch_bounds__(256) k_shade(PinholeCam cam, MeshPtrs m, uint32_t n_tris, ShadeIn in, int mode,
                                               float diag, float3 light, float* __restrict__ rgb) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (r >= total) return;
  const int32_t p = in.prim[r];
  float cr, cg, cb;
  if (p < 0 || (uint32_t)p >= n_tris) {
    cr = kBgR; cg = kBgG; cb = kBgB;
  } else if (mode == 0) {  // normal mapped to RGB
    const float3 n = tri_normal(m, (uint32_t)p);
    cr = __fmul_rn(__fadd_rn(n.x, 1.0f), 0.5f);
    cg = __fmul_rn(__fadd_rn(n.y, 1.0f), 0.5f);
    cb = __fmul_rn(__fadd_rn(n.z, 1.0f), 0.5f);
  } else if (mode == 1) {  // depth: closer is brighter
    const float depth = fmaxf(0.0f, fminf(1.0f, __fdiv_rn(in.t[r], diag)));
    cr = cg = cb = __fsub_rn(1.0f, depth);
  } else if (mode == 2) {  // diffuse: directional light + ambient, normal facing the camera
    float3 n = tri_normal(m, (uint32_t)p);
    const float3 d = pinhole_dir(cam, (int)(r % (uint32_t)cam.width), (int)(r / (uint32_t)cam.width));
    if (dot3(n.x, n.y, n.z, d.x, d.y, d.z) > 0.0f) n = make_float3(-n.x, -n.y, -n.z);
    const float diffuse = fmaxf(0.0f, dot3(n.x, n.y, n.z, light.x, light.y, light.z));
    // ambient + diffuse*0.85 and 0.7 + 0.3*|n|, contracted
    const float shade = fminf(1.0f, __fmaf_rn(diffuse, 0.85f, 0.15f));
    cr = __fmul_rn(shade, __fmaf_rn(0.3f, fabsf(n.x), 0.7f));
    cg = __fmul_rn(shade, __fmaf_rn(0.3f, fabsf(n.y), 0.7f));
    cb = __fmul_rn(shade, __fmaf_rn(0.3f, fabsf(n.z), 0.7f));
  } else if (mode == 3) {  // raw node visits (the heatmap colours them afterwards)
    cr = cg = cb = (float)in.vis[r];
  } else {  // unknown mode: magenta
    cr = 1.0f; cg = 0.0f; cb = 1.0f;
  }
  rgb[3 * (size_t)r + 0] = cr;
  rgb[3 * (size_t)r + 1] = cg;
  rgb[3 * (size_t)r + 2] = cb;
}

// The heatmap's normalisation (applyHeatmapColormap, :547-572): the value at index
// min(k - 1, floor(k * 0.999)) of the k nonzero visit counts in ascending order (128 when k = 0),
// at least 1.  Found by a two-level select on the counts' high and low 16 bits: histogram the
// high halves, find the bin holding that rank, histogram the low halves inside it.
// ctl: [0] k, [1] high half of the value, [2] rank inside that bin, [3] value.
__global__ void __launch_bounds__(256) k_heat_hist(const int32_t* __restrict__ vis, uint32_t np, int level,
                                                   uint32_t* __restrict__ hist, const uint32_t* __restrict__ ctl) {
  const uint32_t hi = level == 0 ? 0u : __ldcg(ctl + 1);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const int32_t c = vis[i];
    if (c <= 0) continue;
    const uint32_t u = (uint32_t)c;
    if (level == 0) atomicAdd(hist + (u >> 16), 1u);
    else if ((u >> 16) == hi) atomicAdd(hist + (u & 0xffffu), 1u);
  }
}

// One block of 1024 threads: level 0 counts k, picks the rank and finds its high-half bin;
// level 1 finds the rank inside the low-half histogram.
__global__ void __launch_bounds__(1024) k_heat_find(const uint32_t* __restrict__ hist, int level,
                                                    uint32_t* __restrict__ ctl) {
  constexpr int kBins = 65536, kPer = kBins / 1024;
  __shared__ uint32_t s_sum[1024];
  const int t = threadIdx.x;
  uint32_t sum = 0;
  for (int j = 0; j < kPer; ++j) sum += hist[t * kPer + j];
  s_sum[t] = sum;
  __syncthreads();
  // inclusive scan of the 1024 partial sums (Hillis-Steele)
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t v = t >= o ? s_sum[t - o] : 0u;
    __syncthreads();
    s_sum[t] += v;
    __syncthreads();
  }
  const uint32_t total = s_sum[1023];
  uint32_t rank;
  if (level == 0) {
    if (total == 0) {
      if (t == 0) ctl[0] = 0;
      return;
    }
    const unsigned long long k = total;
    const unsigned long long q = (unsigned long long)((double)k * 0.999);
    rank = (uint32_t)(q < k - 1 ? q : k - 1);
  } else {
    rank = __ldcg(ctl + 2);
  }
  const uint32_t before = t ? s_sum[t - 1] : 0u;
  if (rank >= before && rank < s_sum[t]) {  // exactly one thread holds the rank
    uint32_t cum = before;
    for (int j = 0; j < kPer; ++j) {
      const uint32_t h = hist[t * kPer + j];
      if (rank < cum + h) {
        const uint32_t bin = (uint32_t)(t * kPer + j);
        if (level == 0) {
          ctl[0] = total;
          ctl[1] = bin;
          ctl[2] = rank - cum;
        } else {
          ctl[3] = (__ldcg(ctl + 1) << 16) | bin;
        }
        break;
      }
      cum += h;
    }
  }
}

// getTurboColor + the per-pixel loop of applyHeatmapColormap (:519-535, 574-594): t = count /
// max clamped to [0, 1], linear interpolation between the two nearest of 256 colormap entries;
// a count of 0 gets the background.
__global__ void __launch_bounds__(256) k_heat_color(const int32_t* __restrict__ vis, uint32_t np,
                                                    const float* __restrict__ lut, float fixed_max,
                                                    const uint32_t* __restrict__ ctl, float* __restrict__ rgb,
                                                    float* __restrict__ used_max) {
  float mx = fixed_max;
  if (!(mx > 0.0f)) {
    const uint32_t k = __ldcg(ctl + 0);
    mx = k == 0 ? 128.0f : fmaxf(1.0f, (float)__ldcg(ctl + 3));
  }
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && used_max) *used_max = mx;
  if (i >= np) return;
  const int32_t c = vis[i];
  float cr, cg, cb;
  if (c == 0) {
    cr = kBgR; cg = kBgG; cb = kBgB;
  } else {
    float t = fmaxf(0.0f, fminf(1.0f, __fdiv_rn((float)c, mx)));
    t = fmaxf(0.0f, fminf(1.0f, t));
    const float scaled = __fmul_rn(t, 255.0f);
    const int i0 = (int)scaled;
    const int i1 = min(i0 + 1, 255);
    const float frac = __fsub_rn(scaled, (float)i0);
    const float w0 = __fsub_rn(1.0f, frac);
    cr = __fadd_rn(__fmul_rn(__ldg(lut + 3 * i0 + 0), w0), __fmul_rn(__ldg(lut + 3 * i1 + 0), frac));
    cg = __fadd_rn(__fmul_rn(__ldg(lut + 3 * i0 + 1), w0), __fmul_rn(__ldg(lut + 3 * i1 + 1), frac));
    cb = __fadd_rn(__fmul_rn(__ldg(lut + 3 * i0 + 2), w0), __fmul_rn(__ldg(lut + 3 * i1 + 2), frac));
  }
  rgb[3 * (size_t)i + 0] = cr;
  rgb[3 * (size_t)i + 1] = cg;
  rgb[3 * (size_t)i + 2] = cb;
}

// savePPM's conversion (:502-507): clamp to [0, 1], v * 255 + 0.5, truncated to a byte.
__global__ void __launch_bounds__(256) k_rgb8(const float* __restrict__ rgb, uint32_t nv, uint8_t* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    const float v = fmaxf(0.0f, fminf(1.0f, rgb[i]));
    out[i] = (uint8_t)__fadd_rn(__fmul_rn(v, 255.0f), 0.5f);
  }
}

cudaError_t shade_pixels(const PinholeCam& cam, const MeshPtrs& m, uint32_t n_tris, const ShadeIn& in, int mode,
                         float diag, float3 light, float* rgb, cudaStream_t st) {
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (total == 0) return cudaSuccess;
  k_shade<<<div_up(total, 256), 256, 0, st>>>(cam, m, n_tris, in, mode, diag, light, rgb);
  return cudaGetLastError();
}

size_t heatmap_scratch_bytes() { return (size_t)2 * 65536 * 4 + 16 * 4; }

cudaError_t heatmap(const int32_t* vis, uint32_t np, const float* lut, float fixed_max, void* scratch, float* rgb,
                    float* used_max, cudaStream_t st) {
  if (np == 0) return cudaSuccess;
  uint32_t* h1 = static_cast<uint32_t*>(scratch);
  uint32_t* h2 = h1 + 65536;
  uint32_t* ctl = h2 + 65536;
  cudaError_t e;
  if (!(fixed_max > 0.0f)) {
    if ((e = cudaMemsetAsync(scratch, 0, heatmap_scratch_bytes(), st)) != cudaSuccess) return e;
    const uint32_t grid = std::min<uint32_t>(div_up(np, 256), 152 * 8);
    k_heat_hist<<<grid, 256, 0, st>>>(vis, np, 0, h1, ctl);
    k_heat_find<<<1, 1024, 0, st>>>(h1, 0, ctl);
    k_heat_hist<<<grid, 256, 0, st>>>(vis, np, 1, h2, ctl);
    k_heat_find<<<1, 1024, 0, st>>>(h2, 1, ctl);
  }
  k_heat_color<<<div_up(np, 256), 256, 0, st>>>(vis, np, lut, fixed_max, ctl, rgb, used_max);
  return cudaGetLastError();
}

cudaError_t rgb_to_bytes(const float* rgb, uint32_t nv, uint8_t* out, cudaStream_t st) {
  if (nv == 0) return cudaSuccess;
  k_rgb8<<<std::min<uint32_t>(div_up(nv, 256), 152 * 16), 256, 0, st>>>(rgb, nv, out);
  return cudaGetLastError();
}

cudaError_t trace_rays(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const RayPtrs& rays,
                       uint32_t nr, const HitOut& out, cudaStream_t st) {
  if (nr == 0) return cudaSuccess;
  k_trace<<<div_up(nr, 128), 128, 0, st>>>(nodes, n_nodes, m, n_tris, rays, nr, out);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) k_trace_seg(const Node* __restrict__ nodes, MeshPtrs m, RayPtrs rays,
                                                   uint32_t nr, const RaySeg* __restrict__ segs, uint32_t count,
                                                   HitOut out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nr) return;
  uint32_t lo = 0, hi = count;  // the last segment whose first ray is <= r
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&segs[mid].ray_begin) <= r) lo = mid;
    else hi = mid;
  }
  const RaySeg g = segs[lo];
  MeshPtrs mm;
#pragma unroll
  for (int k = 0; k < 9; ++k) mm.v[k] = m.v[k] + g.tri_base;
  const float3 o = make_float3(__ldg(rays.o[0] + r), __ldg(rays.o[1] + r), __ldg(rays.o[2] + r));
  const float3 d = make_float3(__ldg(rays.d[0] + r), __ldg(rays.d[1] + r), __ldg(rays.d[2] + r));
  trace_one(o, d, nodes + g.node_base, g.n_tris ? (int)(2 * g.n_tris - 1) : 0, mm, g.n_tris, r, out);
}

cudaError_t trace_rays_batched(const Node* nodes, const MeshPtrs& m, const RayPtrs& rays, uint32_t nr,
                               const RaySeg* segs, uint32_t count, const HitOut& out, cudaStream_t st) {
  if (nr == 0 || count == 0) return cudaSuccess;
  k_trace_seg<<<div_up(nr, 128), 128, 0, st>>>(nodes, m, rays, nr, segs, count, out);
  return cudaGetLastError();
}

// One piece (64 KB) per block iteration; 16-byte accesses where both sides allow.
__global__ void __launch_bounds__(256) k_copy_many(const CopyDesc* __restrict__ descs, uint32_t count,
                                                   uint32_t total_pieces) {
  for (uint32_t q = blockIdx.x; q < total_pieces; q += gridDim.x) {
    uint32_t lo = 0, hi = count;  // the last descriptor whose first piece is <= q
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(&descs[mid].first_piece) <= q) lo = mid;
      else hi = mid;
    }
    const CopyDesc c = descs[lo];
    const uint32_t b = (q - c.first_piece) * kCopyPiece;
    if (b >= c.n) continue;
    const uint32_t len = min(c.n - b, kCopyPiece);
    const float* src = c.src + b;
    float* dst = c.dst + b;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
      const uint32_t n4 = len >> 2;
      for (uint32_t i = threadIdx.x; i < n4; i += blockDim.x)
        reinterpret_cast<float4*>(dst)[i] = reinterpret_cast<const float4*>(src)[i];
      for (uint32_t i = (n4 << 2) + threadIdx.x; i < len; i += blockDim.x) dst[i] = src[i];
    } else {
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) dst[i] = src[i];
    }
  }
}

cudaError_t copy_many(const CopyDesc* d_descs, uint32_t count, uint32_t total_pieces, cudaStream_t st) {
  if (count == 0 || total_pieces == 0) return cudaSuccess;
  k_copy_many<<<std::min<uint32_t>(total_pieces, 152 * 8), 256, 0, st>>>(d_descs, count, total_pieces);
  return cudaGetLastError();
}

cudaError_t trace_pinhole(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const PinholeCam& cam,
                          const HitOut& out, cudaStream_t st) {
  uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (total == 0) return cudaSuccess;
  k_trace_pinhole<<<div_up(total, 128), 128, 0, st>>>(nodes, n_nodes, m, n_tris, cam, out);
  return cudaGetLastError();
}

cudaError_t pinhole_rays(const PinholeCam& cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz,
                         cudaStream_t st) {
  uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (total == 0) return cudaSuccess;
  k_pinhole_rays<<<div_up(total, 256), 256, 0, st>>>(cam, ox, oy, oz, dx, dy, dz);
  return cudaGetLastError();
}

}  // namespace bvhgb
