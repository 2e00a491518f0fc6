// trace.cu -- closest-hit ray traversal used to measure tree quality.
//
// Reference: traverseBVH (src/render_engine.cu:289-356) with intersectAABB (:194-214),
// intersectTriangle (:220-273) and generateRay (:155-188).  Same visiting order (left child
// first, 128-entry stack that silently drops pushes when full), same counters (a node counts as
// visited before its box test), same closest-hit rule (strict <).  Every float operation is an
// explicitly rounded intrinsic so that the CPU oracle reproduces the results bit for bit.
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

__device__ __forceinline__ float dot3(float a, float b, float c, float x, float y, float z) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a, x), __fmul_rn(b, y)), __fmul_rn(c, z));
}
__device__ __forceinline__ float cross_c(float a, float b, float c, float d) {  // a*b - c*d
  return __fsub_rn(__fmul_rn(a, b), __fmul_rn(c, d));
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

// generateRay (src/render_engine.cu:155-188) per pixel from a host-computed basis.
__device__ __forceinline__ float3 pinhole_dir(const PinholeBasis& c, int x, int y) {
  const float uu = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)x, 0.5f)), (float)c.width), 1.0f), c.half_w);
  const float vv = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)y, 0.5f)), (float)c.height), 1.0f), c.half_h);
  float dx = __fsub_rn(__fadd_rn(c.f[0], __fmul_rn(uu, c.r[0])), __fmul_rn(vv, c.u[0]));
  float dy = __fsub_rn(__fadd_rn(c.f[1], __fmul_rn(uu, c.r[1])), __fmul_rn(vv, c.u[1]));
  float dz = __fsub_rn(__fadd_rn(c.f[2], __fmul_rn(uu, c.r[2])), __fmul_rn(vv, c.u[2]));
  const float len = __fsqrt_rn(dot3(dx, dy, dz, dx, dy, dz));
  if (len < 1e-12f) return make_float3(0.f, 0.f, 0.f);
  const float inv = __fdiv_rn(1.0f, len);
  return make_float3(__fmul_rn(dx, inv), __fmul_rn(dy, inv), __fmul_rn(dz, inv));
}

__global__ void __launch_bounds__(128) k_trace_pinhole(const Node* __restrict__ nodes, int n_nodes, MeshPtrs m,
                                                       uint32_t n_tris, PinholeBasis cam, HitOut out) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (r >= total) return;
  const int x = (int)(r % (uint32_t)cam.width), y = (int)(r / (uint32_t)cam.width);
  const float3 o = make_float3(cam.eye[0], cam.eye[1], cam.eye[2]);
  trace_one(o, pinhole_dir(cam, x, y), nodes, n_nodes, m, n_tris, r, out);
}

__global__ void k_pinhole_rays(PinholeBasis cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (r >= total) return;
  const float3 d = pinhole_dir(cam, (int)(r % (uint32_t)cam.width), (int)(r / (uint32_t)cam.width));
  ox[r] = cam.eye[0]; oy[r] = cam.eye[1]; oz[r] = cam.eye[2];
  dx[r] = d.x; dy[r] = d.y; dz[r] = d.z;
}

cudaError_t trace_rays(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const RayPtrs& rays,
                       uint32_t nr, const HitOut& out, cudaStream_t st) {
  if (nr == 0) return cudaSuccess;
  k_trace<<<div_up(nr, 128), 128, 0, st>>>(nodes, n_nodes, m, n_tris, rays, nr, out);
  return cudaGetLastError();
}

cudaError_t trace_pinhole(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const PinholeBasis& cam,
                          const HitOut& out, cudaStream_t st) {
  uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (total == 0) return cudaSuccess;
  k_trace_pinhole<<<div_up(total, 128), 128, 0, st>>>(nodes, n_nodes, m, n_tris, cam, out);
  return cudaGetLastError();
}

cudaError_t pinhole_rays(const PinholeBasis& cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz,
                         cudaStream_t st) {
  uint32_t total = (uint32_t)cam.width * (uint32_t)cam.height;
  if (total == 0) return cudaSuccess;
  k_pinhole_rays<<<div_up(total, 256), 256, 0, st>>>(cam, ox, oy, oz, dx, dy, dz);
  return cudaGetLastError();
}

}  // namespace bvhgb
