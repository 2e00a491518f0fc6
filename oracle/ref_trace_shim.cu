// ref_trace_shim.cu -- TEST INFRASTRUCTURE (oracle/_ref only; never part of the library).
//
// Compiled by oracle/ref_build.py into oracle/_ref/ref_trace.fatbin together with the reference's
// own src/render_engine.cu, which it includes unmodified from the reference tree (the include path
// points there; nothing of it is copied into this repository), with the reference's default
// (non-Release) nvcc flags.  It exposes two of the reference's __device__ functions as kernels so
// the GPU tests can run them on exactly the rays the library traces:
//   shim_generate_rays -- generateRay (src/render_engine.cu:155-188) for every pixel;
//   shim_traverse      -- traverseBVH (src/render_engine.cu:289-356) on caller-given rays, the
//                         inverse direction formed as generateRay forms it (:181-185).
// Launched by oracle/ref_runner.cu (ref_generate_rays, ref_traverse).
#include "render_engine.cu"

extern "C" __global__ void shim_generate_rays(Camera cam, int width, int height, float* ox, float* oy, float* oz,
                                              float* dx, float* dy, float* dz) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)width * height) return;
  const int x = (int)(i % width), y = (int)(i / width);
  const Ray r = generateRay(cam, x, y, width, height);
  ox[i] = r.origin.x; oy[i] = r.origin.y; oz[i] = r.origin.z;
  dx[i] = r.direction.x; dy[i] = r.direction.y; dz[i] = r.direction.z;
}

// One ray per thread.  prim = -1 on a miss; normal = the closest hit's normal (0 on a miss).
extern "C" __global__ void shim_traverse(const BVHNode* nodes, int num_nodes, TrianglesSoADevice tris,
                                         const float* ox, const float* oy, const float* oz, const float* dx,
                                         const float* dy, const float* dz, int n, float* t, int* prim, int* visits,
                                         int* aabb_tests, int* tri_tests, float* normal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Ray ray;
  ray.origin = float3_cw(ox[i], oy[i], oz[i]);
  const float3_cw d(dx[i], dy[i], dz[i]);
  ray.direction = d;
  ray.invDirection = float3_cw(fabsf(d.x) > EPSILON ? 1.0f / d.x : (d.x >= 0 ? 1e30f : -1e30f),
                               fabsf(d.y) > EPSILON ? 1.0f / d.y : (d.y >= 0 ? 1e30f : -1e30f),
                               fabsf(d.z) > EPSILON ? 1.0f / d.z : (d.z >= 0 ? 1e30f : -1e30f));
  const HitInfo h = traverseBVH(ray, nodes, num_nodes, tris);
  t[i] = h.t;
  prim[i] = h.hit ? (int)h.primIdx : -1;
  visits[i] = h.nodesVisited;
  aabb_tests[i] = h.aabbTests;
  tri_tests[i] = h.triTests;
  normal[3 * (size_t)i + 0] = h.hit ? h.normal.x : 0.0f;
  normal[3 * (size_t)i + 1] = h.hit ? h.normal.y : 0.0f;
  normal[3 * (size_t)i + 2] = h.hit ? h.normal.z : 0.0f;
}
