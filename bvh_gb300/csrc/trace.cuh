// trace.cuh -- traversal launch interface (internal).
#pragma once
#include "lbvh.cuh"

namespace bvhgb {

struct RayPtrs {
  const float* o[3];
  const float* d[3];
};

struct HitOut {
  float* t;
  int32_t* prim;
  int32_t* vis;
  int32_t* aabb;
  int32_t* tri;
};

// Camera basis computed once on the host (generateRay, src/render_engine.cu:157-167).
struct PinholeBasis {
  float eye[3];
  float f[3];
  float r[3];
  float u[3];
  float half_w, half_h;
  int32_t width, height;
};

cudaError_t trace_rays(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const RayPtrs& rays,
                       uint32_t nr, const HitOut& out, cudaStream_t st);
cudaError_t trace_pinhole(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const PinholeBasis& cam,
                          const HitOut& out, cudaStream_t st);
cudaError_t pinhole_rays(const PinholeBasis& cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz,
                         cudaStream_t st);

}  // namespace bvhgb
