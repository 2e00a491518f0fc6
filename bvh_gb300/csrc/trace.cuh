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

// Camera (include/render_engine.h:24-33) and image size; generateRay's basis
// (src/render_engine.cu:157-167) is derived from it on the device, per ray.
struct PinholeCam {
  float eye[3];
  float look[3];
  float up[3];
  float fov_deg;
  int32_t width, height;
};

struct ShadeIn {
  const float* t;
  const int32_t* prim;
  const int32_t* vis;
};

cudaError_t trace_rays(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const RayPtrs& rays,
                       uint32_t nr, const HitOut& out, cudaStream_t st);
cudaError_t trace_pinhole(const Node* nodes, int n_nodes, const MeshPtrs& m, uint32_t n_tris, const PinholeCam& cam,
                          const HitOut& out, cudaStream_t st);
cudaError_t pinhole_rays(const PinholeCam& cam, float* ox, float* oy, float* oz, float* dx, float* dy, float* dz,
                         cudaStream_t st);
// kRenderKernel's shading of traced pinhole pixels (mode 0 normal, 1 depth, 2 diffuse, 3 visits).
cudaError_t shade_pixels(const PinholeCam& cam, const MeshPtrs& m, uint32_t n_tris, const ShadeIn& in, int mode,
                         float diag, float3 light, float* rgb, cudaStream_t st);
// applyHeatmapColormap on np visit counts with a 256-entry RGB colormap (device); scratch holds
// heatmap_scratch_bytes().  fixed_max <= 0: the 99.9th-percentile normalisation.
size_t heatmap_scratch_bytes();
cudaError_t heatmap(const int32_t* vis, uint32_t np, const float* lut, float fixed_max, void* scratch, float* rgb,
                    float* used_max, cudaStream_t st);
cudaError_t rgb_to_bytes(const float* rgb, uint32_t nv, uint8_t* out, cudaStream_t st);

}  // namespace bvhgb
