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

// Rays of many requests traced in one launch against a batched build (each request's tree at
// node_base, its triangles at tri_base of the concatenated mesh, child and primitive indices
// local to them).  segs: count + 1 entries on the device, ray_begin ascending, the last entry's
// ray_begin = the total ray count.
struct RaySeg {
  uint32_t ray_begin, node_base, tri_base, n_tris;
};
cudaError_t trace_rays_batched(const Node* nodes, const MeshPtrs& m, const RayPtrs& rays, uint32_t nr,
                               const RaySeg* segs, uint32_t count, const HitOut& out, cudaStream_t st);

// Many float copies in one launch: each descriptor moves n floats from src to dst (either side
// may be host memory the device can address, e.g. page-locked buffers).  The work is cut into
// pieces of kCopyPiece floats; first_piece = the pieces of all earlier descriptors (ascending).
constexpr uint32_t kCopyPiece = 16384;
struct CopyDesc {
  const float* src;
  float* dst;
  uint32_t n;
  uint32_t first_piece;
};
inline uint32_t copy_pieces(uint32_t n) { return (n + kCopyPiece - 1) / kCopyPiece; }
cudaError_t copy_many(const CopyDesc* d_descs, uint32_t count, uint32_t total_pieces, cudaStream_t st);
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
