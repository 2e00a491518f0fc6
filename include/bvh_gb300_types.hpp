// bvh_gb300_types.hpp -- standalone declarations of the reference's builder interface.
//
// For programs that do not have the reference's headers: the same names, members, layouts
// and virtual interface as float3_cw / AABB_cw (include/common.h:9-65), BVHNode
// (include/bvh_node.h:8-31), TriangleMesh (include/mesh.h:9-50) and BVHBuilder
// (include/bvh_builder.h:10-37), so code written against either compiles against both.
// Do not include together with the reference's headers.
#pragma once
#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>

struct alignas(16) float3_cw {
  float x, y, z;
  float3_cw() : x(0), y(0), z(0) {}
  float3_cw(float a, float b, float c) : x(a), y(b), z(c) {}
};

struct alignas(16) AABB_cw {
  float3_cw min;
  float3_cw max;
  AABB_cw() : min(FLT_MAX, FLT_MAX, FLT_MAX), max(-FLT_MAX, -FLT_MAX, -FLT_MAX) {}
  float surfaceArea() const {
    float dx = max.x - min.x, dy = max.y - min.y, dz = max.z - min.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
  }
};

struct BVHNode {
  AABB_cw bbox;
  int32_t leftChild;   // child index, or primitive | 0x80000000 for a leaf
  int32_t rightChild;  // child index, -1 for a leaf
  bool isLeaf() const { return leftChild < 0; }
  uint32_t getPrimitiveIndex() const { return (uint32_t)leftChild & 0x7FFFFFFFu; }
};

struct TriangleMesh {
  std::vector<float> v0x, v0y, v0z, v1x, v1y, v1z, v2x, v2y, v2z;
  size_t size() const { return v0x.size(); }
  void resize(size_t n) {
    for (auto* v : {&v0x, &v0y, &v0z, &v1x, &v1y, &v1z, &v2x, &v2y, &v2z}) v->resize(n);
  }
};

class BVHBuilder {
 public:
  virtual ~BVHBuilder() = default;
  virtual std::string getName() const = 0;
  virtual void build(const TriangleMesh& mesh) = 0;
  virtual const std::vector<BVHNode>& getNodes() const = 0;
  virtual const std::vector<uint32_t>& getIndices() const = 0;
  virtual float getLastBuildTimeMS() const = 0;
  virtual std::string getTimingBreakdown() const { return ""; }
};
