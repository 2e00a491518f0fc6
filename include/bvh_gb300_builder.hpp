// bvh_gb300_builder.hpp -- BVHBuilder adapters over the C ABI (header only).
//
// Gb300LBVHBuilder / Gb300LBVHPlusBuilder / Gb300PLOCBuilder derive from the reference's
// BVHBuilder (include/bvh_builder.h:10-37) and stand in for LBVHBuilderCUDA
// (src/cuda/lbvh_builder.cuh:16-64), LBVHPlusBuilderCUDA (src/cuda/lbvh_plus_builder.cuh:11-61)
// and PLOCBuilderCUDA (src/cuda/ploc_builder.cuh:10-67).  build() uploads the mesh, builds on
// the GPU and downloads BVHNode/indices (the reference's prepareData/runCompute/
// downloadResults); getLastBuildTimeMS() is the device time of the build kernels.
//
// Include the reference's "bvh_builder.h" before this header to derive from its class, or
// define BVH_GB300_STANDALONE to use bvh_gb300_types.hpp.  Link with -lbvh_gb300.
// Errors throw std::runtime_error (the reference's callers catch std::exception).
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh_gb300.h"
#ifdef BVH_GB300_STANDALONE
#include "bvh_gb300_types.hpp"
#endif

static_assert(sizeof(BVHNode) == sizeof(bvh_node), "BVHNode must be 48 bytes");

class Gb300BuilderBase : public BVHBuilder {
 public:
  explicit Gb300BuilderBase(int32_t algo, int device = 0) : params_(bvh_default_params(algo)) {
    bvh_status s = bvh_ctx_create(&ctx_, device);
    if (s != BVH_OK) throw std::runtime_error(std::string("bvh_ctx_create: ") + bvh_status_string(s));
  }
  ~Gb300BuilderBase() override {
    if (ctx_) bvh_ctx_destroy(ctx_);
  }
  Gb300BuilderBase(const Gb300BuilderBase&) = delete;
  Gb300BuilderBase& operator=(const Gb300BuilderBase&) = delete;

  void build(const TriangleMesh& mesh) override {
    const uint32_t n = static_cast<uint32_t>(mesh.size());
    bvh_mesh_soa m{mesh.v0x.data(), mesh.v0y.data(), mesh.v0z.data(), mesh.v1x.data(), mesh.v1y.data(),
                   mesh.v1z.data(), mesh.v2x.data(), mesh.v2y.data(), mesh.v2z.data(), n};
    nodes_.resize(n ? 2 * (size_t)n - 1 : 0);
    indices_.resize(n);
    uint32_t nn = 0;
    bvh_status s = bvh_build_host(ctx_, &m, &params_, nullptr, reinterpret_cast<bvh_node*>(nodes_.data()),
                                  indices_.data(), &nn);
    if (s != BVH_OK) throw std::runtime_error(getName() + ": " + bvh_status_string(s));
    nodes_.resize(nn);
    timing_ = bvh_timing{};
    if (n) bvh_last_timing(ctx_, &timing_);
  }
  const std::vector<BVHNode>& getNodes() const override { return nodes_; }
  const std::vector<uint32_t>& getIndices() const override { return indices_; }
  float getLastBuildTimeMS() const override { return timing_.total_ms; }
  std::string getTimingBreakdown() const override {
    return "  Scene bounds:     " + std::to_string(timing_.bounds_ms) + " ms\n" +
           "  Morton + boxes:   " + std::to_string(timing_.morton_ms) + " ms\n" +
           "  Radix sort:       " + std::to_string(timing_.sort_ms) + " ms\n" +
           "  Hierarchy+refit:  " + std::to_string(timing_.emit_ms) + " ms\n" +
           "  Optimise/cluster: " + std::to_string(timing_.optimize_ms) + " ms";
  }
  bvh_params& params() { return params_; }
  const bvh_timing& timing() const { return timing_; }

 protected:
  bvh_ctx* ctx_ = nullptr;
  bvh_params params_;
  std::vector<BVHNode> nodes_;
  std::vector<uint32_t> indices_;
  bvh_timing timing_{};
};

// LBVHBuilderCUDA ("LBVH", 30-bit Morton); morton_bits 60 or 63 select longer keys.
class Gb300LBVHBuilder : public Gb300BuilderBase {
 public:
  explicit Gb300LBVHBuilder(int morton_bits = 30, int device = 0) : Gb300BuilderBase(BVH_ALGO_LBVH, device) {
    params_.morton_bits = morton_bits;
  }
  std::string getName() const override {
    return params_.morton_bits == 30 ? "LBVH" : "LBVH-" + std::to_string(params_.morton_bits);
  }
};

// LBVHPlusBuilderCUDA ("LBVH+", 60-bit Morton, one treelet pass).
class Gb300LBVHPlusBuilder : public Gb300BuilderBase {
 public:
  explicit Gb300LBVHPlusBuilder(int rounds = 1, int morton_bits = 60, int device = 0)
      : Gb300BuilderBase(BVH_ALGO_LBVH_PLUS, device) {
    params_.treelet_rounds = rounds;
    params_.morton_bits = morton_bits;
  }
  std::string getName() const override { return "LBVH+"; }
};

// PLOCBuilderCUDA(r) ("PLOC CUDA (r=25)").
class Gb300PLOCBuilder : public Gb300BuilderBase {
 public:
  explicit Gb300PLOCBuilder(int r = 25, int device = 0) : Gb300BuilderBase(BVH_ALGO_PLOC, device) {
    params_.ploc_radius = r;
  }
  std::string getName() const override { return "PLOC CUDA (r=" + std::to_string(params_.ploc_radius) + ")"; }
};
