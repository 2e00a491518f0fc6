// ref_eval_shim.cpp -- C entry points into the reference's own BVHEvaluator (TEST INFRASTRUCTURE).
//
// Compiled together with the reference's src/evaluator.cpp (unmodified, from the reference
// tree) into oracle/_ref/libref_eval.so by oracle/ref_build.py, on machines that have the
// reference sources.  The tests use it to pin the CPU oracle's SAH and depth statistics.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "evaluator.h"

namespace {
// A BVHBuilder that hands out a given tree, so BVHEvaluator::evaluate can score it.
class FixedTree : public BVHBuilder {
 public:
  std::vector<BVHNode> nodes;
  std::vector<uint32_t> idx;
  std::string getName() const override { return "fixed"; }
  void build(const TriangleMesh&) override {}
  const std::vector<BVHNode>& getNodes() const override { return nodes; }
  const std::vector<uint32_t>& getIndices() const override { return idx; }
  float getLastBuildTimeMS() const override { return 0.0f; }
};
}  // namespace

extern "C" {

int ref_sizeof_node(void) { return (int)sizeof(BVHNode); }

// stats: [0] sah, [1] node count, [2] leaf count, [3] max depth, [4] avg leaf depth
int ref_evaluate(const void* nodes48, uint32_t n_nodes, float* stats) {
  FixedTree t;
  t.nodes.resize(n_nodes);
  if (n_nodes) std::memcpy(t.nodes.data(), nodes48, (size_t)n_nodes * sizeof(BVHNode));
  TriangleMesh mesh;
  BVHStats s = BVHEvaluator::evaluate(&t, mesh);
  stats[0] = s.sahCost;
  stats[1] = (float)s.nodeCount;
  stats[2] = (float)s.leafCount;
  stats[3] = (float)s.maxDepth;
  stats[4] = s.avgLeafDepth;
  return 0;
}

}  // extern "C"
