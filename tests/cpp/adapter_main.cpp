// Builds meshes through the C++ BVHBuilder adapters and prints node checksums (test program).
// Compiled either against the reference's headers (drop-in check) or standalone.
// Argument: a triangle count (a seeded random mesh) or the path of a mesh file (nine float32
// arrays v0x..v2z of n entries each, back to back).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#ifndef BVH_GB300_STANDALONE
#include "evaluator.h"
#endif
#include "bvh_gb300_builder.hpp"

static bool load_mesh(const char* path, TriangleMesh& mesh) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  const long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  const size_t n = (size_t)bytes / 36;
  mesh.resize(n);
  std::vector<float>* arrays[9] = {&mesh.v0x, &mesh.v0y, &mesh.v0z, &mesh.v1x, &mesh.v1y,
                                   &mesh.v1z, &mesh.v2x, &mesh.v2y, &mesh.v2z};
  bool ok = true;
  for (auto* a : arrays) ok = ok && fread(a->data(), 4, n, f) == n;
  fclose(f);
  return ok;
}

int main(int argc, char** argv) {
  TriangleMesh mesh;
  const std::string arg = argc > 1 ? argv[1] : "10000";
  if (arg.find_first_not_of("0123456789") != std::string::npos) {
    if (!load_mesh(arg.c_str(), mesh)) {
      printf("error: cannot read %s\n", arg.c_str());
      return 1;
    }
  } else {
    const size_t n = (size_t)atol(arg.c_str());
    mesh.resize(n);
    std::mt19937 g(1234);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    for (size_t i = 0; i < n; ++i) {
      float x = u(g), y = u(g), z = u(g);
      mesh.v0x[i] = x; mesh.v0y[i] = y; mesh.v0z[i] = z;
      mesh.v1x[i] = x + 0.004f; mesh.v1y[i] = y; mesh.v1z[i] = z;
      mesh.v2x[i] = x; mesh.v2y[i] = y + 0.004f; mesh.v2z[i] = z + 0.002f;
    }
  }
  try {
  Gb300LBVHBuilder lbvh;  // constructors throw when no context can be created (no GPU)
  Gb300LBVHPlusBuilder plus;
  Gb300PLOCBuilder ploc(25);
  BVHBuilder* builders[] = {&lbvh, &plus, &ploc};
  for (BVHBuilder* b : builders) {
    try {
#ifndef BVH_GB300_STANDALONE
      BVHStats st = BVHEvaluator::evaluate(b, mesh);  // the reference's own evaluator, unchanged
      printf("%s nodes=%d leaves=%d sah=%.6f depth=%d\n", b->getName().c_str(), st.nodeCount, st.leafCount,
             st.sahCost, st.maxDepth);
#else
      b->build(mesh);
      const auto& nodes = b->getNodes();
      unsigned long long h = 1469598103934665603ull;
      for (const BVHNode& nd : nodes) {
        unsigned char buf[40];
        memcpy(buf, &nd.bbox.min, 12); memcpy(buf + 12, &nd.bbox.max, 12);
        memcpy(buf + 24, &nd.leftChild, 4); memcpy(buf + 28, &nd.rightChild, 4);
        memset(buf + 32, 0, 8);
        for (int k = 0; k < 32; ++k) h = (h ^ buf[k]) * 1099511628211ull;
      }
      printf("%s nodes=%zu hash=%016llx ms=%.3f\n", b->getName().c_str(), nodes.size(), h, b->getLastBuildTimeMS());
#endif
    } catch (const std::exception& e) {
      printf("%s error: %s\n", b->getName().c_str(), e.what());
      return 1;
    }
  }
  } catch (const std::exception& e) {
    printf("error: %s\n", e.what());
    return 1;
  }
  return 0;
}
