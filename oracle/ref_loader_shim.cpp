// ref_loader_shim.cpp -- C entry point into the reference's own loadOBJ (TEST INFRASTRUCTURE).
//
// Compiled together with the reference's src/loader.cpp (unmodified, from the reference tree)
// into oracle/_ref/libref_loader.so by oracle/ref_build.py, on machines that have the reference
// sources.  The tests compare the library's parallel OBJ reader with it.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

#include "mesh.h"

TriangleMesh loadOBJ(const std::string& filename);

extern "C" {

// Loads `path` with loadOBJ; out[k] receives malloc'd arrays of n floats (v0x..v2z).
// Returns 0, or 1 when loadOBJ threw.
int ref_load_obj(const char* path, float** out, uint32_t* n) {
  try {
    TriangleMesh m = loadOBJ(path);
    const std::vector<float>* v[9] = {&m.v0x, &m.v0y, &m.v0z, &m.v1x, &m.v1y, &m.v1z, &m.v2x, &m.v2y, &m.v2z};
    *n = (uint32_t)m.size();
    for (int k = 0; k < 9; ++k) {
      out[k] = static_cast<float*>(malloc((m.size() ? m.size() : 1) * sizeof(float)));
      if (m.size()) memcpy(out[k], v[k]->data(), m.size() * sizeof(float));
    }
    return 0;
  } catch (const std::exception&) {
    return 1;
  }
}

void ref_free(float** out) {
  for (int k = 0; k < 9; ++k) free(out[k]);
}
}
