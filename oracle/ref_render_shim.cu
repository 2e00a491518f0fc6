// ref_render_shim.cu -- TEST INFRASTRUCTURE (oracle/_ref only; never part of the library).
//
// Compiled by oracle/ref_build.py together with the reference's own src/render_engine.cu, which it
// includes unmodified from the reference tree (the include path points there; nothing of it is
// copied into this repository).  It exports the renderer's host post-processing -- the heatmap
// normalisation and colormap (applyHeatmapColormap with getTurboColor, src/render_engine.cu:519-595),
// the PPM byte conversion (savePPM, :490-511) and the colormap table (kTurboColormap, :43) -- so
// the CPU tests can pin the oracle's restatements against the reference itself.
#include "render_engine.cu"

extern "C" {

// The reference's 256 x 3 colormap, row-major.
void ref_turbo_table(float* out) {
  for (int i = 0; i < 256; ++i)
    for (int c = 0; c < 3; ++c) out[3 * i + c] = kTurboColormap[i][c];
}

// applyHeatmapColormap over width x height node-visit counts into rgb (3 floats per pixel).
void ref_apply_heatmap(float* rgb, const int* counts, int width, int height, float fixed_max) {
  applyHeatmapColormap(rgb, counts, width, height, fixed_max);
}

// savePPM to `path`; returns 1 on success.
int ref_save_ppm(const char* path, const float* rgb, int width, int height) {
  return savePPM(std::string(path), rgb, width, height) ? 1 : 0;
}

}  // extern "C"
