/*
 * bvh_oracle.h -- CPU restatement of the reference BVH builders (TEST INFRASTRUCTURE).
 *
 * The tests compare the GPU library in bvh_gb300/ against this library: only the tests, the
 * smoke check and bench.py's CPU-baseline leg call it.  It is never linked into, or
 * called by, the product path.
 *
 * Each function restates one piece of the reference (EdinHg/BVH) and cites the
 * reference file:line it follows.  Arithmetic is written so that gcc cannot contract
 * it (-ffp-contract=off); where the reference's device code may be FMA-contracted by
 * nvcc (AABB_cw::surfaceArea, include/common.h:41-44) the contraction form is a
 * runtime switch (orc_set_sa_form), pinned by measurement against the reference
 * kernels on the GPU.
 */
#ifndef BVH_ORACLE_H
#define BVH_ORACLE_H
#include <stdint.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* AABB_cw (include/common.h:29-65): two 16-byte aligned float3 = 32 bytes. */
typedef struct orc_aabb { float mn[3]; float pad0; float mx[3]; float pad1; } orc_aabb;
/* BVHNode (include/bvh_node.h:8-31): AABB_cw + two int32 children, padded to 48 bytes. */
typedef struct orc_node { orc_aabb box; int32_t left, right; int32_t pad[2]; } orc_node;

/* Nine SoA vertex arrays, TriangleMesh (include/mesh.h:9-12) order v0x..v2z. */
typedef struct orc_mesh { const float* v[9]; uint32_t n; } orc_mesh;

enum { ORC_OK = 0, ORC_ERR_INVALID = 1, ORC_ERR_NO_PROGRESS = 3 };

/* Surface-area evaluation form of 2*(dx*dy + dy*dz + dz*dx); 0 = no contraction.
 * Forms 1..7 are the FMA contractions listed in bvh_oracle.c (orc_sa). */
void orc_set_sa_form(int form);
int orc_get_sa_form(void);
float orc_sa(const orc_aabb* b);
/* float min/max with the device's semantics (NaN operand ignored, -0 < +0). */
float orc_fmin(float a, float b);
float orc_fmax(float a, float b);

/* Per-triangle AABB and centroid: kComputeBoundsAndCentroids_nt, src/cuda/lbvh_builder.cu:47-66. */
void orc_tri_bounds(const orc_mesh* m, orc_aabb* boxes, float* centroids4 /* n*4, may be NULL */);
/* Scene AABB: union of all triangle boxes, src/cuda/lbvh_builder.cu:73-165. */
void orc_scene_bounds(const orc_aabb* boxes, uint32_t n, orc_aabb* out);
/* Morton codes of the centroids normalised to the scene box.
 * bits=30: src/cuda/lbvh_builder.cu:11-27,167-181 (x in the top slot).
 * bits=60: src/cuda/lbvh_plus_builder.cu:20-35,276-290 (z in the top slot, 20 bits/axis).
 * bits=63: the 60-bit layout with 21 bits per axis (no reference counterpart). */
void orc_morton(const float* centroids4, uint32_t n, int bits, const orc_aabb* scene, uint64_t* codes);
/* Stable sort of (key, index) pairs by key; index payload starts as 0..n-1 when init_idx. */
void orc_sort_pairs(uint64_t* keys, uint32_t* idx, uint32_t n, int key_bits, int init_idx);
/* Karras hierarchy over sorted keys: kBuildInternalNodes_nt, src/cuda/lbvh_builder.cu:183-229
 * (key_width 32) and kBuildInternalNodes_P, src/cuda/lbvh_plus_builder.cu:292-324 (key_width 64).
 * Writes children of internal nodes 0..n-2 (boxes untouched). */
void orc_karras(const uint64_t* keys, const uint32_t* idx, uint32_t n, int key_width, orc_node* nodes);
/* Leaves at n-1+i: kInitLeafNodes_nt, src/cuda/lbvh_builder.cu:231-241. */
void orc_init_leaves(const orc_aabb* tri_boxes, const uint32_t* idx, uint32_t n, orc_node* nodes);
/* Bottom-up union of child boxes: kRefitHierarchy_nt, src/cuda/lbvh_builder.cu:243-274. */
void orc_refit(orc_node* nodes, uint32_t n_nodes);

/* Whole LBVH build (LBVHBuilderCUDA::runCompute, src/cuda/lbvh_builder.cu:376-463).
 * nodes: 2n-1 entries; indices: n; sorted_keys (optional): n. */
int orc_lbvh(const orc_mesh* m, int bits, orc_node* nodes, uint32_t* indices, uint64_t* sorted_keys);
/* LBVH+ (LBVHPlusBuilderCUDA::runCompute, src/cuda/lbvh_plus_builder.cu:441-508): Karras tree,
 * refit, then `rounds` bottom-up refit+treelet passes (the reference runs one). */
int orc_lbvh_plus(const orc_mesh* m, int bits, int rounds, orc_node* nodes, uint32_t* indices);
/* One treelet restructuring at `root` (optimizeTreeletSerial, src/cuda/lbvh_plus_builder.cu:71-247). */
void orc_treelet(orc_node* nodes, uint32_t* parent, int root);
/* PLOC (PLOCBuilderCUDA::build, src/cuda/ploc_builder.cu:403-586) with new nodes numbered in
 * ascending cluster order within each iteration.  Returns ORC_ERR_NO_PROGRESS when an iteration
 * merges nothing or max_iter is reached. */
int orc_ploc(const orc_mesh* m, int radius, int max_iter, orc_node* nodes, uint32_t* indices,
             uint32_t* n_nodes, int* iterations, uint64_t* cluster_sum);

/* Closest-hit traversal (traverseBVH, src/render_engine.cu:289-356) of explicit rays. */
void orc_trace(const orc_node* nodes, uint32_t n_nodes, const orc_mesh* m,
               const float* ray_o /* 3*nr */, const float* ray_d /* 3*nr */, uint32_t nr,
               float* t, int32_t* prim, int32_t* visited, int32_t* aabb_tests, int32_t* tri_tests);
/* Pinhole primary rays (generateRay, src/render_engine.cu:155-188), written as origin/direction. */
void orc_pinhole_rays(const float eye[3], const float look[3], const float up[3], float fovy,
                      int width, int height, float* ray_o, float* ray_d);

/* SAH (BVHEvaluator::computeSAH, src/evaluator.cpp:38-88) and depth statistics (:90-113). */
float orc_sah(const orc_node* nodes, uint32_t n_nodes);
void orc_depth_stats(const orc_node* nodes, uint32_t n_nodes, int* max_depth, float* avg_leaf_depth,
                     uint32_t* leaf_count);

/* Canonical comparison of two trees (node ids may differ): 0 if every subtree matches in
 * leaf primitive, child order and box bits. */
int orc_tree_equal_canonical(const orc_node* a, uint32_t na, const orc_node* b, uint32_t nb);

/* Number of OpenMP threads used (1 when built without OpenMP). */
int orc_threads(void);
void orc_set_threads(int t);

/* kRenderKernel's shading (src/render_engine.cu:395-446), applyHeatmapColormap (:519-595) and
 * savePPM's byte conversion (:502-507). */
void orc_shade(const orc_mesh* m, const float* rd, const float* t, const int32_t* prim, const int32_t* vis,
               uint32_t np, int mode, float diag, const float light[3], float* rgb);
float orc_heatmap(const int32_t* vis, uint32_t np, const float* lut, float fixed_max, float* rgb);
void orc_rgb8(const float* rgb, uint32_t nv, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif
