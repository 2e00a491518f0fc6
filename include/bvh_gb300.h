/*
 * bvh_gb300.h -- C ABI of the GB300 BVH construction library (libbvh_gb300.so).
 *
 * Plain pointers and sizes only; no CUDA or C++ types appear in the signatures (streams
 * are passed as `void*` holding a cudaStream_t, NULL = the legacy default stream).
 *
 * Each entry point replaces one piece of the reference (EdinHg/BVH) path:
 *   bvh_build_host    BVHBuilder::build(const TriangleMesh&) + getNodes/getIndices
 *                     (include/bvh_builder.h:10-37) for LBVHBuilderCUDA
 *                     (src/cuda/lbvh_builder.cu:484-488), LBVHPlusBuilderCUDA
 *                     (src/cuda/lbvh_plus_builder.cu:529-533) and PLOCBuilderCUDA
 *                     (src/cuda/ploc_builder.cu:403-586): host SoA in, host BVHNode array out.
 *   bvh_build_device  the same build on device-resident SoA input, result kept on the device
 *                     (the reference's runCompute without prepareData/downloadResults,
 *                     e.g. src/cuda/lbvh_builder.cu:376-463).
 *   bvh_last_timing   getLastBuildTimeMS / getTimingBreakdown (include/bvh_builder.h:29-36).
 *   bvh_trace         traverseBVH over explicit rays (src/render_engine.cu:289-356).
 *   bvh_trace_pinhole kRenderKernel's primary rays + traversal (src/render_engine.cu:362-446),
 *                     returning per-pixel hit t / primitive / counters instead of colours.
 *   bvh_shade,        kRenderKernel's shading (src/render_engine.cu:395-446) and renderImage's
 *   bvh_heatmap,      host post-processing -- applyHeatmapColormap (:541-595), savePPM's
 *   bvh_rgb8          conversion (:502-507) -- on the device.
 *   bvh_build_batched many independent meshes in one launch sequence (no reference counterpart;
 *                     each result equals bvh_build_device of that mesh alone).
 *
 * Result layout: BVHNode (include/bvh_node.h:8-31), 48 bytes per node; root at index 0; a leaf
 * has bit 31 of `left` set, the original triangle index in bits 0-30 and right = -1.
 * Errors never terminate the process (the reference's CUDA_CHECK calls exit(),
 * include/common.h:68-76); every call returns a bvh_status.
 */
#ifndef BVH_GB300_H
#define BVH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bvh_status {
  BVH_OK = 0,
  BVH_ERR_INVALID_ARG = 1,   /* bad pointer, size, algorithm or parameter */
  BVH_ERR_OUT_OF_MEMORY = 2, /* device or pinned allocation failed, or over the context budget */
  BVH_ERR_NO_PROGRESS = 3,   /* PLOC found no mutual pair (NaN/Inf areas) or hit its iteration cap */
  BVH_ERR_DEVICE = 4,        /* CUDA runtime error (the context may be unusable) */
  BVH_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
  BVH_ERR_UNSUPPORTED = 6    /* combination not implemented */
} bvh_status;

typedef enum bvh_algo {
  BVH_ALGO_LBVH = 0,      /* LBVHBuilderCUDA (30-bit) or 60/63-bit Morton */
  BVH_ALGO_LBVH_PLUS = 1, /* LBVHPlusBuilderCUDA: Karras tree + treelet restructuring */
  BVH_ALGO_PLOC = 2       /* PLOCBuilderCUDA(radius) */
} bvh_algo;

/* BVHNode, 48 bytes (AABB_cw = two 16-byte float3 + int32 children + padding). */
typedef struct bvh_node {
  float min_x, min_y, min_z, pad0;
  float max_x, max_y, max_z, pad1;
  int32_t left;  /* child index, or (primitive | 0x80000000) for a leaf */
  int32_t right; /* child index, or -1 for a leaf */
  int32_t aux0;  /* implementation detail (parent index while building); ignore */
  int32_t aux1;
} bvh_node;

/* TriangleMesh SoA (include/mesh.h:9-12): nine float arrays of n entries.  For device builds
 * the pointers are device pointers; 16-byte aligned arrays take the vectorised path. */
typedef struct bvh_mesh_soa {
  const float* v0x; const float* v0y; const float* v0z;
  const float* v1x; const float* v1y; const float* v1z;
  const float* v2x; const float* v2y; const float* v2z;
  uint32_t n;
} bvh_mesh_soa;

typedef struct bvh_params {
  int32_t algo;           /* bvh_algo */
  int32_t morton_bits;    /* LBVH: 30 (reference LBVH), 60 (reference LBVH+ keys) or 63; PLOC: 30 */
  int32_t treelet_rounds; /* LBVH+: refit+restructure passes (the reference runs 1) */
  int32_t ploc_radius;    /* PLOC search radius r (reference default 25) */
  int32_t max_iterations; /* PLOC iteration cap, 0 = n (an iteration that merges nothing always stops) */
  int32_t reserved[3];
} bvh_params;

/* A device-resident tree owned by the context; valid until the next build on that context. */
typedef struct bvh_tree {
  const bvh_node* nodes;   /* device pointer, n_nodes entries */
  const uint32_t* indices; /* device pointer, n_prims entries: original index of the i-th sorted triangle */
  uint32_t n_nodes;
  uint32_t n_prims;
} bvh_tree;

typedef struct bvh_timing {
  float total_ms;    /* device time of the whole build (kernels only, upload excluded) */
  float bounds_ms;   /* scene AABB */
  float morton_ms;   /* triangle boxes, Morton codes, histograms */
  float sort_ms;     /* radix sort */
  float emit_ms;     /* hierarchy + refit (LBVH) / cluster init (PLOC) */
  float optimize_ms; /* treelet passes (LBVH+) / clustering loop (PLOC) */
  int32_t ploc_iterations;
  int32_t tree_height;       /* LBVH+: tree height in the last treelet pass (one kernel pair per level) */
  uint64_t ploc_cluster_sum; /* sum of live clusters over PLOC iterations */
  int32_t kernel_launches;   /* PLOC and LBVH+: this library's kernels the build launched (their loops
                                run on the device: PLOC 4 per iteration launched one kernel per
                                phase and 1 each for the middle-iterations and tail kernels; LBVH+ 3
                                per tree height launched per phase and 1 for the narrow heights);
                                0 for LBVH */
  int32_t reserved;
} bvh_timing;

/* Per-ray traversal result (HitInfo, src/render_engine.cu:279-287, minus the normal). */
typedef struct bvh_hits {
  float* t;              /* closest hit distance, 1e30 on a miss */
  int32_t* prim;         /* original triangle index, -1 on a miss */
  int32_t* nodes_visited;
  int32_t* aabb_tests;
  int32_t* tri_tests;
} bvh_hits;

/* Rays as six SoA arrays (origin xyz, direction xyz). */
typedef struct bvh_rays {
  const float* ox; const float* oy; const float* oz;
  const float* dx; const float* dy; const float* dz;
  uint32_t n;
} bvh_rays;

/* Camera (include/render_engine.h:24-33). */
typedef struct bvh_camera {
  float eye[3];
  float look_at[3];
  float up[3];
  float fov_y_deg;
} bvh_camera;

/* Many independent meshes concatenated in one SoA (device pointers, mesh.n = total
 * triangles).  offsets is a HOST array of count+1 entries: mesh m owns triangles
 * [offsets[m], offsets[m+1]), offsets[0] = 0, offsets[count] = mesh.n, every mesh non-empty. */
typedef struct bvh_batch {
  bvh_mesh_soa mesh;
  const uint32_t* offsets;
  uint32_t count;
} bvh_batch;

/* bvh_params.reserved[0] for bvh_build_batched: 1 = capture the launch sequence into a CUDA
 * graph on first use and replay it while the batch layout (pointers, offsets) is unchanged. */
#define BVH_BATCH_USE_GRAPH 1

/* bvh_params.reserved[1]: 1 = drive the device loops from the host instead of CUDA graphs with
 * a conditional WHILE node: PLOC's clustering loop (one launch of each loop kernel per
 * iteration, the live cluster count read back after each) and LBVH+'s loop over tree heights
 * (the height read back once per pass).  Same tree; slower; for tools that cannot follow
 * conditional graph nodes (profilers) and drivers without them. */
#define BVH_HOST_DRIVEN_LOOPS 1

/* bvh_params.reserved[2]: 1 = launch no cooperative kernel.  PLOC's middle iterations and LBVH+'s
 * last, narrow tree heights normally run as one cooperative launch each, with grid barriers; here
 * they run one launch per kernel and iteration (or height), driven from the host, which is also
 * what a build does by itself when the device refuses the cooperative launch (a client limited
 * to part of the GPU).  Same tree; slower. */
#define BVH_NO_COOPERATIVE 1

typedef struct bvh_ctx bvh_ctx;

const char* bvh_status_string(bvh_status s);
/* Library version string. */
const char* bvh_version(void);

/* Create a context on `device` (CUDA ordinal).  Contexts are not thread-safe. */
bvh_status bvh_ctx_create(bvh_ctx** out, int device);
bvh_status bvh_ctx_destroy(bvh_ctx* ctx);
/* Pre-allocate workspace for meshes of up to n triangles (optional; builds grow it). */
bvh_status bvh_ctx_reserve(bvh_ctx* ctx, uint32_t n, int32_t algo);
/* Bytes of device memory the context currently holds. */
bvh_status bvh_ctx_device_bytes(const bvh_ctx* ctx, uint64_t* bytes);

/* Defaults: LBVH, 30-bit, 1 treelet round, radius 25. */
bvh_params bvh_default_params(int32_t algo);

/* Build from device-resident SoA.  Asynchronous on `stream` for LBVH/LBVH+ (PLOC reads one
 * counter per iteration back to the host).  The tree stays owned by the context. */
bvh_status bvh_build_device(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, void* stream,
                            bvh_tree* out);

/* Build from host SoA, as BVHBuilder::build does: upload, build, download.  Synchronous.
 * host_nodes must hold 2n-1 entries (n >= 1), host_indices n entries.  For a plain LBVH the
 * indices and the leaf nodes are copied out on a second stream of the context while the build
 * finishes (pinned host buffers let those copies overlap the kernels). */
bvh_status bvh_build_host(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, void* stream,
                          bvh_node* host_nodes, uint32_t* host_indices, uint32_t* n_nodes);

/* Copy a device tree to host arrays (2n-1 nodes, n indices). */
bvh_status bvh_tree_download(bvh_ctx* ctx, const bvh_tree* tree, void* stream, bvh_node* host_nodes,
                             uint32_t* host_indices);

/* Self-test of the device-side bounded waits (no reference counterpart): the radix sort's
 * look-back wait is run on `device` against a predecessor that never publishes, and the grid
 * barrier of the cooperative PLOC kernel against a block that never arrives, each giving up after
 * `polls` polls (1 .. 16,777,216).  Returns BVH_ERR_TIMEOUT -- the expected outcome: both waits
 * ended and reported it, and the device is still usable -- or BVH_ERR_DEVICE / another error if
 * either did not.  Synchronous; allocates nothing. */
bvh_status bvh_selftest_bounded_wait(int device, uint32_t polls);

/* Timing of the last build; waits for it to finish.  Also reports device-side errors. */
bvh_status bvh_last_timing(bvh_ctx* ctx, bvh_timing* out);
/* Wait for the last build and report device-side errors (bounded waits that gave up). */
bvh_status bvh_sync(bvh_ctx* ctx);

/* Build every mesh of a batch: LBVH with 30-bit Morton codes, or PLOC(ploc_radius) (other
 * combinations: BVH_ERR_UNSUPPORTED).  Result: 2*mesh.n - count nodes; mesh m's tree occupies
 * nodes [2*offsets[m] - m, 2*offsets[m+1] - m - 1) with its root first and child indices relative
 * to that first node, and indices [offsets[m], offsets[m+1]) hold mesh-local original triangle
 * indices -- each mesh's part equals bvh_build_device of that mesh alone.  PLOC clusters all
 * meshes in the same iterations (as many as the slowest mesh needs; bvh_last_timing reports
 * them).  With BVH_BATCH_USE_GRAPH the whole build, PLOC's loop included, is one graph launch.
 * Asynchronous on `stream`. */
bvh_status bvh_build_batched(bvh_ctx* ctx, const bvh_batch* batch, const bvh_params* params, void* stream,
                             bvh_tree* out);

/* Autotuner (no reference counterpart): times every radix-sort variant (items per thread,
 * look-back window, blocks per SM) on n pseudo-random 32-bit keys (every build sorts 32-bit keys:
 * 30-bit codes whole, the high halves of longer codes), keeps the fastest in the context and
 * writes a JSON table of the timings to json_out (may be NULL).  Synchronous. */
bvh_status bvh_autotune(bvh_ctx* ctx, uint32_t n, void* stream, char* json_out, size_t json_cap);
/* Read the sort variant of the context's last build, or set the one it uses (0 .. 4) where no
 * tuning-table entry applies.  Until set (here or by bvh_autotune) a build picks it by mesh size:
 * 8 keys per thread below 600k triangles, 16 up to 2M, 24 (16-wide look-back window) above. */
bvh_status bvh_tuning_get(const bvh_ctx* ctx, int32_t* variant);
bvh_status bvh_tuning_set(bvh_ctx* ctx, int32_t variant);

/* Autotuner for whole builds (no reference counterpart).  Builds `mesh` (device SoA, at least
 * 1,024 triangles) with `params` under each launch shape -- radix-sort variant; for PLOC also the
 * sizes at which the cooperative middle-iterations kernel and the one-block tail kernel take
 * over, and the neighbour-search and merge grids --
 * by coordinate descent, 3 timed builds each, checking that every shape gives the identical
 * tree (a device hash of all node fields; BVH_ERR_DEVICE if one did not).  The fastest is kept in
 * the context's tuning table under (algorithm, floor(log2(n))) and used by later builds of that
 * algorithm and size (batched builds have their own entries, algorithm + 256).  Choices that
 * change the tree -- PLOC radius 10/25/50/100, LBVH+ treelet passes 1/2/3, LBVH Morton bits
 * 30/60/63 -- are built and reported with their time and SAH, never chosen.  json_out (may be
 * NULL) receives {"n", "chosen", "best_ms", "trials": [...], "tree_changing": [...]}.
 * Synchronous. */
bvh_status bvh_autotune_build(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_params* params, void* stream,
                              char* json_out, size_t json_cap);
/* The tuning table as JSON ({"base": {...}, "entries": [{"algo", "bucket", "sort_variant",
 * "ploc_tail_pairs", "ploc_nn_bps", "ploc_mg_bps", "ploc_grid_max"}, ...]}), to persist it; and back (replaces the
 * table; BVH_ERR_INVALID_ARG for malformed input or out-of-range shapes).  The base entry is
 * informational (import reads only "entries"); its sort_variant is -1 while builds pick the
 * variant by mesh size. */
bvh_status bvh_tuning_export(const bvh_ctx* ctx, char* json_out, size_t json_cap);
bvh_status bvh_tuning_import(bvh_ctx* ctx, const char* json);

/* LBVH build that allocates nothing (no counterpart in the reference).  For callers that cannot
 * call cudaMalloc -- a host that forbids device allocations after start-up, a real-time loop
 * with a fixed memory budget -- and so cannot create a bvh_ctx.  Inputs (device SoA) and
 * outputs (device: 2n-1 nodes, n indices) come from the caller; all other scratch is one
 * fixed __device__ array inside the library (about 17 MB per GPU that loads it, held until
 * exit), so n may be at most 262,144 (BVH_ERR_INVALID_ARG beyond).  morton_bits: 30, 60 or 63;
 * the result equals bvh_build_device's.  Asynchronous on `stream`.  The first call on a device
 * also sets kernel attributes; make that first call before any stream capture.  Calls share the
 * array: calls that overlap on the GPU race, so serialise them.  Device-side errors go
 * unreported here: BVH_OK means the kernels were launched.  (The radix sort's bounded look-back
 * wait, a safety net that normal operation never reaches, reports through bvh_sync on the
 * context path only.) */
bvh_status bvh_build_lbvh_static(const bvh_mesh_soa* mesh, int32_t morton_bits, bvh_node* nodes, uint32_t* indices,
                                 void* stream);

/* ---- serving (no reference counterpart) ----------------------------------------------------
 * A continuously batched build+trace server.  Each request carries a host mesh, host rays and
 * host hit buffers (which must stay valid until its result is polled); it gets an LBVH of its
 * mesh and the closest hits of its rays.  Requests are admitted oldest first whenever a slot is
 * free and the memory fits the budget; admitted work overlaps on the GPU.  A request's result
 * does not depend on what else is in flight.
 *   per-request slots (reserved[0] = 0): each request runs alone on a slot's stream (upload,
 *     build, trace, download); morton_bits 30, 60 or 63.
 *   batched ticks (reserved[0] = BVH_SERVE_BATCHED): when a slot is free, every waiting request
 *     that fits joins one batch -- one gather kernel reads all meshes and rays from the callers'
 *     buffers (page-locked buffers, or any host memory where the GPU reads pageable memory;
 *     others are copied), one batched LBVH build, one traversal launch, one scatter kernel writes
 *     all hits back; requests arriving meanwhile form the next batch on another slot.  30-bit
 *     codes only.  reserved[1] = requests per batch at most (0: 64); reserved[2] = triangles per
 *     batch at most (0: 8,388,608; a larger single request still runs, alone).
 * hbm_budget_bytes bounds the device memory all slots hold together, busy or idle: a slot that
 * must grow first takes memory back from idle slots, and requests wait while it cannot. */
typedef struct bvh_server bvh_server;

#define BVH_SERVE_BATCHED 1

typedef struct bvh_serve_config {
  uint64_t hbm_budget_bytes; /* device memory all slots hold together, at most */
  int32_t slots;             /* requests (per-request mode) or batches (batched mode) in flight at most */
  int32_t morton_bits;       /* LBVH keys: 30, 60 or 63 (batched mode: 30) */
  int32_t device;
  uint32_t max_triangles;    /* per-slot buffers allocated up front for this size (0: grow on demand) */
  uint32_t max_rays;
  int32_t reserved[3];       /* [0] mode, [1] requests per batch, [2] triangles per batch (see above) */
} bvh_serve_config;

typedef struct bvh_serve_request {
  bvh_mesh_soa mesh; /* host pointers */
  bvh_rays rays;     /* host pointers */
  bvh_hits hits;     /* host pointers, rays.n entries each (NULL entries are skipped) */
  uint64_t tag;      /* returned in the result */
} bvh_serve_request;

typedef struct bvh_serve_result {
  uint64_t tag;
  int32_t status;       /* bvh_status; BVH_ERR_OUT_OF_MEMORY if it can never fit the budget */
  uint32_t triangles;
  uint32_t rays;
  uint32_t reserved;
  uint64_t t_submit_ns; /* steady-clock times: submitted, admitted to a slot, completed */
  uint64_t t_admit_ns;
  uint64_t t_done_ns;
} bvh_serve_result;

typedef struct bvh_serve_stats {
  uint64_t submitted, admitted, completed, rejected, budget_waits;
  uint64_t triangles, rays;
  uint64_t in_flight_bytes, peak_in_flight_bytes, queued;
} bvh_serve_stats;

bvh_serve_config bvh_serve_default_config(void);
bvh_status bvh_serve_open(const bvh_serve_config* cfg, bvh_server** out);
/* Queue a request (does not block on the GPU). */
bvh_status bvh_serve_submit(bvh_server* sv, const bvh_serve_request* req);
/* Move up to max_results finished requests into out, waiting up to wait_ms for the first. */
int32_t bvh_serve_poll(bvh_server* sv, bvh_serve_result* out, int32_t max_results, int32_t wait_ms);
bvh_status bvh_serve_stats_get(bvh_server* sv, bvh_serve_stats* out);
/* Finish every queued request, then release the server. */
bvh_status bvh_serve_close(bvh_server* sv);

/* ---------------------------------------------------------------------------------------
 * OBJ input: loadOBJ (src/loader.cpp:10-74) as a multi-threaded parse straight to SoA.
 * ------------------------------------------------------------------------------------- */
typedef struct bvh_obj_mesh {
  float* v[9];       /* v0x v0y v0z v1x v1y v1z v2x v2y v2z, n floats each (library-owned) */
  uint32_t n;        /* triangles */
  uint32_t pinned;   /* arrays are page-locked (cudaMallocHost) */
  uint64_t vertices; /* 'v' lines read */
} bvh_obj_mesh;
/* Same rules as loadOBJ: '#' and empty lines skipped; "v x y z"; "f" with v, v/vt, v//vn or
 * v/vt/vn tokens, negative indices counting back from the vertices read so far; fan
 * triangulation; a triangle with an index outside the vertices read so far is skipped.
 * threads <= 0: all hardware threads.  pinned != 0: page-locked arrays (fast upload).
 * BVH_ERR_INVALID_ARG for an unreadable file or an index loadOBJ's std::stoi would reject. */
bvh_status bvh_load_obj(const char* path, int32_t threads, int32_t pinned, bvh_obj_mesh* out);
void bvh_obj_free(bvh_obj_mesh* m);

/* Tree statistics (BVHEvaluator::evaluate, src/evaluator.cpp:7-113) computed on the GPU for a
 * device node array: SAH with the reference's costs (3 per internal node, 2 per leaf, areas
 * relative to the root), reachable node and leaf counts, maximum and average leaf depth.  The
 * per-node terms are the host evaluator's; they are summed in double.  Synchronous. */
typedef struct bvh_eval_stats {
  double sah;
  double avg_leaf_depth;
  uint64_t node_count;
  uint64_t leaf_count;
  uint32_t max_depth;
  uint32_t reserved;
} bvh_eval_stats;
bvh_status bvh_evaluate(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, void* stream, bvh_eval_stats* out);

/* Closest-hit traversal of explicit rays (device pointers).  Asynchronous. */
bvh_status bvh_trace(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, const bvh_mesh_soa* mesh,
                     const bvh_rays* rays, const bvh_hits* hits, void* stream);
/* Primary pinhole rays (generateRay, src/render_engine.cu:155-188) for a width x height
 * image, one per pixel in row-major order, then traversal.  Asynchronous. */
bvh_status bvh_trace_pinhole(bvh_ctx* ctx, const bvh_node* nodes, uint32_t n_nodes, const bvh_mesh_soa* mesh,
                             const bvh_camera* cam, int32_t width, int32_t height, const bvh_hits* hits,
                             void* stream);
/* The rays bvh_trace_pinhole generates (device pointers, width*height each). */
bvh_status bvh_pinhole_rays(const bvh_camera* cam, int32_t width, int32_t height, float* ox, float* oy, float* oz,
                            float* dx, float* dy, float* dz, void* stream);
/* autoCamera (src/render_engine.cu:601-637) from the root box of a tree (host node). */
bvh_status bvh_auto_camera(const bvh_node* host_root, bvh_camera* cam);

/* Pixel shading of a bvh_trace_pinhole result (kRenderKernel's shading, src/render_engine.cu:
 * 395-446), on the device: `hits` from bvh_trace_pinhole with the same camera and size; mode 0
 * normal mapped to RGB, 1 depth (t / scene_diag, closer is brighter), 2 diffuse (light_dir, a
 * host float[3], normalised by the caller; ambient 0.15), 3 the raw node-visit count (colour it
 * with bvh_heatmap); a miss gets the background (0.15, 0.15, 0.18).  rgb: device float[3 * w * h].
 * Asynchronous. */
bvh_status bvh_shade(bvh_ctx* ctx, const bvh_mesh_soa* mesh, const bvh_camera* cam, int32_t width, int32_t height,
                     const bvh_hits* hits, int32_t mode, float scene_diag, const float* light_dir, float* rgb,
                     void* stream);
/* Traversal-cost heatmap (applyHeatmapColormap, src/render_engine.cu:541-595) on the device: each
 * pixel's node-visit count over fixed_max, or, when fixed_max <= 0, over the 99.9th percentile of
 * the nonzero counts (128 when there are none; at least 1), clamped to [0, 1] and looked up with
 * linear interpolation in `colormap` (device float[256 * 3], RGB per entry -- the reference passes
 * its Turbo table); a count of 0 gets the background.  used_max (device float, may be NULL)
 * receives the normalisation.  Asynchronous. */
bvh_status bvh_heatmap(bvh_ctx* ctx, const int32_t* nodes_visited, uint32_t n_pixels, const float* colormap,
                       float fixed_max, float* rgb, float* used_max, void* stream);
/* Float RGB to bytes as savePPM writes them (src/render_engine.cu:502-507): clamp to [0, 1],
 * v * 255 + 0.5 truncated.  Device buffers of n_values each.  Asynchronous. */
bvh_status bvh_rgb8(const float* rgb, uint32_t n_values, uint8_t* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* BVH_GB300_H */
