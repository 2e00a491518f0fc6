// lbvh.cuh -- host-side interface of the build kernels (internal to the library).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace bvhgb {

struct MeshPtrs {
  const float* v[9];  // v0x v0y v0z v1x v1y v1z v2x v2y v2z (TriangleMesh order)
};

// Device workspace owned by a context; grown on demand, reused across builds.
struct Workspace {
  uint32_t cap_n = 0;        // triangles the buffers can hold
  int sort_variant = 0;      // onesweep variant (bvh_autotune)
  // PLOC launch shapes (bvh_autotune_build); none of them changes the tree
  uint32_t ploc_tail_pairs = 100000;  // hand over to k_ploc_tail below this many pair areas (0: never)
  uint32_t ploc_grid_max = 0xffffffffu;  // k_ploc_grid takes over at this many live clusters
                                         // (capped at what its grid holds; 0: never)
  int ploc_nn_bps = 3;                // neighbour-search blocks per SM
  int ploc_mg_bps = 8;                // merge (count / scatter) blocks per SM
  void* keys[2] = {nullptr, nullptr};
  uint32_t* vals[2] = {nullptr, nullptr};
  Box* boxes = nullptr;      // per-triangle AABB in input order
  Node* nodes = nullptr;     // 2n-1 output nodes
  unsigned long long* slots = nullptr;  // n-1 rendezvous words (epoch << 32 | endpoint)
  uint32_t* scratch = nullptr;          // histograms, look-back descriptors, counters
  uint8_t* delta = nullptr;             // n-1 adjacent common-prefix lengths (+1)
  size_t scratch_words = 0;
  // PLOC buffers
  Box* cbox[2] = {nullptr, nullptr};
  int32_t* cid[2] = {nullptr, nullptr};
  int32_t* nbr = nullptr;
  uint32_t ploc_cap = 0;
  cudaGraphExec_t ploc_exec = nullptr;  // clustering loop graph, valid for the key below
  uint32_t* ploc_host = nullptr;        // pinned words for the host-driven loops
  cudaGraphExec_t tl_exec = nullptr;    // LBVH+ loop over heights, valid for the key below
  uint32_t tl_key_n = 0;
  const void* tl_key_nodes = nullptr;
  const void* tl_key_list = nullptr;
  const void* tl_key_desc = nullptr;
  const void* tl_key_ctl = nullptr;
  bool tl_narrow = false;               // the last treelet pass launched k_tl_narrow
  bool no_cooperative = false;          // run no cooperative kernel (their host-driven fallbacks)
  uint32_t ploc_key_n = 0;
  int ploc_key_r = 0;
  const void* ploc_key_nodes = nullptr;
  const void* ploc_key_scratch = nullptr;
  uint32_t ploc_key_shape = 0;  // nn and merge blocks per SM the cached loop graph was made with
  cudaStream_t aux_stream = nullptr;  // a second stream for capturing loop bodies
  uint64_t epoch_builds = 0;           // builds that bumped this workspace's epoch (epoch_tick)
  // the batched PLOC loop graph and what it was made for
  cudaGraphExec_t ploc_seg_exec = nullptr;
  uint32_t ploc_seg_key_n = 0, ploc_seg_key_count = 0;
  int ploc_seg_key_r = 0;
  const void* ploc_seg_key[4] = {};
  uint32_t ploc_seg_key_shape = 0;
  // device-side mesh copy for host-pointer builds
  float* mesh_dev = nullptr;
  uint32_t mesh_cap = 0;
  // batched builds
  uint32_t* bat_offsets = nullptr;    // device: count + 1 offsets, then the work items
  uint32_t* bat_offsets_h = nullptr;  // pinned staging of the same
  uint32_t bat_items = 0;             // work items in the staged layout
  size_t bat_words_cap = 0;
  float* bat_mbox = nullptr;          // device, count * 8
  uint32_t* bat_indices = nullptr;    // device, n (mesh-local original indices)
  uint32_t bat_count_cap = 0, bat_n_cap = 0;
  // recorded (when set) between the LBVH emission and its frontier climb: from there on the leaf
  // nodes [n-1, 2n-1) of a plain LBVH are final and can be copied out while the climb runs
  cudaEvent_t leaves_ready = nullptr;
};

// First epoch value; every build adds kEpochStride (emission uses E, treelet round r uses E+1+r).
constexpr uint32_t kEpochStride = 64;
// The 32-bit epoch repeats after this many builds (it wraps to kEpochStride); the build that
// reuses an epoch first clears the rendezvous slots (epoch_tick).
constexpr uint64_t kEpochCycle = (1ull << 26) - 1;

// Scratch layout (32-bit words, offsets from Workspace::scratch).
struct ScratchLayout {
  size_t status;     // 1 word, device status bits
  size_t ticket;     // 1 word, bounds-reduction arrival counter (self-resetting)
  size_t epoch;      // 1 word, rendezvous tag of the current build (bumped by 64 per build)
  size_t scene;      // 8 words, SceneParams
  size_t counters;   // 16 words, per-pass tile counters
  size_t hist;       // passes * 256
  size_t desc;       // passes * tiles * 256
  size_t partials;   // bounds partials, kBoundsBlocks * 8
  size_t ploc;       // PLOC control words (20)
  size_t zero_begin; // first word zeroed at the start of each build
  size_t zero_end;
  size_t total;
};

constexpr int kBoundsBlocks = 152 * 4;
constexpr int kSortThreads = 256;
constexpr int kMaxPasses = 4;  // 8-bit passes over 32-bit keys
constexpr int kFrontierCounter = 15;  // counters[15]: emission frontier length (passes use 0..7)
constexpr int kLongRunCounter = 14;   // counters[14]: runs listed for the block-wide fix-up

ScratchLayout scratch_layout(uint32_t n);
int sort_tile();  // smallest tile over all variants (sizes the look-back scratch)
int sort_variant_count();
int sort_variant_tile(int v);
int default_sort_variant(uint32_t n);  // by key count, where no tuning chose a variant
void sort_variant_describe(int v, int* ipt, int* window, int* minb);
// Times every onesweep variant on `n` pseudo-random 32-bit keys and keeps the fastest in ws.
cudaError_t autotune_sort(Workspace& ws, uint32_t n, cudaStream_t st, float* ms_out /* per variant */);

// Builds stage events: [0] start, [1] bounds, [2] morton, [3] sort, [4] emit, [5] optimise.
struct StageEvents {
  cudaEvent_t ev[8];
  bool use = false;
};

// LBVH over device-resident SoA input; result in ws.nodes / ws.vals[final].
// morton_bits: 30, 60 or 63.  treelet_rounds > 0 selects LBVH+.
cudaError_t lbvh_build(Workspace& ws, const MeshPtrs& m, uint32_t n, int morton_bits, int treelet_rounds,
                       cudaStream_t st, StageEvents* evs, uint32_t** out_indices, bool host_loops = false);

// PLOC (radius r) over device-resident SoA input, fully asynchronous (the clustering loop is a
// CUDA graph WHILE node).  Node count is 2n-1; iterations and the live-cluster sum are left in
// the PLOC control words (kPlocIterWord, kPlocSumWord) and a loop that cannot finish sets
// kStatusNoProgress.
cudaError_t ploc_build(Workspace& ws, const MeshPtrs& m, uint32_t n, int radius, int max_iter,
                       cudaStream_t st, StageEvents* evs, uint32_t** out_indices, bool host_loop = false);
constexpr int kPlocIterWord = 6;
constexpr int kPlocSumWord = 8;

// Shared pieces used by PLOC: bounds + Morton-30 + sort (indices sorted by code).
cudaError_t prefix_sort30(Workspace& ws, const MeshPtrs& m, uint32_t n, cudaStream_t st, StageEvents* evs,
                          uint32_t** sorted_idx);

// Runs the sort's bounded look-back wait against a predecessor that never publishes, giving up
// after `limit` polls; *status_out = the status word it left (kStatusSortTimeout expected).
cudaError_t wait_selftest(uint32_t limit, uint32_t* status_out);
// Runs the cooperative PLOC kernel's grid barrier against a block that never arrives, giving up
// after `limit` polls per block; *status_out = the status word it left (kStatusGridTimeout).
cudaError_t grid_wait_selftest(uint32_t limit, uint32_t* status_out);

// Kernel attributes (dynamic shared memory limits), set once per device before any capture.
cudaError_t prepare_kernels();

// Count one build that bumps the epoch; before the build that would reuse an old epoch, clear the
// rendezvous slots on `st`.  Not counted while `st` is being captured: each launch of the graph
// counts instead (call it before cudaGraphLaunch).
cudaError_t epoch_tick(Workspace& ws, cudaStream_t st);

// Grow `ws` to hold n triangles (cudaMalloc; synchronising).
cudaError_t workspace_reserve(Workspace& ws, uint32_t n, cudaStream_t st);
cudaError_t workspace_reserve_ploc(Workspace& ws, uint32_t n);
// PLOC kernel attributes for a radius (shared memory of the neighbour search); before any capture.
cudaError_t ploc_prepare(int radius);
// Live clusters at which k_ploc_tail takes over for a radius and a pair budget (0: never).
uint32_t ploc_tail_threshold(int radius, uint32_t pairs);
// Order-independent 64-bit hash of every node's min, max, left and right (with its index), on the
// device; *out (device) receives it.  Equal trees hash equal.
cudaError_t tree_hash(const Node* nodes, uint32_t n_nodes, unsigned long long* out, cudaStream_t st);
void workspace_free(Workspace& ws);

// Tree statistics on the device (BVHEvaluator, src/evaluator.cpp:38-113).
struct EvalResult {
  double sah = 0, avg_leaf_depth = 0;
  unsigned long long nodes = 0, leaves = 0;
  uint32_t max_depth = 0;
};
size_t evaluate_scratch_bytes(uint32_t n_nodes);
cudaError_t evaluate_tree(const Node* nodes, uint32_t n_nodes, void* scratch, cudaStream_t st, EvalResult* out);

// Completes a sort of codes held split: hkeys = code >> lbits (sorted by the radix passes),
// lows = the low lbits bits by original index.  Orders every run of equal hkeys by (low bits,
// position), moving only the values; run starts that need the block-wide path are listed in
// long_list (room for n / 6 words) behind the zeroed counter long_count.  scratch_a/scratch_b (8 B per position) and
// tvals serve the block-wide sort of runs longer than 1024.
// With D non-null it also writes the delta bytes D[k] = delta(k, k+1) + 1 of the final order
// (60/63-bit codes: clz of the 64-bit code XOR, 64 + clz of the index XOR for equal codes), so
// no separate delta pass is needed; long_list must then lie outside D.
cudaError_t sort_fix_runs_split(const uint32_t* hkeys, uint32_t* vals, const uint32_t* lows, uint32_t n, int lbits,
                                unsigned long long* scratch_a, unsigned long long* scratch_b, uint32_t* tvals,
                                uint32_t* long_list, uint32_t* long_count, uint8_t* D, cudaStream_t st);

// Treelet restructuring passes (LBVH+) after emission; fb = the sort's final ping-pong buffer
// (the other one is scratch).
cudaError_t treelet_rounds_run(Workspace& ws, uint32_t n, int rounds, cudaStream_t st, int fb,
                               bool host_loop = false);
// Treelet control words (scratch + L.hist + kTlCtlWord): [0] too high, [1] tree height.
constexpr size_t kTlCtlWord = 256 + 264 + 256;

// Stable sort of the 32-bit keys in ws.keys[0] with implicit indices over `passes` 8-bit digits;
// *final_buf = the ping-pong buffer holding the result.
cudaError_t run_sort_u32(Workspace& ws, uint32_t n, int passes, cudaStream_t st, const ScratchLayout& L,
                         int* final_buf);

// A slice of one mesh handled by one block of the batched per-mesh kernels.
struct SegItem {
  uint32_t mesh, begin, end, pad;
};
constexpr uint32_t kSegChunk = 16384;

// The shared prefix of the batched builds: per-mesh boxes, keys mesh << 30 | code30, stable sort.
struct BatchedSort {
  int fb = 0;              // ping-pong buffer holding the sorted keys (high 32 bits) and indices
  int shift0 = 0;          // key bits below the sorted high 32
  uint32_t* lows = nullptr;  // those low bits by original index (inside the node buffer)
};
cudaError_t batched_prefix(Workspace& ws, const MeshPtrs& m, uint32_t n, uint32_t count, const SegItem* d_items,
                           uint32_t n_items, float* d_mbox, cudaStream_t st, StageEvents* evs, BatchedSort* out);

// Batched PLOC(radius) over the same layout: every mesh's tree equals its single build.  d_mbox
// (8 words per mesh) holds the per-mesh loop state once the keys are made.
cudaError_t batched_ploc_build(Workspace& ws, const MeshPtrs& m, uint32_t n, const uint32_t* d_offsets,
                               uint32_t count, const SegItem* d_items, uint32_t n_items, float* d_mbox,
                               uint32_t* d_indices, int radius, uint32_t max_iter, cudaStream_t st,
                               StageEvents* evs, bool host_loop);

// Batched LBVH-30 over `count` meshes concatenated in one SoA (offsets and work items on the device).
cudaError_t batched_build(Workspace& ws, const MeshPtrs& m, uint32_t n, const uint32_t* d_offsets, uint32_t count,
                          const SegItem* d_items, uint32_t n_items, float* d_mbox, uint32_t* d_indices,
                          cudaStream_t st, StageEvents* evs);

}  // namespace bvhgb
