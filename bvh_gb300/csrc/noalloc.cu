// noalloc.cu -- an LBVH build that allocates no memory (bvh_build_lbvh_static).
//
// For callers that cannot call cudaMalloc: code that runs inside a host application's
// real-time or pre-allocated memory budget, plugins whose host forbids device allocations
// after start-up, and callers that must not take the device-wide synchronisation that
// cudaMalloc/cudaFree can imply.  Everything except the caller's inputs and outputs lives in
// one file-scope __device__ array of fixed size, which every GPU that loads this library holds
// until the process exits.  All calls share that array, so calls that overlap on the GPU (two
// streams, two threads) race and corrupt each other's results; serialise them.
// The call returns before its kernels finish and has no buffer of the caller's to report into,
// so device-side errors go unreported: the radix sort's look-back waits are bounded and record a
// timeout in the array's status word, which the context path reads, but this path does not.
// (A look-back only waits on tiles that started before it, so the bound is a safety net; it is
// not reached in normal operation.)
#include <mutex>

#include "../../include/bvh_gb300.h"
#include "lbvh.cuh"

using namespace bvhgb;

namespace {

constexpr uint32_t kStaticMaxTris = 1u << 18;  // 262,144 triangles

// Layout of the static scratch for kStaticMaxTris (bytes, 256-aligned pieces).
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kKeysBytes = align256((size_t)kStaticMaxTris * 8);
constexpr size_t kValsBytes = align256((size_t)kStaticMaxTris * 4);
constexpr size_t kBoxBytes = align256((size_t)kStaticMaxTris * sizeof(Box));
constexpr size_t kSlotBytes = align256((size_t)kStaticMaxTris * 8);
constexpr size_t kDeltaBytes = align256((size_t)kStaticMaxTris + 16);
// scratch words: fixed part + look-back descriptors for the smallest sort tile (8 x 256 keys)
constexpr size_t kDescWords = (size_t)kMaxPasses * ((kStaticMaxTris + 2047) / 2048) * 256;
constexpr size_t kScratchBytes = align256((8 + 16 + 8 + 16 + (size_t)kBoundsBlocks * 8 + 16 + kMaxPasses * 256 +
                                           kDescWords + 64) * 4);
constexpr size_t kStaticBytes = 2 * kKeysBytes + kValsBytes + kBoxBytes + kSlotBytes + kDeltaBytes + kScratchBytes;

__device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
bool g_prepared[kMaxDevices] = {};          // kernel attributes set on this device
uint64_t g_epoch_builds[kMaxDevices] = {};  // builds on this device's array (clears its slots on epoch reuse)

// On every call, with the caller's device current: the array's device address (host code must
// not use the symbol itself, which is only a host-side stand-in).  The lookup is cheap and is
// not cached, so a module reloaded after cudaDeviceReset is found at its new address.  The
// kernels' attributes are set once per device (allocates nothing).
cudaError_t static_scratch(int device, unsigned char** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_prepared[device]) {
    e = prepare_kernels();
    if (e != cudaSuccess) return e;
    g_prepared[device] = true;
  }
  *out = static_cast<unsigned char*>(p);
  return cudaSuccess;
}

}  // namespace

extern "C" bvh_status bvh_build_lbvh_static(const bvh_mesh_soa* mesh, int32_t morton_bits, bvh_node* nodes,
                                            uint32_t* indices, void* stream) {
  if (!mesh || (morton_bits != 30 && morton_bits != 60 && morton_bits != 63)) return BVH_ERR_INVALID_ARG;
  const uint32_t n = mesh->n;
  if (n == 0) return BVH_OK;
  if (n > kStaticMaxTris || !nodes || !indices) return BVH_ERR_INVALID_ARG;
  const float* v[9] = {mesh->v0x, mesh->v0y, mesh->v0z, mesh->v1x, mesh->v1y, mesh->v1z,
                       mesh->v2x, mesh->v2y, mesh->v2z};
  MeshPtrs m;
  for (int k = 0; k < 9; ++k) {
    if (!v[k]) return BVH_ERR_INVALID_ARG;
    m.v[k] = v[k];
  }
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return BVH_ERR_DEVICE;
  unsigned char* base = nullptr;
  if (static_scratch(device, &base) != cudaSuccess) return BVH_ERR_DEVICE;
  // A workspace view over the static array and the caller's outputs: the radix sort's last pass
  // writes the sorted indices into `indices` (an even number of passes ends in buffer 0) and the
  // emission writes `nodes`.  Slots are epoch-tagged and the per-build scratch is cleared by the
  // first kernel, so nothing left from the previous call needs clearing here.
  Workspace ws;
  size_t o = 0;
  ws.keys[0] = base + o; o += kKeysBytes;
  ws.keys[1] = base + o; o += kKeysBytes;
  ws.vals[0] = indices;
  ws.vals[1] = reinterpret_cast<uint32_t*>(base + o); o += kValsBytes;
  ws.boxes = reinterpret_cast<Box*>(base + o); o += kBoxBytes;
  ws.slots = reinterpret_cast<unsigned long long*>(base + o); o += kSlotBytes;
  ws.delta = base + o; o += kDeltaBytes;
  ws.scratch = reinterpret_cast<uint32_t*>(base + o);
  ws.nodes = reinterpret_cast<Node*>(nodes);
  ws.cap_n = kStaticMaxTris;
  ws.scratch_words = kScratchBytes / 4;
  if (scratch_layout(kStaticMaxTris).total > ws.scratch_words) return BVH_ERR_DEVICE;  // layout guard
  uint32_t* out_idx = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    ws.epoch_builds = g_epoch_builds[device];
    g_epoch_builds[device] = ws.epoch_builds + 1;
  }
  ws.sort_variant = default_sort_variant(n);
  cudaError_t e = lbvh_build(ws, m, n, morton_bits, 0, reinterpret_cast<cudaStream_t>(stream), nullptr, &out_idx);
  if (e != cudaSuccess) return BVH_ERR_DEVICE;
  return out_idx == indices ? BVH_OK : BVH_ERR_DEVICE;
}
