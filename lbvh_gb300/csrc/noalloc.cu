// Allocation-free triangle build: lbvh_build_triangles_noalloc.
//
// Who needs this: some callers cannot allocate device memory at the point
// where they want a BVH -- a real-time render or simulation loop that sizes
// every buffer at start-up and forbids cudaMalloc on its frame path (cudaMalloc
// can synchronize the device and take milliseconds), a plugin running inside
// a host application that owns the GPU memory budget and hands the plugin
// only fixed buffers, or a process whose device memory is already held by
// another framework's caching allocator. They pass the triangles and the node
// array; everything else the build needs lives in one file-scope device array
// below.
//
// The scratch array is fixed at kNoAllocMaxPrims primitives (about 1.5 MB).
// Every GPU that loads this library reserves it until the process exits.
// All calls on a device share it and it keeps the last call's contents, so
// each call clears, in stream order, everything a build expects to start
// empty: the build counters and the error word, the radix sort's look-back
// words and the tree's arrival slots for this call's size. Nothing carries
// over from one call to the next, so a call's result depends only on its own
// inputs. Calls whose work overlaps on the GPU -- two streams, or two host
// threads -- race on the array and corrupt each other's results: serialize
// them per device.
//
// Set-up: the first call on each device looks the array's device address up
// with cudaGetSymbolAddress (the array's name in host code is only a host-side
// stand-in, not a device address) and keeps it for the life of the process.
// Make that first call before capturing any stream. A cudaDeviceReset ends
// the context that address belongs to: do not call this entry point on that
// device again in the same process.
#include "../../include/lbvh_gb300.h"

#include "build.cuh"

#include <mutex>

using namespace lbvh_gb300;

namespace {

constexpr size_t kNoAllocMaxPrims = LBVH_NOALLOC_MAX_PRIMS;
constexpr size_t kAlign = 256;

constexpr size_t
round_up(size_t x)
{
  return (x + kAlign - 1) / kAlign * kAlign;
}

constexpr size_t kTiles = sort_tiles(kNoAllocMaxPrims);
constexpr size_t kBoundsBlocksMax = (kNoAllocMaxPrims + kBoundsThreads * 8 - 1) / (kBoundsThreads * 8);
// scratch layout (byte offsets)
constexpr size_t kOffState = 0;
constexpr size_t kOffPartials = kOffState + round_up(sizeof(BuildState));
constexpr size_t kOffKeysA = kOffPartials + round_up(kBoundsBlocksMax * 48);
constexpr size_t kOffKeysB = kOffKeysA + round_up(4 * kNoAllocMaxPrims);
constexpr size_t kOffLookback = kOffKeysB + round_up(4 * kNoAllocMaxPrims);
constexpr size_t kOffSlots = kOffLookback + round_up(kTiles * 256 * 8);
constexpr size_t kOffPending = kOffSlots + round_up(8 * kNoAllocMaxPrims);
constexpr size_t kScratchBytes = kOffPending + round_up(tree_scratch(kNoAllocMaxPrims).bytes);

// The scratch memory of every allocation-free build on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

struct DeviceSlot
{
  std::once_flag once;
  cudaError_t setup_error = cudaSuccess;
  unsigned char* scratch = nullptr; // device address of g_noalloc_scratch
  int num_sms = 1;
};

DeviceSlot g_slots[kMaxDevices];

// Tag of the look-back words (kEpoch + pass) and arrival slots (kEpoch) of
// every call. Both are cleared at the start of each call, so a fixed tag
// never meets a word left by an earlier call; it only has to differ from
// the cleared value 0 and keep the sort's four passes apart.
constexpr uint32_t kEpoch = 4;

bool
is_device_pointer(const void* p, int device)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) &&
         (a.type == cudaMemoryTypeManaged || a.device == device);
}

} // namespace

extern "C" int
lbvh_build_triangles_noalloc(const float* d_tris, size_t n, void* d_nodes, uint32_t* d_status, void* stream)
{
  if (!d_tris || !d_nodes)
    return LBVH_ERR_INVALID_ARG;
  if (n < 2 || n > kNoAllocMaxPrims)
    return LBVH_ERR_INVALID_ARG; // beyond the fixed scratch: use lbvh_build_triangles
  if ((reinterpret_cast<uintptr_t>(d_tris) & 15) || (reinterpret_cast<uintptr_t>(d_nodes) & 31))
    return LBVH_ERR_INVALID_ARG;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
    cudaGetLastError();
    return LBVH_ERR_DEVICE;
  }
  if (!is_device_pointer(d_tris, device) || !is_device_pointer(d_nodes, device) ||
      (d_status && !is_device_pointer(d_status, device)))
    return LBVH_ERR_INVALID_ARG; // host memory would need staging buffers

  DeviceSlot& slot = g_slots[device];
  std::call_once(slot.once, [&slot, device]() {
    // runs with `device` current (the caller's current device)
    void* p = nullptr;
    slot.setup_error = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (slot.setup_error == cudaSuccess) {
      slot.scratch = static_cast<unsigned char*>(p);
      slot.setup_error = cudaDeviceGetAttribute(&slot.num_sms, cudaDevAttrMultiProcessorCount, device);
    }
    if (slot.setup_error != cudaSuccess)
      cudaGetLastError();
  });
  if (slot.setup_error != cudaSuccess || !slot.scratch)
    return LBVH_ERR_DEVICE;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = slot.scratch;
  const uint32_t nn = uint32_t(n);
  BuildBuffers b{};
  b.state = reinterpret_cast<BuildState*>(base + kOffState);
  b.partials = base + kOffPartials;
  b.keys_a = reinterpret_cast<uint32_t*>(base + kOffKeysA);
  b.keys_b = reinterpret_cast<uint32_t*>(base + kOffKeysB);
  b.vals_a = nullptr; // parity build: key-only sort
  b.vals_b = nullptr;
  b.lookback = reinterpret_cast<unsigned long long*>(base + kOffLookback);
  b.child = nullptr; // refit links: not used by a build
  b.leaf_parent = nullptr;
  b.node_parent = nullptr;
  b.slots = reinterpret_cast<unsigned long long*>(base + kOffSlots);
  b.pending = base + kOffPending;
  const uint32_t want = (nn + kBoundsThreads * 8 - 1) / (kBoundsThreads * 8);
  const uint32_t cap = uint32_t(slot.num_sms) * 4;
  b.bounds_blocks = want < 1 ? 1 : (want > cap ? cap : want);
  const uint32_t mwant = (nn + kMortonThreads - 1) / kMortonThreads;
  const uint32_t mcap = uint32_t(slot.num_sms) * 8;
  b.morton_blocks = mwant < 1 ? 1 : (mwant > mcap ? mcap : mwant);

  // What must start at zero, cleared by every call: the bounds/sort
  // counters and the error word, the look-back words of this size's sort
  // tiles, and the arrival slots of its n - 1 split positions.
  cudaError_t e = cudaMemsetAsync(b.state, 0, sizeof(BuildState), s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(b.lookback, 0, sort_tiles(nn) * 256 * 8, s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(b.slots, 0, 8 * size_t(nn - 1), s);
  if (e == cudaSuccess)
    e = launch_curve_tris(reinterpret_cast<const Tri*>(d_tris), nn, b, s);
  if (e == cudaSuccess)
    e = launch_sort(nn, false, kEpoch, b, s);
  if (e == cudaSuccess)
    e = launch_fit_tris(reinterpret_cast<const Tri*>(d_tris), nn, b, static_cast<Node*>(d_nodes), kEpoch, s);
  if (e == cudaSuccess && d_status)
    e = cudaMemcpyAsync(d_status, &b.state->error, 4, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return LBVH_ERR_DEVICE;
  }
  return LBVH_OK;
}
