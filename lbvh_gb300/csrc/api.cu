// C ABI (include/lbvh_gb300.h): contexts, workspace, BVH handles, and the
// build / refit / trace entry points that replace the reference's
// lbvh::builder<float>, lbvh::bvh<float> and lbvh::traverser.
#include "../../include/lbvh_gb300.h"

#include "batch.cuh"
#include "build.cuh"
#include "trace.cuh"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

using namespace lbvh_gb300;

namespace {

struct DevBuf
{
  void* ptr = nullptr;
  size_t cap = 0;
};

size_t
align_up(size_t x, size_t a)
{
  return (x + a - 1) / a * a;
}

} // namespace

struct lbvh_ctx
{
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 1;
  BuildState* state = nullptr; // persistent: holds the sticky error word
  uint32_t* h_err = nullptr;   // pinned readback of state->error
  DevBuf ws;                   // build workspace arena
  size_t ws_prims = 0;         // primitives the arena is laid out for
  BuildBuffers bufs{};
  DevBuf slots;                // tree arrival slots (epoch-tagged, persistent)
  DevBuf lookback;             // radix sort look-back words (epoch-tagged)
  DevBuf rays;                 // staging for host rays
  DevBuf hits;                 // staging for host hits
  DevBuf counts;               // staging for host per-ray counts
  DevBuf ray_sort;             // ray order: keys and indices, two of each (16 B per ray)
  uint32_t ray_order = 0;      // LBVH_PARAM_TRACE_RAY_ORDER
  DevBuf prims_in;             // staging for host refit input
  DevBuf roff;                 // staging for host batch ray offsets
  uint32_t* ray_counter = nullptr; // persistent-trace ray dispenser
  // host-pointer traces in chunks: uploads on copy_in and downloads on
  // copy_out overlap the traversal on `stream` (made on first use)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in = nullptr, ev_kernel = nullptr, ev_out = nullptr;
  size_t trace_chunk = size_t(1) << 20; // rays per chunk of a host-pointer trace (0: one piece)
  int trace_in_place = 2;               // LBVH_PARAM_TRACE_IN_PLACE
  TraceParams trace;               // traversal launch shape
  uint32_t batch_threads = 512;    // CTA size of the batched build
  uint32_t batch_radix_bits = 8;   // digit width of the batched build's CTA-local sort
  uint32_t batch_items = 4;        // keys per thread of its ranked chunks
  uint32_t tile_keys = 0;          // keys-only sort tile (0: by size)
  uint32_t msd_min = kMsdMinPrims; // keys-only builds from this size use the bucket sort
  uint32_t bounds_per_sm = 4;      // bounds-pass CTAs per SM
  uint32_t walk_fused = 0;         // 1: CTA-edge walks from the local tree phase's tail, 0: separate kernel
  uint32_t small_max = kSmallMaxPrims; // keys-only builds up to this size run as one cluster launch
  DevBuf batch_ws;                 // batched build: codes, boxes, slots
  uint32_t epoch = 0;          // look-back epoch of the last sort pass
  char msg[512] = { 0 };
};

struct lbvh_bvh
{
  int device = 0;
  uint32_t n = 0;
  uint32_t flags = 0;
  int kind = 0; // 1 triangles, 2 boxes
  DevBuf nodes;
  const void* prims = nullptr; // primitives in input order (borrowed or owned)
  DevBuf prims_owned;
  DevBuf sorted_prims;         // sorted-leaf mode: primitives in leaf order
  DevBuf leaf_prim;            // sorted-leaf mode: leaf slot -> primitive id
  DevBuf curve;                // keep-curve: codes, sorted codes, perm, bounds
  DevBuf wnodes;               // traversal copy (WideNode per internal node)
  bool wnodes_valid = false;   // false after every build / refit
  DevBuf codes;                // the build's sorted Morton codes (the sort's output)
  bool codes_valid = false;    // a refit can rerun the tree phase over them
};

namespace {

constexpr int kKindTris = 1;
constexpr int kKindBoxes = 2;

int
fail(lbvh_ctx* c, int status, const char* fmt, ...)
{
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->msg, sizeof(c->msg), fmt, ap);
    va_end(ap);
  }
  return status;
}

int
cuda_fail(lbvh_ctx* c, cudaError_t e, const char* what)
{
  const int st = (e == cudaErrorMemoryAllocation) ? LBVH_ERR_OOM : LBVH_ERR_DEVICE;
  cudaGetLastError();
  return fail(c, st, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                                                             \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return cuda_fail(c, e_, what);                                                               \
  } while (0)

bool
on_device(const void* p)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The device address of page-locked host memory (cudaHostAlloc'd or
// registered), or null for anything else.
void*
mapped_host(const void* p)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Grow-only stream-ordered buffer.
cudaError_t
reserve(DevBuf& b, size_t bytes, cudaStream_t s, bool* grew = nullptr)
{
  if (grew)
    *grew = false;
  if (b.cap >= bytes)
    return cudaSuccess;
  if (b.ptr) {
    cudaError_t e = cudaFreeAsync(b.ptr, s);
    b.ptr = nullptr;
    b.cap = 0;
    if (e != cudaSuccess)
      return e;
  }
  const size_t want = align_up(bytes, 1 << 16);
  cudaError_t e = cudaMallocAsync(&b.ptr, want, s);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    return e;
  }
  b.cap = want;
  if (grew)
    *grew = true;
  return cudaSuccess;
}

void
release(DevBuf& b, cudaStream_t s)
{
  if (b.ptr)
    cudaFreeAsync(b.ptr, s);
  b.ptr = nullptr;
  b.cap = 0;
}

// One primitive per thread up to 4 CTAs per SM: a thread's primitives are
// loaded one after another, so at small sizes every extra primitive per
// thread adds a memory round trip to the kernel.
uint32_t
bounds_blocks_for(const lbvh_ctx* c, uint32_t n)
{
  const uint32_t want = ceil_div_u32(n, kBoundsThreads);
  const uint32_t cap = uint32_t(c->num_sms) * c->bounds_per_sm;
  return want < 1 ? 1 : (want > cap ? cap : want);
}

uint32_t
morton_blocks_for(const lbvh_ctx* c, uint32_t n)
{
  const uint32_t want = ceil_div_u32(n, kMortonThreads);
  const uint32_t cap = uint32_t(c->num_sms) * 8;
  return want < 1 ? 1 : (want > cap ? cap : want);
}

// Lays out the build arena for n primitives and the arrival flags.
int
ws_reserve(lbvh_ctx* c, size_t n)
{
  const size_t tiles = sort_tiles_any(n);
  const size_t A = 256;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, A);
    return o;
  };
  const size_t o_part = take(size_t(c->num_sms) * kMaxBoundsBlocksPerSm * 48);
  const size_t o_ka = take(4 * n);
  const size_t o_kb = take(4 * n);
  const size_t o_va = take(4 * n);
  const size_t o_vb = take(4 * n);
  const size_t o_child = take(8 * n);
  const size_t o_lp = take(4 * n);
  const size_t o_np = take(4 * n);
  const size_t o_pend = take(tree_scratch(n).bytes);
  const size_t o_boxes = take(24 * n);
  CK(reserve(c->ws, off, c->stream), "workspace allocation");
  // The look-back buffer only ever holds look-back words: fresh words read as
  // "not published" (epoch 0 is never used), so it is cleared only on growth.
  bool grew = false;
  CK(reserve(c->lookback, tiles * 256 * 8, c->stream, &grew), "look-back allocation");
  if (grew)
    CK(cudaMemsetAsync(c->lookback.ptr, 0, c->lookback.cap, c->stream), "look-back clear");
  // Like the look-back words, slots carry the epoch of the build that wrote
  // them, so they are cleared only when (re)allocated.
  grew = false;
  CK(reserve(c->slots, 8 * n, c->stream, &grew), "slot allocation");
  if (grew)
    CK(cudaMemsetAsync(c->slots.ptr, 0, c->slots.cap, c->stream), "slot clear");
  char* base = static_cast<char*>(c->ws.ptr);
  BuildBuffers& b = c->bufs;
  b.state = c->state;
  b.partials = base + o_part;
  b.keys_a = reinterpret_cast<uint32_t*>(base + o_ka);
  b.keys_b = reinterpret_cast<uint32_t*>(base + o_kb);
  b.vals_a = reinterpret_cast<uint32_t*>(base + o_va);
  b.vals_b = reinterpret_cast<uint32_t*>(base + o_vb);
  b.lookback = static_cast<unsigned long long*>(c->lookback.ptr);
  b.child = reinterpret_cast<uint2*>(base + o_child);
  b.leaf_parent = reinterpret_cast<uint32_t*>(base + o_lp);
  b.node_parent = reinterpret_cast<uint32_t*>(base + o_np);
  b.pending = base + o_pend;
  b.boxes = reinterpret_cast<Box*>(base + o_boxes);
  b.slots = static_cast<unsigned long long*>(c->slots.ptr);
  c->ws_prims = n;
  return LBVH_OK;
}

// Next epoch base: the four sort passes use base .. base + 3 for their
// look-back words, the tree build or refit uses base for its slots. Epoch 0
// means "never written"; on wrap-around both buffers are cleared.
int
next_epoch(lbvh_ctx* c, uint32_t* base)
{
  if (c->epoch == 0 || c->epoch > 0xfffffff0u) {
    if (c->epoch != 0 && c->lookback.ptr)
      CK(cudaMemsetAsync(c->lookback.ptr, 0, c->lookback.cap, c->stream), "look-back clear");
    if (c->epoch != 0 && c->slots.ptr)
      CK(cudaMemsetAsync(c->slots.ptr, 0, c->slots.cap, c->stream), "slot clear");
    c->epoch = 4;
  }
  *base = c->epoch;
  c->epoch += 4;
  return LBVH_OK;
}

// The trace order of m device rays (LBVH_PARAM_TRACE_RAY_ORDER): their
// sort keys (origin cell above direction cell), then the stable pairs sort
// the builds use; *order gets the ray indices in key order.
int
order_rays(lbvh_ctx* c, const lbvh_bvh* b, const float* rays, uint32_t m, const uint32_t** order)
{
  const size_t tiles = sort_tiles_any(m);
  bool grew = false;
  CK(reserve(c->lookback, tiles * 256 * 8, c->stream, &grew), "look-back allocation");
  if (grew)
    CK(cudaMemsetAsync(c->lookback.ptr, 0, c->lookback.cap, c->stream), "look-back clear");
  CK(reserve(c->ray_sort, 16 * size_t(m), c->stream), "ray order allocation");
  BuildBuffers rb = c->bufs;
  uint32_t* base = static_cast<uint32_t*>(c->ray_sort.ptr);
  rb.keys_a = base;
  rb.keys_b = base + m;
  rb.vals_a = base + 2 * size_t(m);
  rb.vals_b = base + 3 * size_t(m);
  rb.lookback = static_cast<unsigned long long*>(c->lookback.ptr);
  rb.msd = false;
  // the sort's digit histograms and tile dispensers start at zero (a build
  // resets them itself)
  CK(cudaMemsetAsync(&c->state->hist[0][0], 0, sizeof(c->state->hist) + sizeof(c->state->tile_counter), c->stream),
     "ray order state reset");
  uint32_t epoch;
  int st = next_epoch(c, &epoch);
  if (st)
    return st;
  CK(launch_ray_keys(rays, m, static_cast<const Node*>(b->nodes.ptr), rb.keys_a, c->state, c->stream),
     "ray key launch");
  CK(launch_sort(m, true, epoch, rb, c->stream, 3), "ray sort launch"); // 24-bit keys: three passes
  *order = rb.vals_b;
  return LBVH_OK;
}

// Reads and clears the sticky device error word after a stream sync.
int
check_device(lbvh_ctx* c)
{
  CK(cudaMemcpyAsync(c->h_err, &c->state->error, 4, cudaMemcpyDeviceToHost, c->stream), "status read");
  CK(cudaStreamSynchronize(c->stream), "stream synchronize");
  const uint32_t err = *c->h_err;
  if (!err)
    return LBVH_OK;
  CK(cudaMemsetAsync(&c->state->error, 0, 4, c->stream), "status clear");
  CK(cudaMemsetAsync(c->state, 0, offsetof(BuildState, error), c->stream), "state clear");
  CK(cudaStreamSynchronize(c->stream), "stream synchronize");
  if (err & kErrLookbackTimeout)
    return fail(c, LBVH_ERR_TIMEOUT, "radix sort look-back wait expired");
  return fail(c, LBVH_ERR_BAD_TOPOLOGY, "node array is not a binary tree over its leaves");
}

int
set_device(lbvh_ctx* c)
{
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  return LBVH_OK;
}

// Refits of at least this many primitives rerun the tree phase over the
// build's sorted codes; smaller ones walk the node links.
constexpr uint32_t kRefitFromCodesMin = 1u << 19;

int build_multi(lbvh_ctx* c, BuildBuffers& b, const void* dprims, uint32_t nn, uint32_t flags, lbvh_bvh* bvh,
                int kind, Node* nodes);

// Shared build body for triangles and boxes.
int
build_common(lbvh_ctx* c, const float* prims, size_t n, uint32_t flags, lbvh_bvh* bvh, int kind)
{
  if (!c || !prims || !bvh)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (n < 2 || n > kMaxPrims)
    return fail(c, LBVH_ERR_INVALID_ARG, "primitive count %zu outside [2, %u]", n, kMaxPrims);
  if (flags & ~(LBVH_BUILD_SORTED_LEAVES | LBVH_BUILD_KEEP_CURVE))
    return fail(c, LBVH_ERR_INVALID_ARG, "unknown build flags 0x%x", flags);
  int st = set_device(c);
  if (st)
    return st;
  const uint32_t nn = uint32_t(n);
  const size_t rec = (kind == kKindTris) ? sizeof(Tri) : sizeof(Box);

  const void* dprims = prims;
  if (!on_device(prims)) {
    CK(reserve(bvh->prims_owned, rec * n, c->stream), "primitive allocation");
    CK(cudaMemcpyAsync(bvh->prims_owned.ptr, prims, rec * n, cudaMemcpyHostToDevice, c->stream), "primitive upload");
    dprims = bvh->prims_owned.ptr;
  }
  if (kind == kKindTris && (reinterpret_cast<uintptr_t>(dprims) & 15))
    return fail(c, LBVH_ERR_INVALID_ARG, "device triangles must be 16-byte aligned");
  if (kind == kKindBoxes && (reinterpret_cast<uintptr_t>(dprims) & 7))
    return fail(c, LBVH_ERR_INVALID_ARG, "device boxes must be 8-byte aligned");

  if ((st = ws_reserve(c, n)))
    return st;
  CK(reserve(bvh->nodes, sizeof(Node) * (n - 1), c->stream), "node allocation");
  CK(reserve(bvh->codes, 4 * n, c->stream), "code allocation");
  bvh->codes_valid = false;
  // this build's buffers: the context workspace, except that the codes are
  // sorted into the BVH's own buffer (the sort ends in keys_a), where a refit
  // finds them
  BuildBuffers b = c->bufs;
  b.keys_a = static_cast<uint32_t*>(bvh->codes.ptr);
  b.bounds_blocks = bounds_blocks_for(c, nn);
  b.morton_blocks = morton_blocks_for(c, nn);
  const bool keep = flags & LBVH_BUILD_KEEP_CURVE;
  const bool sorted_leaves = flags & LBVH_BUILD_SORTED_LEAVES;
  b.msd = !keep && !sorted_leaves && nn >= c->msd_min; // keys-only sort of a large build
  b.tile_keys = c->tile_keys;
  b.walk_fused = c->walk_fused;
  if (b.msd) {
    // ranges of at least 8,192 codes, a few per SM; their count rows
    // (ranges x 16 KB <= 2n + 16 KB) live in vals_a, unused by keys-only sorts
    const uint32_t want = std::min(uint32_t(c->num_sms) * 8, ceil_div_u32(nn, 8192u));
    b.msd_range = (ceil_div_u32(nn, want) + 255u) & ~255u;
    b.msd_ranges = ceil_div_u32(nn, b.msd_range);
    // the partition: about one CTA per SM (its 160 KB of shared memory allow
    // no second), each over `group` whole ranges
    b.msd_group = ceil_div_u32(b.msd_ranges, uint32_t(c->num_sms));
    b.sort_ctas = uint32_t(c->num_sms);
    b.top_rows = b.vals_a;
  }

  Node* nodes = static_cast<Node*>(bvh->nodes.ptr);
  const bool small = !keep && !sorted_leaves && nn <= c->small_max && nn <= small_build_limit();
  if (small) { // the whole build in one cluster launch
    if (kind == kKindTris)
      CK(launch_small_build_tris(static_cast<const Tri*>(dprims), nn, b.keys_a, nodes, c->state, c->stream),
         "build launch");
    else
      CK(launch_small_build_boxes(static_cast<const Box*>(dprims), nn, b.keys_a, nodes, c->state, c->stream),
         "build launch");
  } else {
    if ((st = build_multi(c, b, dprims, nn, flags, bvh, kind, nodes)))
      return st;
  }
  bvh->n = nn;
  bvh->flags = flags;
  bvh->kind = kind;
  bvh->wnodes_valid = false;
  bvh->codes_valid = true;
  bvh->prims = dprims;
  bvh->device = c->device;
  if (!on_device(prims))
    return check_device(c); // host caller: finish and report before returning
  return LBVH_OK;
}

// The multi-kernel build: bounds + codes, the sort, the tree phases.
int
build_multi(lbvh_ctx* c, BuildBuffers& b, const void* dprims, uint32_t nn, uint32_t flags, lbvh_bvh* bvh, int kind,
            Node* nodes)
{
  int st = LBVH_OK;
  const size_t n = nn;
  const size_t rec = (kind == kKindTris) ? sizeof(Tri) : sizeof(Box);
  const bool keep = flags & LBVH_BUILD_KEEP_CURVE;
  const bool sorted_leaves = flags & LBVH_BUILD_SORTED_LEAVES;
  if (kind == kKindTris)
    CK(launch_curve_tris(static_cast<const Tri*>(dprims), nn, b, c->stream), "curve launch");
  else
    CK(launch_curve_boxes(static_cast<const Box*>(dprims), nn, b, c->stream), "curve launch");

  uint32_t* curve = nullptr;
  if (keep) {
    CK(reserve(bvh->curve, 12 * n + 64, c->stream), "curve allocation");
    curve = static_cast<uint32_t*>(bvh->curve.ptr);
    CK(cudaMemcpyAsync(curve, b.keys_a, 4 * n, cudaMemcpyDeviceToDevice, c->stream), "curve copy");
    CK(cudaMemcpyAsync(curve + 3 * n, c->state, 24, cudaMemcpyDeviceToDevice, c->stream), "bounds copy");
  }
  uint32_t epoch;
  if ((st = next_epoch(c, &epoch)))
    return st;
  CK(launch_sort(nn, keep || sorted_leaves, epoch, b, c->stream), "sort launch");
  if (keep) {
    CK(cudaMemcpyAsync(curve + n, b.keys_a, 4 * n, cudaMemcpyDeviceToDevice, c->stream), "curve copy");
    CK(cudaMemcpyAsync(curve + 2 * n, b.vals_a, 4 * n, cudaMemcpyDeviceToDevice, c->stream), "curve copy");
  }
  if (sorted_leaves) {
    CK(reserve(bvh->sorted_prims, rec * n, c->stream), "sorted primitive allocation");
    CK(reserve(bvh->leaf_prim, 4 * n, c->stream), "leaf map allocation");
    CK(cudaMemcpyAsync(bvh->leaf_prim.ptr, b.vals_a, 4 * n, cudaMemcpyDeviceToDevice, c->stream), "leaf map copy");
    if (kind == kKindTris) {
      Tri* sp = static_cast<Tri*>(bvh->sorted_prims.ptr);
      CK(launch_gather_tris(static_cast<const Tri*>(dprims), b.vals_a, nn, sp, c->stream), "gather launch");
      CK(launch_fit_tris(sp, nn, b, nodes, epoch, c->stream), "fit launch");
    } else {
      Box* sp = static_cast<Box*>(bvh->sorted_prims.ptr);
      CK(launch_gather_boxes(static_cast<const Box*>(dprims), b.vals_a, nn, sp, c->stream), "gather launch");
      CK(launch_fit_boxes(sp, nn, b, nodes, epoch, c->stream), "fit launch");
    }
  } else {
    if (kind == kKindTris)
      CK(launch_fit_staged(nn, b, nodes, epoch, c->stream), "fit launch");
    else
      CK(launch_fit_boxes(static_cast<const Box*>(dprims), nn, b, nodes, epoch, c->stream), "fit launch");
  }
  return st;
}

int
refit_common(lbvh_ctx* c, lbvh_bvh* bvh, const float* prims, int kind)
{
  if (!c || !bvh || !prims)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (bvh->n < 2 || bvh->kind != kind)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH was not built from this primitive kind");
  int st = set_device(c);
  if (st)
    return st;
  const uint32_t n = bvh->n;
  const size_t rec = (kind == kKindTris) ? sizeof(Tri) : sizeof(Box);
  const bool host = !on_device(prims);
  const void* dprims = prims;
  if (host) {
    CK(reserve(bvh->prims_owned, rec * n, c->stream), "primitive allocation");
    CK(cudaMemcpyAsync(bvh->prims_owned.ptr, prims, rec * n, cudaMemcpyHostToDevice, c->stream), "primitive upload");
    dprims = bvh->prims_owned.ptr;
  }
  if ((st = ws_reserve(c, n)))
    return st;
  uint32_t epoch;
  if ((st = next_epoch(c, &epoch)))
    return st;
  Node* nodes = static_cast<Node*>(bvh->nodes.ptr);
  if (bvh->codes_valid && n >= kRefitFromCodesMin) {
    // The build's sorted codes determine the topology: rerun its tree phase
    // (the same nodes, the same fit order) over the moved primitives. Its
    // merge-fallback flag is reset here, as the bounds pass does in a build.
    // (Measured: 0.59 against 1.19 ms at 16M triangles, 0.100 against 0.115
    // ms at 2^20; below 2^19 the walk over the links is the faster.)
    BuildBuffers b = c->bufs;
    b.keys_a = static_cast<uint32_t*>(bvh->codes.ptr);
    CK(cudaMemsetAsync(&c->state->tree_fallback, 0, 4, c->stream), "state reset");
    const Tri* tris = static_cast<const Tri*>(dprims);
    const Box* boxes = static_cast<const Box*>(dprims);
    if (bvh->flags & LBVH_BUILD_SORTED_LEAVES) {
      const uint32_t* perm = static_cast<const uint32_t*>(bvh->leaf_prim.ptr);
      if (kind == kKindTris) {
        Tri* sp = static_cast<Tri*>(bvh->sorted_prims.ptr);
        CK(launch_gather_tris(tris, perm, n, sp, c->stream), "gather launch");
        tris = sp;
      } else {
        Box* sp = static_cast<Box*>(bvh->sorted_prims.ptr);
        CK(launch_gather_boxes(boxes, perm, n, sp, c->stream), "gather launch");
        boxes = sp;
      }
    }
    if (kind == kKindTris)
      CK(launch_fit_tris(tris, n, b, nodes, epoch, c->stream), "refit launch");
    else
      CK(launch_fit_boxes(boxes, n, b, nodes, epoch, c->stream), "refit launch");
  } else if (bvh->flags & LBVH_BUILD_SORTED_LEAVES) {
    // a tree without its codes (loaded from nodes): bottom-up over the links
    const uint32_t* perm = static_cast<const uint32_t*>(bvh->leaf_prim.ptr);
    if (kind == kKindTris) {
      Tri* sp = static_cast<Tri*>(bvh->sorted_prims.ptr);
      CK(launch_gather_tris(static_cast<const Tri*>(dprims), perm, n, sp, c->stream), "gather launch");
      CK(launch_refit_tris(sp, n, c->bufs, nodes, epoch, c->stream), "refit launch");
    } else {
      Box* sp = static_cast<Box*>(bvh->sorted_prims.ptr);
      CK(launch_gather_boxes(static_cast<const Box*>(dprims), perm, n, sp, c->stream), "gather launch");
      CK(launch_refit_boxes(sp, n, c->bufs, nodes, epoch, c->stream), "refit launch");
    }
  } else if (kind == kKindTris) {
    CK(launch_refit_tris(static_cast<const Tri*>(dprims), n, c->bufs, nodes, epoch, c->stream), "refit launch");
  } else {
    CK(launch_refit_boxes(static_cast<const Box*>(dprims), n, c->bufs, nodes, epoch, c->stream), "refit launch");
  }
  bvh->prims = dprims;
  bvh->wnodes_valid = false;
  if (host)
    return check_device(c);
  return LBVH_OK;
}

} // namespace

extern "C" {

int
lbvh_version(void)
{
  return 100;
}

const char*
lbvh_status_string(int s)
{
  switch (s) {
    case LBVH_OK:
      return "ok";
    case LBVH_ERR_INVALID_ARG:
      return "invalid argument";
    case LBVH_ERR_OOM:
      return "out of device memory";
    case LBVH_ERR_TIMEOUT:
      return "device wait timed out";
    case LBVH_ERR_DEVICE:
      return "CUDA error";
    case LBVH_ERR_BAD_TOPOLOGY:
      return "malformed tree";
    case LBVH_ERR_NOT_RESIDENT:
      return "scene not resident";
    case LBVH_ERR_BUDGET:
      return "larger than the HBM budget";
    case LBVH_ERR_CANCELLED:
      return "cancelled";
    case LBVH_ERR_EXPIRED:
      return "expired in the queue";
    default:
      return "unknown status";
  }
}

int
lbvh_ctx_create(int device, void* stream, lbvh_ctx** out)
{
  if (!out)
    return LBVH_ERR_INVALID_ARG;
  *out = nullptr;
  lbvh_ctx* c = new (std::nothrow) lbvh_ctx;
  if (!c)
    return LBVH_ERR_OOM;
  c->device = device;
  auto bail = [&](cudaError_t e) {
    const int st = (e == cudaErrorMemoryAllocation) ? LBVH_ERR_OOM : LBVH_ERR_DEVICE;
    cudaGetLastError();
    if (c->h_err)
      cudaFreeHost(c->h_err);
    if (c->ray_counter)
      cudaFree(c->ray_counter);
    if (c->state)
      cudaFree(c->state);
    delete c;
    return st;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess)
    return bail(e);
  c->stream = static_cast<cudaStream_t>(stream); // NULL: the default stream
  if ((e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
    return bail(e);
  if ((e = cudaMalloc(&c->state, sizeof(BuildState))) != cudaSuccess)
    return bail(e);
  if ((e = cudaMemset(c->state, 0, sizeof(BuildState))) != cudaSuccess)
    return bail(e);
  if ((e = cudaMallocHost(&c->h_err, 64)) != cudaSuccess)
    return bail(e);
  if ((e = cudaMalloc(&c->ray_counter, 256)) != cudaSuccess)
    return bail(e);
  *out = c;
  return LBVH_OK;
}

int
lbvh_ctx_destroy(lbvh_ctx* c)
{
  if (!c)
    return LBVH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  release(c->ws, c->stream);
  release(c->slots, c->stream);
  release(c->lookback, c->stream);
  release(c->batch_ws, c->stream);
  release(c->rays, c->stream);
  release(c->hits, c->stream);
  release(c->counts, c->stream);
  release(c->prims_in, c->stream);
  release(c->roff, c->stream);
  cudaStreamSynchronize(c->stream);
  cudaFree(c->state);
  cudaFree(c->ray_counter);
  cudaFreeHost(c->h_err);
  for (cudaEvent_t e : { c->ev_in, c->ev_kernel, c->ev_out })
    if (e)
      cudaEventDestroy(e);
  for (cudaStream_t q : { c->copy_in, c->copy_out })
    if (q) {
      cudaStreamSynchronize(q);
      cudaStreamDestroy(q);
    }
  delete c;
  return LBVH_OK;
}

int
lbvh_ctx_synchronize(lbvh_ctx* c)
{
  if (!c)
    return LBVH_ERR_INVALID_ARG;
  int st = set_device(c);
  if (st)
    return st;
  return check_device(c);
}

const char*
lbvh_ctx_last_error(const lbvh_ctx* c)
{
  return c ? c->msg : "null context";
}

int
lbvh_ctx_reserve(lbvh_ctx* c, size_t n_prims, size_t n_rays)
{
  if (!c)
    return LBVH_ERR_INVALID_ARG;
  int st = set_device(c);
  if (st)
    return st;
  if (n_prims >= 2 && (st = ws_reserve(c, n_prims)))
    return st;
  if (n_rays) {
    CK(reserve(c->rays, 32 * n_rays, c->stream), "ray staging allocation");
    CK(reserve(c->hits, 16 * n_rays, c->stream), "hit staging allocation");
  }
  return LBVH_OK;
}

int
lbvh_ctx_set_param(lbvh_ctx* c, int param, int value)
{
  if (!c)
    return LBVH_ERR_INVALID_ARG;
  switch (param) {
    case LBVH_PARAM_TRACE_BLOCKS_PER_SM:
      if (value < 1 || value > 32)
        return fail(c, LBVH_ERR_INVALID_ARG, "trace blocks per SM %d outside [1, 32]", value);
      c->trace.blocks_per_sm = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_BATCH_THREADS:
      if (value < 256 || value > kBatchMaxThreads || value % 32)
        return fail(c, LBVH_ERR_INVALID_ARG, "batch CTA size %d: a multiple of 32 in [256, %d]", value,
                    kBatchMaxThreads);
      c->batch_threads = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TRACE_REFILL:
      if (value < 1 || value > 32)
        return fail(c, LBVH_ERR_INVALID_ARG, "refill threshold %d outside [1, 32]", value);
      c->trace.refill = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TRACE_CHUNK:
      if (value < 0)
        return fail(c, LBVH_ERR_INVALID_ARG, "trace chunk %d is negative", value);
      c->trace_chunk = size_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TRACE_IN_PLACE:
      if (value < 0 || value > 2)
        return fail(c, LBVH_ERR_INVALID_ARG, "trace in-place mode %d outside [0, 2]", value);
      c->trace_in_place = value;
      return LBVH_OK;
    case LBVH_PARAM_TRACE_LEAF_BATCH:
      if (value < 1 || value > 32)
        return fail(c, LBVH_ERR_INVALID_ARG, "leaf batch %d outside [1, 32]", value);
      c->trace.leaf_batch = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_BATCH_RADIX_BITS:
      if (value != 4 && value != 6 && value != 8)
        return fail(c, LBVH_ERR_INVALID_ARG, "batch radix width %d is not 4, 6 or 8 bits", value);
      c->batch_radix_bits = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_BATCH_KEYS_PER_THREAD:
      if (value != 4 && value != 8)
        return fail(c, LBVH_ERR_INVALID_ARG, "batch keys per thread %d is not 4 or 8", value);
      c->batch_items = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_SORT_TILE_KEYS:
      if (value != 0 && value != kSmallTile && value != kSortTile)
        return fail(c, LBVH_ERR_INVALID_ARG, "sort tile %d is not 0, %d or %d keys", value, kSmallTile, kSortTile);
      c->tile_keys = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_BUCKET_SORT_MIN:
      if (value < 65536)
        return fail(c, LBVH_ERR_INVALID_ARG, "bucket-sort threshold %d below 65536", value);
      c->msd_min = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_BOUNDS_BLOCKS_PER_SM:
      if (value < 1 || value > int(kMaxBoundsBlocksPerSm))
        return fail(c, LBVH_ERR_INVALID_ARG, "bounds CTAs per SM %d outside [1, %u]", value, kMaxBoundsBlocksPerSm);
      c->bounds_per_sm = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TREE_WALK_FUSED:
      if (value < 0 || value > 1)
        return fail(c, LBVH_ERR_INVALID_ARG, "fused tree walk %d is not 0 or 1", value);
      c->walk_fused = uint32_t(value);
      c->bufs.walk_fused = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_LOOKBACK_SPIN_LIMIT:
      if (value < 1 || value > (1 << 24))
        return fail(c, LBVH_ERR_INVALID_ARG, "look-back spin limit %d outside [1, 2^24]", value);
      c->bufs.spin_limit = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_SMALL_BUILD_MAX:
      if (value < 0 || value > int(kSmallMaxPrims))
        return fail(c, LBVH_ERR_INVALID_ARG, "one-launch build limit %d outside [0, %u]", value, kSmallMaxPrims);
      c->small_max = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TRACE_RAY_ORDER:
      if (value < 0 || value > 1)
        return fail(c, LBVH_ERR_INVALID_ARG, "ray order %d is not 0 or 1", value);
      c->ray_order = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TEST_TREE_MERGE_CAP:
      if (value < 0 || value > int(kMergeCap))
        return fail(c, LBVH_ERR_INVALID_ARG, "tree merge capacity %d outside [0, %u]", value, kMergeCap);
      c->bufs.merge_cap = uint32_t(value);
      return LBVH_OK;
    case LBVH_PARAM_TEST_LOOKBACK_STALL:
      if (value < 0 || value > 1)
        return fail(c, LBVH_ERR_INVALID_ARG, "look-back stall %d is not 0 or 1", value);
      c->bufs.wait_xor = value ? 0x80000000u : 0u; // a tag no tile publishes
      return LBVH_OK;
    default:
      return fail(c, LBVH_ERR_INVALID_ARG, "unknown parameter %d", param);
  }
}

int
lbvh_make_triangles(lbvh_ctx* c, const float* verts, size_t n, float* tris_out)
{
  if (!c || !verts || !tris_out)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (n > kMaxPrims)
    return fail(c, LBVH_ERR_INVALID_ARG, "triangle count %zu too large", n);
  int st = set_device(c);
  if (st)
    return st;
  if (n == 0)
    return LBVH_OK;
  const bool hin = !on_device(verts), hout = !on_device(tris_out);
  const float* dv = verts;
  float* dt = tris_out;
  if (hin) {
    CK(reserve(c->prims_in, 36 * n, c->stream), "staging allocation");
    CK(cudaMemcpyAsync(c->prims_in.ptr, verts, 36 * n, cudaMemcpyHostToDevice, c->stream), "vertex upload");
    dv = static_cast<const float*>(c->prims_in.ptr);
  }
  if (hout) {
    CK(reserve(c->hits, 48 * n, c->stream), "staging allocation");
    dt = static_cast<float*>(c->hits.ptr);
  } else if (reinterpret_cast<uintptr_t>(dt) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device triangle output must be 16-byte aligned");
  }
  CK(launch_make_triangles(dv, uint32_t(n), reinterpret_cast<Tri*>(dt), c->stream), "make_triangles launch");
  if (hout) {
    CK(cudaMemcpyAsync(tris_out, dt, 48 * n, cudaMemcpyDeviceToHost, c->stream), "triangle download");
    return check_device(c);
  }
  return hin ? check_device(c) : LBVH_OK;
}

int
lbvh_bvh_create(lbvh_ctx* c, lbvh_bvh** out)
{
  if (!c || !out)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  *out = new (std::nothrow) lbvh_bvh;
  if (!*out)
    return fail(c, LBVH_ERR_OOM, "host allocation failed");
  (*out)->device = c->device;
  return LBVH_OK;
}

int
lbvh_bvh_destroy(lbvh_ctx* c, lbvh_bvh* b)
{
  if (!c || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  set_device(c);
  release(b->nodes, c->stream);
  release(b->prims_owned, c->stream);
  release(b->sorted_prims, c->stream);
  release(b->leaf_prim, c->stream);
  release(b->curve, c->stream);
  release(b->wnodes, c->stream);
  release(b->codes, c->stream);
  delete b;
  return LBVH_OK;
}

int
lbvh_build_triangles(lbvh_ctx* c, const float* tris, size_t n, uint32_t flags, lbvh_bvh* bvh)
{
  return build_common(c, tris, n, flags, bvh, kKindTris);
}

int
lbvh_build_boxes(lbvh_ctx* c, const float* boxes, size_t n, uint32_t flags, lbvh_bvh* bvh)
{
  return build_common(c, boxes, n, flags, bvh, kKindBoxes);
}

int
lbvh_refit_triangles(lbvh_ctx* c, lbvh_bvh* bvh, const float* tris)
{
  return refit_common(c, bvh, tris, kKindTris);
}

int
lbvh_refit_boxes(lbvh_ctx* c, lbvh_bvh* bvh, const float* boxes)
{
  return refit_common(c, bvh, boxes, kKindBoxes);
}

int
lbvh_bvh_import_triangles(lbvh_ctx* c, const void* nodes, size_t n_nodes, const float* tris, lbvh_bvh* bvh)
{
  if (!c || !nodes || !tris || !bvh)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (n_nodes < 1 || n_nodes + 1 > kMaxPrims)
    return fail(c, LBVH_ERR_INVALID_ARG, "node count %zu outside [1, %u]", n_nodes, kMaxPrims - 1);
  int st = set_device(c);
  if (st)
    return st;
  const size_t n = n_nodes + 1;
  bvh->codes_valid = false; // a given node array: refits go over its links
  CK(reserve(bvh->nodes, sizeof(Node) * n_nodes, c->stream), "node allocation");
  CK(cudaMemcpyAsync(bvh->nodes.ptr, nodes, sizeof(Node) * n_nodes, cudaMemcpyDefault, c->stream), "node upload");
  const void* dprims = tris;
  if (!on_device(tris)) {
    CK(reserve(bvh->prims_owned, sizeof(Tri) * n, c->stream), "primitive allocation");
    CK(cudaMemcpyAsync(bvh->prims_owned.ptr, tris, sizeof(Tri) * n, cudaMemcpyHostToDevice, c->stream),
       "primitive upload");
    dprims = bvh->prims_owned.ptr;
  } else if (reinterpret_cast<uintptr_t>(tris) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device triangles must be 16-byte aligned");
  }
  if ((st = ws_reserve(c, n)))
    return st;
  CK(launch_validate(static_cast<const Node*>(bvh->nodes.ptr), uint32_t(n_nodes), c->bufs, c->stream),
     "validation launch");
  bvh->n = 0; // unusable until validated
  if ((st = check_device(c)))
    return st;
  bvh->n = uint32_t(n);
  bvh->flags = 0;
  bvh->kind = kKindTris;
  bvh->prims = dprims;
  bvh->device = c->device;
  bvh->wnodes_valid = false;
  return LBVH_OK;
}

int
lbvh_bvh_info(const lbvh_bvh* b, size_t* n_prims, size_t* n_nodes, uint32_t* flags)
{
  if (!b)
    return LBVH_ERR_INVALID_ARG;
  if (n_prims)
    *n_prims = b->n;
  if (n_nodes)
    *n_nodes = b->n ? b->n - 1 : 0;
  if (flags)
    *flags = b->flags;
  return LBVH_OK;
}

int
lbvh_bvh_nodes(lbvh_ctx* c, const lbvh_bvh* b, void* dst)
{
  if (!c || !b || !dst)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (b->n < 2)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH has not been built");
  int st = set_device(c);
  if (st)
    return st;
  const bool host = !on_device(dst);
  CK(cudaMemcpyAsync(dst, b->nodes.ptr, sizeof(Node) * (b->n - 1), cudaMemcpyDefault, c->stream), "node copy");
  return host ? check_device(c) : LBVH_OK;
}

int
lbvh_bvh_primitives(lbvh_ctx* c, const lbvh_bvh* b, void* dst)
{
  if (!c || !b || !dst)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (b->n < 2 || !b->prims)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH has not been built");
  int st = set_device(c);
  if (st)
    return st;
  const size_t rec = b->kind == kKindTris ? sizeof(Tri) : sizeof(Box);
  const bool host = !on_device(dst);
  CK(cudaMemcpyAsync(dst, b->prims, rec * b->n, cudaMemcpyDefault, c->stream), "primitive copy");
  return host ? check_device(c) : LBVH_OK;
}

const void*
lbvh_bvh_device_nodes(const lbvh_bvh* b)
{
  return b ? b->nodes.ptr : nullptr;
}

int
lbvh_bvh_curve(lbvh_ctx* c, const lbvh_bvh* b, uint32_t* codes, uint32_t* sorted_codes, uint32_t* perm, float* bounds6)
{
  if (!c || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (!(b->flags & LBVH_BUILD_KEEP_CURVE) || !b->curve.ptr)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH was not built with LBVH_BUILD_KEEP_CURVE");
  int st = set_device(c);
  if (st)
    return st;
  const size_t n = b->n;
  const uint32_t* cv = static_cast<const uint32_t*>(b->curve.ptr);
  bool host = false;
  void* outs[4] = { codes, sorted_codes, perm, bounds6 };
  const void* srcs[4] = { cv, cv + n, cv + 2 * n, cv + 3 * n };
  const size_t sizes[4] = { 4 * n, 4 * n, 4 * n, 24 };
  for (int k = 0; k < 4; k++) {
    if (!outs[k])
      continue;
    host |= !on_device(outs[k]);
    CK(cudaMemcpyAsync(outs[k], srcs[k], sizes[k], cudaMemcpyDefault, c->stream), "curve copy");
  }
  return host ? check_device(c) : LBVH_OK;
}

// The traversal copy of a BVH is a cache, made on first use after a build,
// refit or import.
static int
ensure_wnodes(lbvh_ctx* c, lbvh_bvh* b)
{
  if (b->wnodes_valid)
    return LBVH_OK;
  CK(reserve(b->wnodes, sizeof(WideNode) * b->n, c->stream), "traversal layout allocation");
  CK(launch_repack(static_cast<const Node*>(b->nodes.ptr), b->n - 1, static_cast<WideNode*>(b->wnodes.ptr), c->stream),
     "repack launch");
  b->wnodes_valid = true;
  return LBVH_OK;
}

int
lbvh_bvh_prepare_trace(lbvh_ctx* c, lbvh_bvh* b)
{
  if (!c || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (b->n < 2 || b->kind != kKindTris)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH was not built from triangles");
  int st = set_device(c);
  if (st)
    return st;
  return ensure_wnodes(c, b);
}

static int
ensure_copy_streams(lbvh_ctx* c)
{
  if (c->copy_in)
    return LBVH_OK;
  CK(cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking), "copy stream");
  CK(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming), "copy event");
  CK(cudaEventCreateWithFlags(&c->ev_kernel, cudaEventDisableTiming), "copy event");
  CK(cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming), "copy event");
  CK(cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking), "copy stream");
  return LBVH_OK;
}


int
trace_common(lbvh_ctx* c, const lbvh_bvh* b, const float* rays, size_t m, void* hits, uint32_t* n_box, uint32_t* n_tri)
{
  if (!c || !b || (m && (!rays || !hits)))
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (b->n < 2 || b->kind != kKindTris)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH was not built from triangles");
  if (m > 0x7fffffffull)
    return fail(c, LBVH_ERR_INVALID_ARG, "ray count %zu too large", m);
  if (m == 0)
    return LBVH_OK;
  int st = set_device(c);
  if (st)
    return st;
  const bool counts = n_box && n_tri;
  bool hr = !on_device(rays), hh = !on_device(hits);
  const bool hc = counts && (!on_device(n_box) || !on_device(n_tri));
  const bool host_io = hr || hh || hc; // results in host memory: finish before returning
  // page-locked host rays / hits the traversal reaches in place (16-byte
  // aligned ones; others are copied like pageable memory)
  if (hr && c->trace_in_place >= 1) {
    const void* d = mapped_host(rays);
    if (d && !(reinterpret_cast<uintptr_t>(d) & 15)) {
      rays = static_cast<const float*>(d);
      hr = false;
    }
  }
  bool hits_in_place = false;
  if (hh && c->trace_in_place >= 2) {
    void* d = mapped_host(hits);
    if (d && !(reinterpret_cast<uintptr_t>(d) & 15)) {
      hits = d;
      hh = false;
      hits_in_place = true;
    }
  }
  // host rays or hits: copies in chunks that overlap the traversal
  const size_t chunk = c->trace_chunk;
  const bool pipelined = !counts && (hr || hh) && chunk && m >= 2 * chunk;
  const float* dr = rays;
  Hit* dh = static_cast<Hit*>(hits);
  uint32_t* db = n_box;
  uint32_t* dt = n_tri;
  if (hr) {
    CK(reserve(c->rays, 32 * m, c->stream), "ray staging allocation");
    if (!pipelined)
      CK(cudaMemcpyAsync(c->rays.ptr, rays, 32 * m, cudaMemcpyHostToDevice, c->stream), "ray upload");
    dr = static_cast<const float*>(c->rays.ptr);
  } else if (reinterpret_cast<uintptr_t>(rays) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device rays must be 16-byte aligned");
  }
  if (hh) {
    CK(reserve(c->hits, 16 * m, c->stream), "hit staging allocation");
    dh = static_cast<Hit*>(c->hits.ptr);
  } else if (reinterpret_cast<uintptr_t>(hits) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device hits must be 16-byte aligned");
  }
  if (hc) {
    CK(reserve(c->counts, 8 * m, c->stream), "count staging allocation");
    db = static_cast<uint32_t*>(c->counts.ptr);
    dt = db + m;
  }
  const Tri* tris = (b->flags & LBVH_BUILD_SORTED_LEAVES) ? static_cast<const Tri*>(b->sorted_prims.ptr)
                                                          : static_cast<const Tri*>(b->prims);
  const uint32_t* leaf_prim =
    (b->flags & LBVH_BUILD_SORTED_LEAVES) ? static_cast<const uint32_t*>(b->leaf_prim.ptr) : nullptr;
  if ((st = ensure_wnodes(c, const_cast<lbvh_bvh*>(b))))
    return st;
  if (pipelined) {
    if ((st = ensure_copy_streams(c)))
      return st;
    // the staging buffers were last used by an earlier call on this context,
    // which finished before it returned; each chunk has its own region
    for (size_t o = 0; o < m; o += chunk) {
      const size_t mc = m - o < chunk ? m - o : chunk;
      if (hr) {
        CK(cudaMemcpyAsync(const_cast<float*>(dr) + 8 * o, rays + 8 * o, 32 * mc, cudaMemcpyHostToDevice, c->copy_in),
           "ray upload");
        CK(cudaEventRecord(c->ev_in, c->copy_in), "copy event");
        CK(cudaStreamWaitEvent(c->stream, c->ev_in, 0), "copy wait");
      }
      CK(launch_trace_tris(static_cast<const WideNode*>(b->wnodes.ptr), b->n - 1, tris, leaf_prim, dr + 8 * o,
                           uint32_t(mc), dh + o, nullptr, nullptr, c->ray_counter, c->num_sms, c->trace, c->stream),
         "trace launch");
      if (hh) {
        CK(cudaEventRecord(c->ev_kernel, c->stream), "copy event");
        CK(cudaStreamWaitEvent(c->copy_out, c->ev_kernel, 0), "copy wait");
        CK(cudaMemcpyAsync(static_cast<Hit*>(hits) + o, dh + o, 16 * mc, cudaMemcpyDeviceToHost, c->copy_out),
           "hit download");
      }
    }
    if (hh) {
      CK(cudaEventRecord(c->ev_out, c->copy_out), "copy event");
      CK(cudaStreamWaitEvent(c->stream, c->ev_out, 0), "copy wait");
    }
    return check_device(c);
  }
  const uint32_t* order = nullptr;
  if (c->ray_order && !(hits_in_place && !counts) && m >= 4096 && (st = order_rays(c, b, dr, uint32_t(m), &order)))
    return st;
  CK(launch_trace_tris(static_cast<const WideNode*>(b->wnodes.ptr), b->n - 1, tris, leaf_prim, dr, uint32_t(m), dh,
                       counts ? db : nullptr, counts ? dt : nullptr, c->ray_counter, c->num_sms, c->trace,
                       c->stream, hits_in_place && !counts, order),
     "trace launch");
  if (hh)
    CK(cudaMemcpyAsync(hits, dh, 16 * m, cudaMemcpyDeviceToHost, c->stream), "hit download");
  if (hc) {
    CK(cudaMemcpyAsync(n_box, db, 4 * m, cudaMemcpyDefault, c->stream), "count download");
    CK(cudaMemcpyAsync(n_tri, dt, 4 * m, cudaMemcpyDefault, c->stream), "count download");
  }
  if (host_io)
    return check_device(c);
  return LBVH_OK;
}

int
lbvh_trace_spheres(lbvh_ctx* c, const lbvh_bvh* b, const float* spheres, const float* rays, size_t m, void* hits)
{
  if (!c || !b || !spheres || (m && (!rays || !hits)))
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (b->n < 2)
    return fail(c, LBVH_ERR_INVALID_ARG, "BVH has not been built");
  if (b->flags & LBVH_BUILD_SORTED_LEAVES)
    return fail(c, LBVH_ERR_INVALID_ARG, "sphere traces need reference leaf order (a build without sorted leaves)");
  if (m > 0x7fffffffull)
    return fail(c, LBVH_ERR_INVALID_ARG, "ray count %zu too large", m);
  if (m == 0)
    return LBVH_OK;
  int st = set_device(c);
  if (st)
    return st;
  const size_t n = b->n;
  const bool hs = !on_device(spheres), hr = !on_device(rays), hh = !on_device(hits);
  const float* ds = spheres;
  const float* dr = rays;
  SphereHit* dh = static_cast<SphereHit*>(hits);
  if (hs) {
    CK(reserve(c->prims_in, 16 * n, c->stream), "sphere staging allocation");
    CK(cudaMemcpyAsync(c->prims_in.ptr, spheres, 16 * n, cudaMemcpyHostToDevice, c->stream), "sphere upload");
    ds = static_cast<const float*>(c->prims_in.ptr);
  } else if (reinterpret_cast<uintptr_t>(spheres) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device spheres must be 16-byte aligned");
  }
  if (hr) {
    CK(reserve(c->rays, 32 * m, c->stream), "ray staging allocation");
    CK(cudaMemcpyAsync(c->rays.ptr, rays, 32 * m, cudaMemcpyHostToDevice, c->stream), "ray upload");
    dr = static_cast<const float*>(c->rays.ptr);
  } else if (reinterpret_cast<uintptr_t>(rays) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device rays must be 16-byte aligned");
  }
  if (hh) {
    CK(reserve(c->hits, sizeof(SphereHit) * m, c->stream), "hit staging allocation");
    dh = static_cast<SphereHit*>(c->hits.ptr);
  } else if (reinterpret_cast<uintptr_t>(hits) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device hits must be 16-byte aligned");
  }
  if ((st = ensure_wnodes(c, const_cast<lbvh_bvh*>(b))))
    return st;
  CK(launch_trace_spheres(static_cast<const WideNode*>(b->wnodes.ptr), reinterpret_cast<const float4*>(ds), dr,
                          uint32_t(m), dh, c->num_sms, c->stream),
     "sphere trace launch");
  if (hh)
    CK(cudaMemcpyAsync(hits, dh, sizeof(SphereHit) * m, cudaMemcpyDeviceToHost, c->stream), "hit download");
  return (hs || hr || hh) ? check_device(c) : LBVH_OK;
}

int
lbvh_trace_triangles(lbvh_ctx* c, const lbvh_bvh* b, const float* rays, size_t m, void* hits)
{
  return trace_common(c, b, rays, m, hits, nullptr, nullptr);
}

int
lbvh_trace_triangles_counts(lbvh_ctx* c, const lbvh_bvh* b, const float* rays, size_t m, void* hits,
                            uint32_t* n_box, uint32_t* n_tri)
{
  if (!n_box || !n_tri)
    return fail(c, LBVH_ERR_INVALID_ARG, "null count output");
  return trace_common(c, b, rays, m, hits, n_box, n_tri);
}

} // extern "C"

// ---------------------------------------------------------------------------
// batched meshes

struct lbvh_batch
{
  int device = 0;
  uint32_t n_meshes = 0;
  uint32_t total = 0;
  DevBuf off;                // device copy of the n_meshes + 1 offsets
  const void* tris = nullptr;
  DevBuf tris_owned;
  DevBuf nodes;              // total - n_meshes nodes
  DevBuf wnodes;             // traversal copy + flag word
  bool wnodes_valid = false;
  std::vector<uint32_t> host_off; // host copy of the offsets when they were given on the host
  uint32_t flags = 0;
  DevBuf sorted_tris;        // sorted-leaf mode: each mesh's triangles in leaf order
  DevBuf leaf_prim;          // sorted-leaf mode: mesh-local triangle id of each leaf slot
};

namespace {

// Validates offsets on the host when they live there (exact error), else
// leaves it to the device check (reported at the next synchronization).
int
host_offsets_ok(lbvh_ctx* c, const uint32_t* off, size_t n_meshes, size_t total, size_t min_count)
{
  if (on_device(off))
    return LBVH_OK;
  if (off[0] != 0 || off[n_meshes] != total)
    return fail(c, LBVH_ERR_INVALID_ARG, "offsets must start at 0 and end at the total (%zu)", total);
  for (size_t k = 0; k < n_meshes; k++)
    if (off[k + 1] < off[k] || off[k + 1] - off[k] < min_count)
      return fail(c, LBVH_ERR_INVALID_ARG, "segment %zu has %u items (at least %zu needed)", k,
                  off[k + 1] < off[k] ? 0u : off[k + 1] - off[k], min_count);
  return LBVH_OK;
}

int
batch_wnodes(lbvh_ctx* c, lbvh_batch* b)
{
  if (b->wnodes_valid)
    return LBVH_OK;
  const uint32_t total_nodes = b->total - b->n_meshes;
  CK(reserve(b->wnodes, sizeof(WideNode) * (total_nodes + 1), c->stream), "traversal layout allocation");
  CK(launch_batch_repack(static_cast<const Node*>(b->nodes.ptr), total_nodes, static_cast<const uint32_t*>(b->off.ptr),
                         b->n_meshes, static_cast<WideNode*>(b->wnodes.ptr), c->stream),
     "repack launch");
  b->wnodes_valid = true;
  return LBVH_OK;
}

} // namespace

extern "C" {

int
lbvh_batch_prepare_trace(lbvh_ctx* c, lbvh_batch* b)
{
  if (!c || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (!b->n_meshes)
    return fail(c, LBVH_ERR_INVALID_ARG, "batch has not been built");
  int st = set_device(c);
  if (st)
    return st;
  return batch_wnodes(c, b);
}

int
lbvh_batch_create(lbvh_ctx* c, lbvh_batch** out)
{
  if (!c || !out)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  *out = new (std::nothrow) lbvh_batch;
  if (!*out)
    return fail(c, LBVH_ERR_OOM, "host allocation failed");
  (*out)->device = c->device;
  return LBVH_OK;
}

int
lbvh_batch_destroy(lbvh_ctx* c, lbvh_batch* b)
{
  if (!c || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  set_device(c);
  release(b->off, c->stream);
  release(b->tris_owned, c->stream);
  release(b->nodes, c->stream);
  release(b->wnodes, c->stream);
  release(b->sorted_tris, c->stream);
  release(b->leaf_prim, c->stream);
  delete b;
  return LBVH_OK;
}

int
lbvh_batch_build_triangles(lbvh_ctx* c, const float* tris, size_t total, const uint32_t* offsets, size_t n_meshes,
                           lbvh_batch* b)
{
  return lbvh_batch_build(c, tris, total, offsets, n_meshes, 0, b);
}

int
lbvh_batch_build(lbvh_ctx* c, const float* tris, size_t total, const uint32_t* offsets, size_t n_meshes,
                 uint32_t flags, lbvh_batch* b)
{
  if (!c || !tris || !offsets || !b)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (flags & ~LBVH_BUILD_SORTED_LEAVES)
    return fail(c, LBVH_ERR_INVALID_ARG, "unsupported batch build flags 0x%x", flags);
  const bool sorted = flags & LBVH_BUILD_SORTED_LEAVES;
  if (n_meshes < 1 || total < 2 * n_meshes || total > kMaxPrims)
    return fail(c, LBVH_ERR_INVALID_ARG, "%zu meshes over %zu triangles", n_meshes, total);
  int st = set_device(c);
  if (st)
    return st;
  if ((st = host_offsets_ok(c, offsets, n_meshes, total, 2)))
    return st;
  const bool host = !on_device(tris);
  CK(reserve(b->off, 4 * (n_meshes + 1), c->stream), "offset allocation");
  CK(cudaMemcpyAsync(b->off.ptr, offsets, 4 * (n_meshes + 1), cudaMemcpyDefault, c->stream), "offset upload");
  if (on_device(offsets))
    b->host_off.clear();
  else
    b->host_off.assign(offsets, offsets + n_meshes + 1);
  const void* dt = tris;
  if (host) {
    CK(reserve(b->tris_owned, sizeof(Tri) * total, c->stream), "primitive allocation");
    CK(cudaMemcpyAsync(b->tris_owned.ptr, tris, sizeof(Tri) * total, cudaMemcpyHostToDevice, c->stream),
       "primitive upload");
    dt = b->tris_owned.ptr;
  } else if (reinterpret_cast<uintptr_t>(tris) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device triangles must be 16-byte aligned");
  }
  CK(reserve(b->nodes, sizeof(Node) * (total - n_meshes), c->stream), "node allocation");
  // every array on a 256-byte boundary (the boxes are read as 8-byte pairs)
  const size_t o_keys_a = align_up(24 * total, 256);
  const size_t o_keys_b = o_keys_a + align_up(4 * total, 256);
  const size_t o_slots = o_keys_b + align_up(4 * total, 256);
  const size_t o_vals_b = o_slots + align_up(4 * total, 256);
  const size_t ws_bytes = o_vals_b + (sorted ? align_up(4 * total, 256) : 0);
  CK(reserve(c->batch_ws, ws_bytes, c->stream), "batch workspace allocation");
  if (sorted) {
    CK(reserve(b->sorted_tris, sizeof(Tri) * total, c->stream), "sorted triangle allocation");
    CK(reserve(b->leaf_prim, 4 * total, c->stream), "leaf map allocation");
  }
  char* ws = static_cast<char*>(c->batch_ws.ptr);
  BatchBuffers bb{};
  bb.off = static_cast<const uint32_t*>(b->off.ptr);
  bb.n_meshes = uint32_t(n_meshes);
  bb.total = uint32_t(total);
  bb.queue = c->ray_counter + 8;
  bb.boxes = reinterpret_cast<Box*>(ws);
  bb.keys_a = reinterpret_cast<uint32_t*>(ws + o_keys_a);
  bb.keys_b = reinterpret_cast<uint32_t*>(ws + o_keys_b);
  bb.slots = reinterpret_cast<uint32_t*>(ws + o_slots);
  bb.error = &c->state->error;
  if (sorted) { // the permutation lands in the batch's own leaf map
    bb.vals_a = static_cast<uint32_t*>(b->leaf_prim.ptr);
    bb.vals_b = reinterpret_cast<uint32_t*>(ws + o_vals_b);
    bb.sorted_tris = static_cast<Tri*>(b->sorted_tris.ptr);
  }
  CK(launch_batch_build(static_cast<const Tri*>(dt), bb, static_cast<Node*>(b->nodes.ptr), c->batch_threads,
                        c->batch_radix_bits, c->batch_items, c->num_sms, c->stream),
     "batch build launch");
  b->n_meshes = uint32_t(n_meshes);
  b->total = uint32_t(total);
  b->tris = dt;
  b->device = c->device;
  b->wnodes_valid = false;
  b->flags = flags;
  return host ? check_device(c) : LBVH_OK;
}

int
lbvh_batch_info(const lbvh_batch* b, size_t* n_meshes, size_t* total_prims, size_t* total_nodes)
{
  if (!b)
    return LBVH_ERR_INVALID_ARG;
  if (n_meshes)
    *n_meshes = b->n_meshes;
  if (total_prims)
    *total_prims = b->total;
  if (total_nodes)
    *total_nodes = b->total - b->n_meshes;
  return LBVH_OK;
}

int
lbvh_batch_nodes(lbvh_ctx* c, const lbvh_batch* b, void* dst)
{
  if (!c || !b || !dst)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (!b->n_meshes)
    return fail(c, LBVH_ERR_INVALID_ARG, "batch has not been built");
  int st = set_device(c);
  if (st)
    return st;
  const bool host = !on_device(dst);
  CK(cudaMemcpyAsync(dst, b->nodes.ptr, sizeof(Node) * (b->total - b->n_meshes), cudaMemcpyDefault, c->stream),
     "node copy");
  return host ? check_device(c) : LBVH_OK;
}

int
lbvh_batch_mesh_nodes(lbvh_ctx* c, const lbvh_batch* b, size_t k, void* dst)
{
  if (!c || !b || !dst)
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (!b->n_meshes)
    return fail(c, LBVH_ERR_INVALID_ARG, "batch has not been built");
  if (k >= b->n_meshes)
    return fail(c, LBVH_ERR_INVALID_ARG, "mesh %zu of %u", k, b->n_meshes);
  int st = set_device(c);
  if (st)
    return st;
  uint32_t o[2];
  if (!b->host_off.empty()) {
    o[0] = b->host_off[k];
    o[1] = b->host_off[k + 1];
  } else { // offsets were given on the device: read the two that matter
    CK(cudaMemcpyAsync(c->h_err + 1, static_cast<const uint32_t*>(b->off.ptr) + k, 8, cudaMemcpyDeviceToHost,
                       c->stream),
       "offset read");
    CK(cudaStreamSynchronize(c->stream), "stream synchronize");
    o[0] = c->h_err[1];
    o[1] = c->h_err[2];
  }
  const bool host = !on_device(dst);
  CK(cudaMemcpyAsync(dst, static_cast<const Node*>(b->nodes.ptr) + (o[0] - k), sizeof(Node) * (o[1] - o[0] - 1),
                     cudaMemcpyDefault, c->stream),
     "node copy");
  return host ? check_device(c) : LBVH_OK;
}

int
lbvh_batch_trace_triangles(lbvh_ctx* c, const lbvh_batch* b, const float* rays, const uint32_t* ray_offsets, size_t m,
                           void* hits)
{
  if (!c || !b || !ray_offsets || (m && (!rays || !hits)))
    return fail(c, LBVH_ERR_INVALID_ARG, "null argument");
  if (!b->n_meshes)
    return fail(c, LBVH_ERR_INVALID_ARG, "batch has not been built");
  if (m > 0x7fffffffull)
    return fail(c, LBVH_ERR_INVALID_ARG, "ray count %zu too large", m);
  int st = set_device(c);
  if (st)
    return st;
  if ((st = host_offsets_ok(c, ray_offsets, b->n_meshes, m, 0)))
    return st;
  if (m == 0)
    return LBVH_OK;
  lbvh_batch* mb = const_cast<lbvh_batch*>(b); // the traversal copy is a cache
  const uint32_t total_nodes = b->total - b->n_meshes;
  if ((st = batch_wnodes(c, mb)))
    return st;
  // Host ray offsets are staged in the context, never in the batch, so that
  // contexts on different streams can trace one batch at the same time.
  const uint32_t* droff = ray_offsets;
  if (!on_device(ray_offsets)) {
    CK(reserve(c->roff, 4 * (b->n_meshes + 1), c->stream), "ray offset allocation");
    CK(cudaMemcpyAsync(c->roff.ptr, ray_offsets, 4 * (b->n_meshes + 1), cudaMemcpyHostToDevice, c->stream),
       "ray offset upload");
    droff = static_cast<const uint32_t*>(c->roff.ptr);
  } else if (reinterpret_cast<uintptr_t>(ray_offsets) & 3) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device ray offsets must be 4-byte aligned");
  }
  const bool hr = !on_device(rays), hh = !on_device(hits);
  const float* dr = rays;
  Hit* dh = static_cast<Hit*>(hits);
  if (hr) {
    CK(reserve(c->rays, 32 * m, c->stream), "ray staging allocation");
    CK(cudaMemcpyAsync(c->rays.ptr, rays, 32 * m, cudaMemcpyHostToDevice, c->stream), "ray upload");
    dr = static_cast<const float*>(c->rays.ptr);
  } else if (reinterpret_cast<uintptr_t>(rays) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device rays must be 16-byte aligned");
  }
  if (hh) {
    CK(reserve(c->hits, 16 * m, c->stream), "hit staging allocation");
    dh = static_cast<Hit*>(c->hits.ptr);
  } else if (reinterpret_cast<uintptr_t>(hits) & 15) {
    return fail(c, LBVH_ERR_INVALID_ARG, "device hits must be 16-byte aligned");
  }
  const bool sorted = b->flags & LBVH_BUILD_SORTED_LEAVES;
  CK(launch_batch_trace(static_cast<const WideNode*>(mb->wnodes.ptr), total_nodes,
                        static_cast<const Tri*>(sorted ? b->sorted_tris.ptr : b->tris),
                        sorted ? static_cast<const uint32_t*>(b->leaf_prim.ptr) : nullptr,
                        static_cast<const uint32_t*>(b->off.ptr), droff,
                        b->n_meshes, dr, uint32_t(m), dh, c->ray_counter, c->num_sms, c->trace, c->stream),
     "batch trace launch");
  if (hh)
    CK(cudaMemcpyAsync(hits, dh, 16 * m, cudaMemcpyDeviceToHost, c->stream), "hit download");
  return (hr || hh) ? check_device(c) : LBVH_OK;
}

} // extern "C"
