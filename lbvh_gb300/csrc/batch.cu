// Batched LBVH build and trace: thousands of independent meshes of uneven
// size in one persistent launch each.
//
// Build: one CTA builds one whole mesh at a time, taking mesh ids from an
// atomic dispenser, so all synchronization of a build is CTA-scope:
//   1. centroid bounds (block reduction with the reference's tie rule) while
//      staging the leaf boxes;
//   2. Morton codes with the mesh's own bounds, plus the four 8-bit digit
//      histograms in shared memory;
//   3. a stable LSD radix sort of the mesh's codes: four passes, each over
//      CTA-sized chunks in order, ranked per warp with __match_any_sync and
//      placed from running digit offsets in shared memory (one CTA owns the
//      whole segment, so no look-back is needed);
//   4. the bottom-up tree construction of k_tree_local (same node indices and
//      records as the reference's divide_node + fit_boxes, lbvh.h:1588-1867),
//      with the mesh's arrival slots in global memory and CTA-scope fences.
// Each mesh's node block is bit-identical to the reference's node array for
// that mesh alone.
#include "batch.cuh"
#include "device_util.cuh"

#include <atomic>
#include <type_traits>

namespace lbvh_gb300 {

namespace {

constexpr uint32_t kSlotEmpty = 0xffffffffu;

// The leaf boxes and sorted codes are written by the same CTA earlier in the
// kernel, so they are read with coherent (L2) loads, never the read-only path.
struct CgBoxLeaf
{
  const Box* boxes;
  __device__ __forceinline__ Box operator()(uint32_t i) const
  {
    const float2* p = reinterpret_cast<const float2*>(boxes + i);
    const float2 a = __ldcg(p), b = __ldcg(p + 1), c = __ldcg(p + 2);
    return Box{ { a.x, a.y, b.x }, { b.y, c.x, c.y } };
  }
};

// Sorted-leaf mode: the box of leaf slot j is that of triangle perm[j].
struct CgPermBoxLeaf
{
  const Box* boxes;
  const uint32_t* perm;
  __device__ __forceinline__ Box operator()(uint32_t j) const { return CgBoxLeaf{ boxes }(__ldcg(perm + j)); }
};

__device__ __forceinline__ int
delta_cg(const uint32_t* codes, uint32_t n, uint32_t k)
{
  if (k >= n - 1)
    return -1;
  const uint32_t a = __ldcg(codes + k), b = __ldcg(codes + k + 1);
  return a == b ? int(__clz(k ^ (k + 1))) + 32 : int(__clz(a ^ b));
}

} // namespace

// Block-wide exclusive scan of 256 values held by threads 0..255 (other
// threads pass 0 and get 0). s_tmp holds 32 words.
__device__ __forceinline__ uint32_t
scan256(uint32_t v, uint32_t* s_tmp)
{
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31 && warp < 8)
    s_tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < 8 ? s_tmp[lane] : 0u;
    uint32_t t = w;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o)
        t += y;
    }
    if (lane < 8)
      s_tmp[lane] = t - w;
  }
  __syncthreads();
  const uint32_t r = (warp < 8) ? x - v + s_tmp[warp] : 0u;
  __syncthreads();
  return r;
}

// One CTA per mesh at a time (see the file comment). The sort uses digits of
// kBits bits (ceil(30 / kBits) passes over the 30-bit codes) and ranks
// chunks of kItems keys per thread. Dynamic shared memory: one
// 2^kBits-counter histogram per warp for the chunk ranking.
template<bool kSorted, int kBits, int kItems>
__global__ __launch_bounds__(kBatchMaxThreads) void
k_batch_build(const Tri* __restrict__ tris, BatchBuffers b, Node* __restrict__ nodes)
{
  constexpr uint32_t kDigits = 1u << kBits;
  constexpr uint32_t kPasses = (30 + kBits - 1) / kBits;
  static_assert(kDigits <= 256, "the digit scan covers 256 counters");
  extern __shared__ uint32_t s_whist[]; // [warps][kDigits]
  __shared__ uint32_t s_hist[kPasses][kDigits];
  __shared__ uint32_t s_run[kDigits];
  __shared__ ArgBox s_part[32];
  __shared__ uint32_t s_tmp[32];
  __shared__ float s_lo[3], s_scale[3];
  __shared__ uint32_t s_mesh, s_next;

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nthreads = blockDim.x, nwarps = nthreads >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;

  for (;;) {
    if (tid == 0)
      s_mesh = atomicAdd(b.queue, 1u);
    __syncthreads();
    const uint32_t mesh = s_mesh;
    if (mesh >= b.n_meshes)
      return;
    const uint32_t s0 = b.off[mesh];
    const uint32_t n = b.off[mesh + 1] - s0;
    Node* mnodes = nodes + (s0 - mesh);
    if (n < 2) {
      if (tid == 0)
        atomicOr(b.error, kErrBadTopology);
      __syncthreads();
      continue;
    }

    // ---- 1. centroid bounds, staging the leaf boxes ----
    ArgBox a = empty_arg();
    for (uint32_t i = tid; i < n; i += nthreads) {
      const Box bx = load_tri_box(tris + s0, i);
      float2* o = reinterpret_cast<float2*>(b.boxes + s0 + i);
      o[0] = make_float2(bx.lo[0], bx.lo[1]);
      o[1] = make_float2(bx.lo[2], bx.hi[0]);
      o[2] = make_float2(bx.hi[1], bx.hi[2]);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float c = fmul(fadd(bx.lo[k], bx.hi[k]), 0.5f); // center_of, lbvh.h:1160-1167
        if (c < a.v[k]) {
          a.v[k] = c;
          a.i[k] = i;
        }
        if (a.v[k + 3] < c) {
          a.v[k + 3] = c;
          a.i[k + 3] = i;
        }
      }
    }
    a = block_reduce_arg(a, s_part);
    for (uint32_t k = tid; k < kPasses * kDigits; k += nthreads)
      (&s_hist[0][0])[k] = 0;
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        s_lo[k] = a.v[k];
        s_scale[k] = fdiv(1024.0f, fadd(fsub(a.v[k + 3], a.v[k]), 1.0f)); // lbvh.h:1437-1441
      }
    }
    __syncthreads();

    // ---- 2. Morton codes (lbvh.h:1422-1475) + digit histograms ----
    {
      const float lo0 = s_lo[0], lo1 = s_lo[1], lo2 = s_lo[2];
      const float sc0 = s_scale[0], sc1 = s_scale[1], sc2 = s_scale[2];
      const CgBoxLeaf leaf{ b.boxes + s0 };
      for (uint32_t i = tid; i < n; i += nthreads) {
        const Box bx = leaf(i);
        const uint32_t x = __float2uint_rz(fmul(fsub(fmul(fadd(bx.lo[0], bx.hi[0]), 0.5f), lo0), sc0));
        const uint32_t y = __float2uint_rz(fmul(fsub(fmul(fadd(bx.lo[1], bx.hi[1]), 0.5f), lo1), sc1));
        const uint32_t z = __float2uint_rz(fmul(fsub(fmul(fadd(bx.lo[2], bx.hi[2]), 0.5f), lo2), sc2));
        const uint32_t code = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
        b.keys_a[s0 + i] = code;
#pragma unroll
        for (uint32_t pass = 0; pass < kPasses; pass++)
          atomicAdd(&s_hist[pass][(code >> (pass * kBits)) & (kDigits - 1)], 1u);
      }
    }
    __syncthreads();

    // ---- 3. stable LSD radix sort of the mesh's codes, kPasses x kBits bits ----
    uint32_t* src = b.keys_a + s0;
    uint32_t* dst = b.keys_b + s0;
    uint32_t* vsrc = kSorted ? b.vals_a + s0 : nullptr; // pass 0 generates the indices
    uint32_t* vdst = kSorted ? b.vals_b + s0 : nullptr;
    const uint32_t chunk = nthreads * kItems;
    for (uint32_t pass = 0; pass < kPasses; pass++) {
      const uint32_t shift = pass * kBits;
      const uint32_t start = scan256(tid < kDigits ? s_hist[pass][tid] : 0u, s_tmp);
      if (tid < kDigits)
        s_run[tid] = start;
      for (uint32_t c0 = 0; c0 < n; c0 += chunk) {
        for (uint32_t k = tid; k < nwarps * kDigits; k += nthreads)
          s_whist[k] = 0;
        __syncthreads();
        uint32_t key[kItems], dig[kItems], rank[kItems], val[kSorted ? kItems : 1];
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t idx = c0 + warp * (32 * kItems) + uint32_t(k) * 32 + lane;
          key[k] = idx < n ? __ldcg(src + idx) : 0u;
          dig[k] = idx < n ? (key[k] >> shift) & (kDigits - 1) : kDigits; // kDigits: not a key
          if (kSorted)
            val[kSorted ? k : 0] = idx < n ? (pass == 0 ? idx : __ldcg(vsrc + idx)) : 0u;
        }
        // warp ranking: items in (k, lane) order are in index order
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t d = dig[k];
          const uint32_t peers = __match_any_sync(0xffffffffu, d);
          const uint32_t pre = __popc(peers & lt_mask);
          uint32_t before = 0;
          if (d < kDigits)
            before = s_whist[warp * kDigits + d];
          __syncwarp();
          if (d < kDigits && pre == 0)
            s_whist[warp * kDigits + d] = before + __popc(peers);
          __syncwarp();
          rank[k] = before + pre;
        }
        __syncthreads();
        uint32_t total = 0;
        if (tid < kDigits) {
          for (uint32_t w = 0; w < nwarps; w++) {
            const uint32_t c = s_whist[w * kDigits + tid];
            s_whist[w * kDigits + tid] = total;
            total += c;
          }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kItems; k++)
          if (dig[k] < kDigits) {
            const uint32_t at = s_run[dig[k]] + s_whist[warp * kDigits + dig[k]] + rank[k];
            dst[at] = key[k];
            if (kSorted)
              vdst[at] = val[kSorted ? k : 0];
          }
        __syncthreads();
        if (tid < kDigits)
          s_run[tid] += total;
      }
      __syncthreads();
      uint32_t* t = src;
      src = dst;
      dst = t;
      if (kSorted) {
        t = vsrc ? vsrc : b.vals_a + s0;
        vsrc = vdst;
        vdst = t;
      }
    }
    if (kPasses % 2) { // an odd pass count ends in keys_b / vals_b: move the result back
      for (uint32_t i = tid; i < n; i += nthreads) {
        b.keys_a[s0 + i] = __ldcg(b.keys_b + s0 + i);
        if (kSorted)
          b.vals_a[s0 + i] = __ldcg(b.vals_b + s0 + i);
      }
      __syncthreads();
    }
    // the sorted codes are in keys_a (the permutation in vals_a)
    if (kSorted) { // each mesh's triangles in leaf order, for the trace
      const uint32_t* perm = b.vals_a + s0;
      const float4* in = reinterpret_cast<const float4*>(tris + s0);
      float4* out = reinterpret_cast<float4*>(b.sorted_tris + s0);
      for (uint32_t i = tid; i < n; i += nthreads) {
        const uint32_t p = __ldcg(perm + i);
        out[3 * i + 0] = __ldg(in + 3 * p + 0);
        out[3 * i + 1] = __ldg(in + 3 * p + 1);
        out[3 * i + 2] = __ldg(in + 3 * p + 2);
      }
    }

    // ---- 4. bottom-up tree construction (see k_tree_local) ----
    const uint32_t* codes = b.keys_a + s0;
    uint32_t* slots = b.slots + s0;
    using TreeLeaf = typename std::conditional<kSorted, CgPermBoxLeaf, CgBoxLeaf>::type;
    TreeLeaf leaf;
    if constexpr (kSorted)
      leaf = CgPermBoxLeaf{ b.boxes + s0, b.vals_a + s0 };
    else
      leaf = CgBoxLeaf{ b.boxes + s0 };
    for (uint32_t j = tid; j + 1 < n; j += nthreads)
      slots[j] = kSlotEmpty;
    if (tid == 0)
      s_next = 0;
    __syncthreads();
    bool active = false, internal = false;
    uint32_t L = 0, R = 0, lref = 0, rref = 0;
    Box box{};
    for (;;) {
      const uint32_t idle = __ballot_sync(0xffffffffu, !active);
      if (idle) {
        uint32_t first = 0;
        if ((idle & lt_mask) == 0 && !active)
          first = atomicAdd(&s_next, uint32_t(__popc(idle)));
        first = __shfl_sync(0xffffffffu, first, __ffs(idle) - 1);
        if (!active) {
          const uint32_t j = first + __popc(idle & lt_mask);
          if (j < n) {
            L = R = j;
            box = leaf(j);
            internal = false;
            active = true;
          }
        }
      }
      if (!__any_sync(0xffffffffu, active))
        break;
      if (!active)
        continue;
      const bool is_left = delta_cg(codes, n, R) > delta_cg(codes, n, L - 1);
      const uint32_t sp = is_left ? R : L - 1;
      if (internal)
        store_node(mnodes, is_left ? R : L, box, lref, rref);
      __threadfence_block();
      const uint32_t old = atomicExch_block(slots + sp, is_left ? L : R);
      if (old == kSlotEmpty) {
        active = false; // first arrival: the sibling completes the parent
        continue;
      }
      __threadfence_block();
      const uint32_t LP = is_left ? L : old, RP = is_left ? old : R;
      const uint32_t cl = (LP == sp) ? (sp | kLeafBit) : sp;
      const uint32_t cr = (RP == sp + 1) ? ((sp + 1) | kLeafBit) : (sp + 1);
      const uint32_t sib = is_left ? cr : cl;
      const Box other = (sib & kLeafBit) ? leaf(sib & ~kLeafBit) : load_node_box(mnodes, sib);
      box = is_left ? join(box, other) : join(other, box);
      L = LP;
      R = RP;
      lref = cl;
      rref = cr;
      internal = true;
      if (L == 0 && R == n - 1) {
        store_node(mnodes, 0, box, lref, rref);
        active = false;
      }
    }
    __syncthreads(); // the next mesh reuses the shared memory
  }
}

// Offsets check (off[0] == 0, every mesh >= 2 triangles, off[n] == total);
// a bad array sets the error word and the build kernel does nothing.
__global__ void
k_check_offsets(const uint32_t* __restrict__ off, uint32_t n_meshes, uint32_t total, uint32_t* __restrict__ error)
{
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_meshes)
    return;
  const uint32_t a = off[k], b = off[k + 1];
  if ((k == 0 && a != 0) || b < a || b - a < 2 || b > total || (k + 1 == n_meshes && b != total))
    atomicOr(error, kErrBadTopology);
}

__global__ void
k_batch_gate(const uint32_t* __restrict__ error, uint32_t* __restrict__ queue, uint32_t n_meshes)
{
  // a rejected offsets array leaves no mesh to take
  *queue = (*error & kErrBadTopology) ? n_meshes : 0u;
}

template<bool kSorted, int kBits>
static cudaError_t
launch_batch_kernel(uint32_t items, uint32_t grid, uint32_t threads, const Tri* tris, const BatchBuffers& b, Node* nodes,
                    cudaStream_t s)
{
  const size_t smem = size_t(threads / 32) * (1u << kBits) * 4;
  if (items == 8)
    k_batch_build<kSorted, kBits, 8><<<grid, threads, smem, s>>>(tris, b, nodes);
  else
    k_batch_build<kSorted, kBits, 4><<<grid, threads, smem, s>>>(tris, b, nodes);
  return cudaGetLastError();
}

template<bool kSorted>
static cudaError_t
launch_batch_sorted(uint32_t radix_bits, uint32_t items, uint32_t grid, uint32_t threads, const Tri* tris,
                    const BatchBuffers& b, Node* nodes, cudaStream_t s)
{
  switch (radix_bits) {
    case 4:
      return launch_batch_kernel<kSorted, 4>(items, grid, threads, tris, b, nodes, s);
    case 6:
      return launch_batch_kernel<kSorted, 6>(items, grid, threads, tris, b, nodes, s);
    default:
      return launch_batch_kernel<kSorted, 8>(items, grid, threads, tris, b, nodes, s);
  }
}

cudaError_t
launch_batch_build(const Tri* tris, const BatchBuffers& b, Node* nodes, uint32_t threads, uint32_t radix_bits,
                   uint32_t items, int num_sms, cudaStream_t s)
{
  if (threads < 256 || threads > kBatchMaxThreads || threads % 32)
    return cudaErrorInvalidValue;
  if ((radix_bits != 4 && radix_bits != 6 && radix_bits != 8) || (items != 4 && items != 8))
    return cudaErrorInvalidValue;
  k_check_offsets<<<ceil_div_u32(b.n_meshes, 256), 256, 0, s>>>(b.off, b.n_meshes, b.total, b.error);
  k_batch_gate<<<1, 1, 0, s>>>(b.error, b.queue, b.n_meshes);
  const uint32_t per_sm = 2048 / threads;
  const uint32_t cap = uint32_t(num_sms) * per_sm;
  const uint32_t grid = b.n_meshes < cap ? b.n_meshes : cap;
  if (b.sorted_tris)
    return launch_batch_sorted<true>(radix_bits, items, grid, threads, tris, b, nodes, s);
  return launch_batch_sorted<false>(radix_bits, items, grid, threads, tris, b, nodes, s);
}

} // namespace lbvh_gb300
