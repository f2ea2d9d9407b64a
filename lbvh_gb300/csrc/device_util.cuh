// Device helpers shared by the per-scene and the batched build kernels.
#pragma once

#include "common.cuh"

namespace lbvh_gb300 {

// ---- centroid-bounds reduction with the reference's tie rule --------------
//
// The reference folds `acc = std::min(acc, c)` in index order, so on a tie
// (only +0 vs -0 can tie with different bits) the first element in index
// order wins. Every candidate carries its index and every combine picks the
// lower index on compare-equal values, which gives the same winner for any
// reduction tree. Accumulators start at +/-inf and only take a candidate on a
// strict comparison, so NaN never enters, as in the reference.

struct ArgBox
{
  float v[6];
  uint32_t i[6];
};

__device__ __forceinline__ void
take_lo(float& v, uint32_t& i, float v2, uint32_t i2)
{
  if (v2 < v || (!(v < v2) && i2 < i)) {
    v = v2;
    i = i2;
  }
}
__device__ __forceinline__ void
take_hi(float& v, uint32_t& i, float v2, uint32_t i2)
{
  if (v < v2 || (!(v2 < v) && i2 < i)) {
    v = v2;
    i = i2;
  }
}

__device__ __forceinline__ void
combine(ArgBox& a, const ArgBox& b)
{
#pragma unroll
  for (int k = 0; k < 3; k++)
    take_lo(a.v[k], a.i[k], b.v[k], b.i[k]);
#pragma unroll
  for (int k = 3; k < 6; k++)
    take_hi(a.v[k], a.i[k], b.v[k], b.i[k]);
}

__device__ __forceinline__ ArgBox
empty_arg()
{
  ArgBox a;
  const float inf = __int_as_float(0x7f800000);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    a.v[k] = inf;
    a.v[k + 3] = -inf;
  }
#pragma unroll
  for (int k = 0; k < 6; k++)
    a.i[k] = 0xffffffffu;
  return a;
}

__device__ __forceinline__ ArgBox
block_reduce_arg(ArgBox a, ArgBox* s_part)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ArgBox b;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      b.v[k] = __shfl_down_sync(0xffffffffu, a.v[k], o);
      b.i[k] = __shfl_down_sync(0xffffffffu, a.i[k], o);
    }
    combine(a, b);
  }
  if (lane == 0)
    s_part[warp] = a;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? s_part[lane] : empty_arg();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ArgBox b;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        b.v[k] = __shfl_down_sync(0xffffffffu, a.v[k], o);
        b.i[k] = __shfl_down_sync(0xffffffffu, a.i[k], o);
      }
      combine(a, b);
    }
  }
  return a; // valid in thread 0
}

// ---- radix-tree construction ----------------------------------------------

// delta(k, k + 1) of the reference's divide_node (lbvh.h:1602-1621) for the
// boundary between sorted positions k and k + 1 of n codes: clz of the code
// xor, clz(k ^ (k + 1)) + 32 on equal codes, -1 outside [0, n - 2].
__device__ __forceinline__ int
boundary_delta(const uint32_t* __restrict__ codes, uint32_t n, uint32_t k)
{
  if (k >= n - 1) // k = L - 1 wraps for L = 0; k = n - 1 is past the end
    return -1;
  const uint32_t a = __ldg(codes + k), b = __ldg(codes + k + 1);
  return a == b ? int(__clz(k ^ (k + 1))) + 32 : int(__clz(a ^ b));
}

// One node record in one 256-bit store (sm_100 and later): every node array
// the build kernels write is 32-byte aligned (cudaMallocAsync, or a caller's
// array that the allocation-free entry point checks). The memory clobber
// keeps the store ahead of the release that may follow it.
__device__ __forceinline__ void
store_node(Node* __restrict__ nodes, uint32_t idx, const Box& b, uint32_t l, uint32_t r)
{
  asm volatile("st.global.cg.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(nodes + idx), "f"(b.lo[0]), "f"(b.lo[1]), "f"(b.lo[2]), "f"(b.hi[0]), "f"(b.hi[1]), "f"(b.hi[2]),
                 "f"(__uint_as_float(l)), "f"(__uint_as_float(r))
               : "memory");
}

// Arrival at a device-scope slot: swaps in `v` and returns the previous word,
// with release semantics (this thread's earlier stores, e.g. the record of the
// node it just finished, become visible to whoever reads `v`) and acquire
// semantics (the stores that the previous writer made before its own swap,
// e.g. the sibling's record, are visible to this thread's later loads).
__device__ __forceinline__ unsigned long long
arrive_acq_rel(unsigned long long* slot, unsigned long long v)
{
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(slot), "l"(v) : "memory");
  return old;
}

// The same arrival on a global slot, ordered at block scope: for walks
// whose every arrival comes from threads of one CTA.
__device__ __forceinline__ unsigned long long
arrive_acq_rel_cta_global(unsigned long long* slot, unsigned long long v)
{
  unsigned long long old;
  asm volatile("atom.acq_rel.cta.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(slot), "l"(v) : "memory");
  return old;
}

// The same arrival on a shared-memory slot, ordered at block scope.
__device__ __forceinline__ uint32_t
arrive_acq_rel_cta(uint32_t* slot, uint32_t v)
{
  uint32_t old;
  const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(slot));
  asm volatile("atom.acq_rel.cta.shared::cta.exch.b32 %0, [%1], %2;" : "=r"(old) : "r"(addr), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ Box
load_node_box(const Node* __restrict__ nodes, uint32_t idx)
{
  const float4 a = __ldcg(reinterpret_cast<const float4*>(nodes + idx));
  const float2 b = __ldcg(reinterpret_cast<const float2*>(nodes + idx) + 2);
  return Box{ { a.x, a.y, a.z }, { a.w, b.x, b.y } };
}

// Node records of the local tree phase in shared memory, 32 bytes each, with
// the two 16-byte halves of record j swapped when bit 2 of j is set: a warp
// touching records at random positions then spreads its 16-byte accesses
// over all eight 16-byte bank groups, not the four that (2 j + half) mod 8
// reaches otherwise.
__device__ __forceinline__ float4*
rec_half(Node* recs, uint32_t j, uint32_t half)
{
  return reinterpret_cast<float4*>(recs + j) + (half ^ ((j >> 2) & 1u));
}
__device__ __forceinline__ const float4*
rec_half(const Node* recs, uint32_t j, uint32_t half)
{
  return reinterpret_cast<const float4*>(recs + j) + (half ^ ((j >> 2) & 1u));
}
__device__ __forceinline__ void
stage_record_at(Node* recs, uint32_t j, const Box& b, uint32_t l, uint32_t r)
{
  *rec_half(recs, j, 0) = make_float4(b.lo[0], b.lo[1], b.lo[2], b.hi[0]);
  *rec_half(recs, j, 1) = make_float4(b.hi[1], b.hi[2], __uint_as_float(l), __uint_as_float(r));
}
__device__ __forceinline__ Box
staged_box_at(const Node* recs, uint32_t j)
{
  const float4 a = *rec_half(recs, j, 0);
  const float2 b = *reinterpret_cast<const float2*>(rec_half(recs, j, 1));
  return Box{ { a.x, a.y, a.z }, { a.w, b.x, b.y } };
}
// The left-child word of record j (0: no record staged there).
__device__ __forceinline__ float*
staged_left_at(Node* recs, uint32_t j)
{
  return &rec_half(recs, j, 1)->z;
}

// A box at an 8-byte aligned address (arrays of Box), as three 8-byte accesses.
__device__ __forceinline__ Box
load_box8(const Box* p)
{
  const float2* q = reinterpret_cast<const float2*>(p);
  const float2 a = q[0], b = q[1], c = q[2];
  return Box{ { a.x, a.y, b.x }, { b.y, c.x, c.y } };
}
__device__ __forceinline__ void
store_box8(Box* p, const Box& b)
{
  float2* q = reinterpret_cast<float2*>(p);
  q[0] = make_float2(b.lo[0], b.lo[1]);
  q[1] = make_float2(b.lo[2], b.hi[0]);
  q[2] = make_float2(b.hi[1], b.hi[2]);
}

// Asynchronous 16-byte copy global -> shared (cp.async, L2 only); bytes
// beyond src_bytes (0..16) are zero-filled and not read.
__device__ __forceinline__ void
copy16_async(void* smem, const void* gmem, uint32_t src_bytes)
{
  const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}

__device__ __forceinline__ void
copy_async_commit()
{
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Waits until at most kPending of this thread's committed groups are in flight.
template<int kPending>
__device__ __forceinline__ void
copy_async_wait()
{
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kPending) : "memory");
}

} // namespace lbvh_gb300
