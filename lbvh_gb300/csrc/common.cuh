// Shared device types and exact-arithmetic helpers for the LBVH kernels.
//
// Every floating-point operation that reaches an output is written with an
// explicit round-to-nearest intrinsic (__fadd_rn, __fsub_rn, __fmul_rn,
// __fdiv_rn), which the compiler never fuses into an FMA, and the library is
// also compiled with -fmad=false. This reproduces the reference
// (tay10r/lbvh, lbvh.h) built without FP contraction, bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lbvh_gb300 {

constexpr uint32_t kLeafBit = 0x80000000u; // highest_bit<u32>(), lbvh.h:170-175
constexpr uint32_t kMiss = 0xffffffffu;    // intersection_container miss, lbvh.h:366

// Sticky device error bits (BuildState::error).
constexpr uint32_t kErrLookbackTimeout = 1u << 0;
constexpr uint32_t kErrBadTopology = 1u << 1;

// reference triangle<float> (lbvh.h:1959-1983): {p0, e0, e1, normal},
// 48 bytes = three 16-byte vectors:
//   a = {p0.x, p0.y, p0.z, e0.x}, b = {e0.y, e0.z, e1.x, e1.y},
//   c = {e1.z, n.x, n.y, n.z}
struct __align__(16) Tri
{
  float4 a, b, c;
};

// reference node<float> (lbvh.h:220-255): 32 bytes, alignas(32).
struct __align__(32) Node
{
  float lo[3], hi[3];
  uint32_t left, right;
};
static_assert(sizeof(Node) == 32, "node layout");

struct Box
{
  float lo[3], hi[3];
};

struct __align__(16) Hit
{
  uint32_t prim;
  float t, u, v;
};

// Device-side state of a build, one per context (persistent, so the sticky
// error word survives workspace growth).
struct BuildState
{
  float lo[3], hi[3];          // centroid bounds
  float scale[3];              // 1024 / (size + 1), lbvh.h:1437-1441
  uint32_t pad0;
  uint32_t hist[4][256];       // radix digit histograms of the Morton codes
  uint32_t tile_counter[4];    // onesweep tile id dispensers, one per pass
  uint32_t done_counter;       // last-block detection in the bounds kernel
  uint32_t tree_fallback;      // tree build: a merge window overflowed; the last level walks instead
  uint32_t error;              // sticky kErr* bits
  uint32_t pad1;
  // keys-only sort by buckets of the top 12 code bits (see k_top_scan)
  uint32_t top_hist[4096];     // histogram of code >> 18
  uint32_t top_base[4097];     // bucket starts (exclusive scan), top_base[4096] = n
  uint32_t use_msd;            // 1: the bucket sort runs; 0: the four onesweep passes run
  uint32_t top_nonempty;       // number of non-empty buckets
  uint32_t bucket_next;        // bucket sort: next entry of top_list to take
  uint32_t top_list[4096];     // the non-empty buckets, ascending
};

// ---- exact scalar ops --------------------------------------------------

__device__ __forceinline__ float
fadd(float a, float b)
{
  return __fadd_rn(a, b);
}
__device__ __forceinline__ float
fsub(float a, float b)
{
  return __fsub_rn(a, b);
}
__device__ __forceinline__ float
fmul(float a, float b)
{
  return __fmul_rn(a, b);
}
__device__ __forceinline__ float
fdiv(float a, float b)
{
  return __fdiv_rn(a, b);
}

// std::min(a, b) = (b < a) ? b : a and std::max(a, b) = (a < b) ? b : a, the
// forms the reference's vector min/max use (lbvh.h:638-660): ties and NaN in
// b keep a.
__device__ __forceinline__ float
smin(float a, float b)
{
  return (b < a) ? b : a;
}
__device__ __forceinline__ float
smax(float a, float b)
{
  return (a < b) ? b : a;
}
// math::min / math::max ternaries (lbvh.h:567-580): ties and NaN in a pick b.
__device__ __forceinline__ float
mmin(float a, float b)
{
  return (a < b) ? a : b;
}
__device__ __forceinline__ float
mmax(float a, float b)
{
  return (a > b) ? a : b;
}

// dot accumulates from 0 in x, y, z order (lbvh.h:621-630); the leading
// 0 + x.x*y.x turns a -0 product into +0 exactly as the reference does.
__device__ __forceinline__ float
dot3(float ax, float ay, float az, float bx, float by, float bz)
{
  float o = fadd(0.0f, fmul(ax, bx));
  o = fadd(o, fmul(ay, by));
  o = fadd(o, fmul(az, bz));
  return o;
}

// triangle_aabb_converter (lbvh.h:2001-2012): p1 = p0 - e0, p2 = p0 + e1,
// min(min(p0, p1), p2) and max(max(p0, p1), p2) with std::min/std::max.
__device__ __forceinline__ Box
tri_box(const float4& a, const float4& b, const float4& c)
{
  const float p0x = a.x, p0y = a.y, p0z = a.z;
  const float e0x = a.w, e0y = b.x, e0z = b.y;
  const float e1x = b.z, e1y = b.w, e1z = c.x;
  const float p1x = fsub(p0x, e0x), p1y = fsub(p0y, e0y), p1z = fsub(p0z, e0z);
  const float p2x = fadd(p0x, e1x), p2y = fadd(p0y, e1y), p2z = fadd(p0z, e1z);
  Box r;
  r.lo[0] = smin(smin(p0x, p1x), p2x);
  r.lo[1] = smin(smin(p0y, p1y), p2y);
  r.lo[2] = smin(smin(p0z, p1z), p2z);
  r.hi[0] = smax(smax(p0x, p1x), p2x);
  r.hi[1] = smax(smax(p0y, p1y), p2y);
  r.hi[2] = smax(smax(p0z, p1z), p2z);
  return r;
}

__device__ __forceinline__ Box
load_tri_box(const Tri* __restrict__ tris, uint32_t i)
{
  const float4* p = reinterpret_cast<const float4*>(tris + i);
  const float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2);
  return tri_box(a, b, c);
}

// union_of(box, box), lbvh.h:1208-1211: a is the accumulated (left) box.
__device__ __forceinline__ Box
join(const Box& a, const Box& b)
{
  Box r;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r.lo[k] = smin(a.lo[k], b.lo[k]);
    r.hi[k] = smax(a.hi[k], b.hi[k]);
  }
  return r;
}

// morton_encoder<4>::expand, lbvh.h:1351-1359
__device__ __forceinline__ uint32_t
expand10(uint32_t n)
{
  n = (n | (n << 16)) & 0x030000ffu;
  n = (n | (n << 8)) & 0x0300f00fu;
  n = (n | (n << 4)) & 0x030c30c3u;
  n = (n | (n << 2)) & 0x09249249u;
  return n;
}

__host__ __device__ constexpr uint32_t
ceil_div_u32(uint32_t a, uint32_t b)
{
  return (a + b - 1) / b;
}

// ---- programmatic dependent launch ----------------------------------------
//
// The build's kernels are launched with programmatic stream serialization
// (launch_pdl): a kernel's CTAs may be scheduled while its predecessor in the
// stream is still running, so the launch latency between two kernels is
// hidden. Every such kernel starts with pdl_begin(): wait until the
// predecessor grid has completed and its writes are visible, then allow the
// successor to be scheduled. Waiting first means that when a kernel's
// successor starts, every kernel before this one has finished. Both
// instructions do nothing for a kernel launched without the attribute.
__device__ __forceinline__ void
pdl_begin()
{
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// kernel<<<grid, block, smem, s>>>(args...) with programmatic stream
// serialization allowed.
template<typename... Params, typename... Args>
inline cudaError_t
launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args)
{
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

} // namespace lbvh_gb300
