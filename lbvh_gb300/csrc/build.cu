// LBVH build kernels for sm_103a: centroid bounds, Morton codes + radix
// histograms, onesweep LSD radix sort, Karras split, bottom-up box fit.
//
// Reference: tay10r/lbvh `lbvh.h`, builder<float>::operator() (lbvh.h:1793-1822).
// Every kernel reproduces the reference's outputs bit for bit; the comments on
// each kernel cite the reference code it replaces.
#include "build.cuh"

#include <cuda/atomic>

namespace lbvh_gb300 {

// ---------------------------------------------------------------------------
// triangle<float>(a, b, c), lbvh.h:1967-1972: e0 = a - b, e1 = c - a,
// normal = cross(e0, e1) with cross as in lbvh.h:609-616.

__global__ void
k_make_triangles(const float* __restrict__ verts, uint32_t n, Tri* __restrict__ out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const float* v = verts + size_t(i) * 9;
  const float ax = v[0], ay = v[1], az = v[2];
  const float bx = v[3], by = v[4], bz = v[5];
  const float cx = v[6], cy = v[7], cz = v[8];
  const float e0x = fsub(ax, bx), e0y = fsub(ay, by), e0z = fsub(az, bz);
  const float e1x = fsub(cx, ax), e1y = fsub(cy, ay), e1z = fsub(cz, az);
  const float nx = fsub(fmul(e0y, e1z), fmul(e0z, e1y));
  const float ny = fsub(fmul(e0z, e1x), fmul(e0x, e1z));
  const float nz = fsub(fmul(e0x, e1y), fmul(e0y, e1x));
  Tri t;
  t.a = make_float4(ax, ay, az, e0x);
  t.b = make_float4(e0y, e0z, e1x, e1y);
  t.c = make_float4(e1z, nx, ny, nz);
  out[i] = t;
}

// ---------------------------------------------------------------------------
// Centroid bounds (centroid_bounds_kernel + serial union, lbvh.h:1282-1293,
// 1532-1543).
//
// The reference folds `acc = std::min(acc, c)` in index order, so on a tie
// (only +0 vs -0 can tie with different bits) the first element in index
// order wins. Here every candidate carries its index and every combine picks
// the lower index on compare-equal values, which gives the same winner for
// any reduction tree. Accumulators start at +/-inf and only take a candidate
// on a strict comparison, so NaN never enters, as in the reference.

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

template<class Leaf>
__global__ __launch_bounds__(kBoundsThreads) void
k_bounds(Leaf leaf, uint32_t n, ArgBox* __restrict__ partials, BuildState* __restrict__ st)
{
  __shared__ ArgBox s_part[kBoundsThreads / 32];
  __shared__ bool s_last;
  const uint32_t chunk = ceil_div_u32(n, gridDim.x);
  const uint32_t b = blockIdx.x * chunk;
  const uint32_t e = min(n, b + chunk);
  ArgBox a = empty_arg();
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const Box bx = leaf(i);
    // center_of, lbvh.h:1160-1167: (min + max) * 0.5
    const float c[3] = { fmul(fadd(bx.lo[0], bx.hi[0]), 0.5f),
                         fmul(fadd(bx.lo[1], bx.hi[1]), 0.5f),
                         fmul(fadd(bx.lo[2], bx.hi[2]), 0.5f) };
    // per-thread elements come in increasing index order: the reference's
    // strict-compare fold keeps the earliest on ties
#pragma unroll
    for (int k = 0; k < 3; k++) {
      if (c[k] < a.v[k]) {
        a.v[k] = c[k];
        a.i[k] = i;
      }
      if (a.v[k + 3] < c[k]) {
        a.v[k + 3] = c[k];
        a.i[k + 3] = i;
      }
    }
  }
  a = block_reduce_arg(a, s_part);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = a;
    __threadfence();
    const uint32_t done = atomicAdd(&st->done_counter, 1u);
    s_last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last)
    return;
  // last block: combine the partials, finish the scale, reset per-build state
  __threadfence();
  ArgBox r = empty_arg();
  for (uint32_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    ArgBox p;
    const ArgBox* src = partials + k;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      p.v[j] = __ldcg(&src->v[j]);
      p.i[j] = __ldcg(&src->i[j]);
    }
    combine(r, p);
  }
  __syncthreads();
  r = block_reduce_arg(r, s_part);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      st->lo[k] = r.v[k];
      st->hi[k] = r.v[k + 3];
      // morton_curve_kernel scale, lbvh.h:1437-1441: 1024 / (size + 1)
      st->scale[k] = fdiv(1024.0f, fadd(fsub(r.v[k + 3], r.v[k]), 1.0f));
    }
    st->done_counter = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      st->tile_counter[k] = 0;
  }
  for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x)
    (&st->hist[0][0])[k] = 0;
}

// ---------------------------------------------------------------------------
// Morton codes (morton_curve_kernel, lbvh.h:1422-1475 with morton_encoder<4>,
// lbvh.h:1345-1359): q = u32((center - min) * scale), code = x<<2 | y<<1 | z.
// Also accumulates the four 8-bit digit histograms the radix sort needs, so
// the sort never re-reads the codes just to count them.

template<class Leaf>
__global__ __launch_bounds__(kMortonThreads) void
k_morton(Leaf leaf, uint32_t n, uint32_t* __restrict__ codes, BuildState* __restrict__ st)
{
  __shared__ uint32_t s_hist[4 * 256];
  for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x)
    s_hist[k] = 0;
  __syncthreads();
  const float lo0 = st->lo[0], lo1 = st->lo[1], lo2 = st->lo[2];
  const float s0 = st->scale[0], s1 = st->scale[1], s2 = st->scale[2];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const Box bx = leaf(i);
    const float cx = fmul(fadd(bx.lo[0], bx.hi[0]), 0.5f);
    const float cy = fmul(fadd(bx.lo[1], bx.hi[1]), 0.5f);
    const float cz = fmul(fadd(bx.lo[2], bx.hi[2]), 0.5f);
    const uint32_t x = __float2uint_rz(fmul(fsub(cx, lo0), s0));
    const uint32_t y = __float2uint_rz(fmul(fsub(cy, lo1), s1));
    const uint32_t z = __float2uint_rz(fmul(fsub(cz, lo2), s2));
    const uint32_t code = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
    codes[i] = code;
    atomicAdd(&s_hist[0 * 256 + (code & 255u)], 1u);
    atomicAdd(&s_hist[1 * 256 + ((code >> 8) & 255u)], 1u);
    atomicAdd(&s_hist[2 * 256 + ((code >> 16) & 255u)], 1u);
    atomicAdd(&s_hist[3 * 256 + (code >> 24)], 1u);
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x) {
    const uint32_t c = s_hist[k];
    if (c)
      atomicAdd(&(&st->hist[0][0])[k], c);
  }
}

// ---------------------------------------------------------------------------
// Onesweep LSD radix sort pass (8-bit digit), stable. Replaces
// space_filling_curve::sort (lbvh.h:1126-1134). The reference's std::sort is
// unstable, but only the sorted code sequence reaches its output (the leaf
// slot p holds primitive p, lbvh.h:1855-1862), so a stable sort reproduces
// it; the permutation it produces is the stable one (ascending original
// index on equal codes).
//
// One CTA per 4096-key tile. Tiles take ids from an atomic dispenser, rank
// their keys per warp with __match_any_sync, publish per-digit counts in an
// epoch-tagged 64-bit look-back word, resolve their global digit offsets by
// decoupled look-back over earlier tiles, reorder in shared memory and write
// each digit run contiguously.
//
// look-back word: [63:32] epoch, [31:30] status (1 aggregate, 2 inclusive
// prefix), [29:0] count. A word whose epoch is not the current one is "not
// yet published", so the buffer never needs clearing between passes.

__device__ __forceinline__ unsigned long long
ld_relaxed_u64(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void
st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t
block_excl_scan_256(uint32_t v, uint32_t* s_warp)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31)
    s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < kSortWarps ? s_warp[lane] : 0u;
    uint32_t s = w;
#pragma unroll
    for (int o = 1; o < kSortWarps; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o)
        s += y;
    }
    if (lane < kSortWarps)
      s_warp[lane] = s - w;
  }
  __syncthreads();
  const uint32_t r = x - v + s_warp[warp];
  __syncthreads();
  return r;
}

template<bool kPairs, bool kIotaVals>
__global__ __launch_bounds__(kSortThreads) void
k_onesweep(const uint32_t* __restrict__ kin,
           uint32_t* __restrict__ kout,
           const uint32_t* __restrict__ vin,
           uint32_t* __restrict__ vout,
           uint32_t n,
           uint32_t pass,
           uint32_t epoch,
           unsigned long long* __restrict__ lookback,
           BuildState* __restrict__ st)
{
  __shared__ uint32_t s_keys[kSortTile];
  __shared__ uint32_t s_vals[kPairs ? kSortTile : 1];
  __shared__ uint32_t s_whist[kSortWarps][256];
  __shared__ uint32_t s_tile_start[256];
  __shared__ uint32_t s_gbase[256];
  __shared__ uint32_t s_warp[kSortWarps];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0)
    s_tile = atomicAdd(&st->tile_counter[pass], 1u);
  for (int i = tid; i < kSortWarps * 256; i += kSortThreads)
    (&s_whist[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * uint32_t(kSortTile);
  const uint32_t shift = pass * 8;

  uint32_t key[kSortItems], val[kPairs ? kSortItems : 1], dig[kSortItems], rank[kSortItems];
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const uint32_t idx = base + uint32_t(warp) * (32 * kSortItems) + uint32_t(k) * 32 + lane;
    if (idx < n) {
      key[k] = kin[idx];
      if (kPairs)
        val[kPairs ? k : 0] = kIotaVals ? idx : vin[idx];
      dig[k] = (key[k] >> shift) & 255u;
    } else {
      key[k] = 0;
      dig[k] = 256; // not a key: ranked in no bucket
    }
  }

  // warp-level stable ranking: items in (k, lane) order are in index order
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const uint32_t d = dig[k];
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t pre = __popc(peers & lt_mask);
    uint32_t before = 0;
    if (d < 256)
      before = s_whist[warp][d];
    __syncwarp();
    if (d < 256 && pre == 0)
      s_whist[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[k] = before + pre;
  }
  __syncthreads();

  // thread tid owns digit tid: warp offsets and the tile total
  uint32_t total = 0;
#pragma unroll
  for (int w = 0; w < kSortWarps; w++) {
    const uint32_t c = s_whist[w][tid];
    s_whist[w][tid] = total;
    total += c;
  }
  unsigned long long* my = lookback + size_t(tile) * 256 + tid;
  const unsigned long long tag = (unsigned long long)epoch << 32;
  st_relaxed_u64(my, tag | ((tile == 0 ? 2ull : 1ull) << 30) | total);

  const uint32_t gofs = block_excl_scan_256(st->hist[pass][tid], s_warp);
  s_tile_start[tid] = block_excl_scan_256(total, s_warp);

  uint32_t excl = 0;
  if (tile > 0) {
    uint32_t p = tile - 1;
    uint32_t spins = 0;
    for (;;) {
      const unsigned long long e = ld_relaxed_u64(lookback + size_t(p) * 256 + tid);
      const uint32_t lo = uint32_t(e);
      const uint32_t status = lo >> 30;
      if (uint32_t(e >> 32) == epoch && status != 0) {
        excl += lo & 0x3fffffffu;
        if (status == 2 || p == 0)
          break;
        --p;
        spins = 0;
      } else if (++spins > kSpinLimit) {
        atomicOr(&st->error, kErrLookbackTimeout);
        break;
      } else if (spins > 64) {
        __nanosleep(64);
      }
    }
    st_relaxed_u64(my, tag | (2ull << 30) | (excl + total));
  }
  s_gbase[tid] = gofs + excl;
  __syncthreads();

  // reorder the tile in shared memory by digit
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const uint32_t d = dig[k];
    if (d < 256) {
      const uint32_t pos = s_tile_start[d] + s_whist[warp][d] + rank[k];
      s_keys[pos] = key[k];
      if (kPairs)
        s_vals[pos] = val[kPairs ? k : 0];
    }
  }
  __syncthreads();

  // write out: consecutive positions of one digit go to consecutive addresses
  const uint32_t tile_n = min(uint32_t(kSortTile), n - base);
  for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t d = (k >> shift) & 255u;
    const uint32_t o = s_gbase[d] + i - s_tile_start[d];
    if (o < n) { // always true unless a look-back wait gave up
      kout[o] = k;
      if (kPairs)
        vout[o] = s_vals[i];
    }
  }
}

// ---------------------------------------------------------------------------
// Karras split, one thread per internal node (divide_node + builder_kernel,
// lbvh.h:1588-1731). The search is the reference's: direction from
// delta(i, i+1) - delta(i, i-1), an exponential probe from l_max = 128 in
// steps of x4, a binary search for the range end, then a binary search for
// the split with ceil-divided steps. delta is clz of the code xor, or
// clz(i ^ j) + 32 on equal codes, or -1 out of range.

__device__ __forceinline__ int
split_delta(const uint32_t* __restrict__ codes, int64_t n, int64_t j, uint32_t cj, int64_t k)
{
  if (k < 0 || k >= n)
    return -1;
  const uint32_t ck = __ldg(codes + k);
  if (cj == ck)
    return __clz(uint32_t(j ^ k)) + 32;
  return __clz(cj ^ ck);
}

__global__ __launch_bounds__(kSplitThreads) void
k_split(const uint32_t* __restrict__ codes,
        uint32_t n,
        uint2* __restrict__ child,
        uint32_t* __restrict__ leaf_parent,
        uint32_t* __restrict__ node_parent)
{
  const uint32_t ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii + 1 >= n)
    return;
  const int64_t i = ii, nn = n;
  const uint32_t ci = __ldg(codes + i);
  const int d = (split_delta(codes, nn, i, ci, i + 1) - split_delta(codes, nn, i, ci, i - 1)) < 0 ? -1 : 1;
  const int dmin = split_delta(codes, nn, i, ci, i - d);
  int64_t lmax = 128;
  for (;;) {
    const int64_t k = i + lmax * d;
    if (k >= nn)
      break;
    if (!(split_delta(codes, nn, i, ci, k) > dmin))
      break;
    lmax *= 4;
  }
  int64_t l = 0;
  for (int64_t div = 2;; div *= 2) {
    const int64_t t = lmax / div;
    if (split_delta(codes, nn, i, ci, i + (l + t) * d) > dmin)
      l += t;
    if (t == 1)
      break;
  }
  const int64_t j = i + l * d;
  const int dnode = split_delta(codes, nn, i, ci, j);
  int64_t s = 0;
  for (int64_t div = 2;; div *= 2) {
    const int64_t t = (l + (div - 1)) / div;
    if (split_delta(codes, nn, i, ci, i + (s + t) * d) > dnode)
      s += t;
    if (div >= l)
      break;
  }
  const int64_t gamma = i + s * d + (d < 0 ? d : 0);
  const int64_t lo = i < j ? i : j;
  const int64_t hi = j > i ? j : i;
  const bool lleaf = lo == gamma;
  const bool rleaf = hi == gamma + 1;
  child[i] = make_uint2(uint32_t(gamma) | (lleaf ? kLeafBit : 0u),
                        uint32_t(gamma + 1) | (rleaf ? kLeafBit : 0u));
  (lleaf ? leaf_parent : node_parent)[gamma] = uint32_t(i);
  (rleaf ? leaf_parent : node_parent)[gamma + 1] = uint32_t(i);
}

// Parent links from an existing node array (for refit).
__global__ void
k_links_from_nodes(const Node* __restrict__ nodes,
                   uint32_t n_nodes,
                   uint2* __restrict__ child,
                   uint32_t* __restrict__ leaf_parent,
                   uint32_t* __restrict__ node_parent)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes)
    return;
  const uint4 lr = *reinterpret_cast<const uint4*>(&nodes[i].hi[1]);
  const uint32_t l = lr.z, r = lr.w;
  child[i] = make_uint2(l, r);
  const uint32_t n = n_nodes + 1;
  if (((l & kLeafBit) ? (l & ~kLeafBit) >= n : l >= n_nodes) || ((r & kLeafBit) ? (r & ~kLeafBit) >= n : r >= n_nodes))
    return; // the fit that follows reports the malformed link
  if (l & kLeafBit)
    leaf_parent[l & ~kLeafBit] = i;
  else
    node_parent[l] = i;
  if (r & kLeafBit)
    leaf_parent[r & ~kLeafBit] = i;
  else
    node_parent[r] = i;
}

// ---------------------------------------------------------------------------
// Bottom-up box fit with per-node arrival flags. Replaces the reference's
// serial fit (builder::fit_boxes, lbvh.h:1826-1867): node box = left box
// (leaf converter or child node box), then union_of(box, right box). The
// union is order-fixed (left first), so the result does not depend on which
// child arrives last.
//
// One thread per leaf slot. Each internal node receives exactly two
// arrivals per build; the flag word counts them, so the first arrival sees an
// even value and stops, the second sees an odd one and fits the node. Flags
// therefore stay even between builds and need no clearing.

template<class Leaf>
__global__ __launch_bounds__(kFitThreads) void
k_fit(Leaf leaf,
      uint32_t n,
      const uint2* __restrict__ child,
      const uint32_t* __restrict__ leaf_parent,
      const uint32_t* __restrict__ node_parent,
      uint32_t* __restrict__ flags,
      Node* __restrict__ nodes,
      BuildState* __restrict__ st)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n)
    return;
  Box box = leaf(p);
  uint32_t self = p | kLeafBit;
  uint32_t q = __ldg(leaf_parent + p);
  for (uint32_t depth = 0;; depth++) {
    if (q >= n - 1 || depth > 2 * kMaxTreeDepth) {
      atomicOr(&st->error, kErrBadTopology);
      return;
    }
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> f(flags[q]);
    const uint32_t old = f.fetch_add(1u, cuda::memory_order_acq_rel);
    if ((old & 1u) == 0)
      return;
    const uint2 lr = __ldg(child + q);
    const uint32_t lx = lr.x & ~kLeafBit, ly = lr.y & ~kLeafBit;
    if (((lr.x & kLeafBit) ? lx >= n : lx >= n - 1) || ((lr.y & kLeafBit) ? ly >= n : ly >= n - 1)) {
      atomicOr(&st->error, kErrBadTopology);
      return;
    }
    Box lb, rb;
    if (lr.x == self)
      lb = box;
    else if (lr.x & kLeafBit)
      lb = leaf(lr.x & ~kLeafBit);
    else {
      const float4 a = __ldcg(reinterpret_cast<const float4*>(nodes + lr.x));
      const float2 b = __ldcg(reinterpret_cast<const float2*>(nodes + lr.x) + 2);
      lb = Box{ { a.x, a.y, a.z }, { a.w, b.x, b.y } };
    }
    if (lr.y == self)
      rb = box;
    else if (lr.y & kLeafBit)
      rb = leaf(lr.y & ~kLeafBit);
    else {
      const float4 a = __ldcg(reinterpret_cast<const float4*>(nodes + lr.y));
      const float2 b = __ldcg(reinterpret_cast<const float2*>(nodes + lr.y) + 2);
      rb = Box{ { a.x, a.y, a.z }, { a.w, b.x, b.y } };
    }
    box = join(lb, rb);
    float4* dst = reinterpret_cast<float4*>(nodes + q);
    __stcg(dst + 0, make_float4(box.lo[0], box.lo[1], box.lo[2], box.hi[0]));
    __stcg(dst + 1, make_float4(box.hi[1], box.hi[2], __uint_as_float(lr.x), __uint_as_float(lr.y)));
    if (q == 0)
      return;
    self = q;
    q = __ldg(node_parent + q);
  }
}

// Sorted-leaf mode: gather triangles into Morton order (leaf slot p holds the
// p-th primitive of the stable sort) and keep the leaf -> primitive map.
__global__ void
k_gather_tris(const Tri* __restrict__ tris,
              const uint32_t* __restrict__ perm,
              uint32_t n,
              Tri* __restrict__ out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  out[i] = tris[__ldg(perm + i)];
}

__global__ void
k_gather_boxes(const Box* __restrict__ boxes,
               const uint32_t* __restrict__ perm,
               uint32_t n,
               Box* __restrict__ out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  out[i] = boxes[__ldg(perm + i)];
}

// ---------------------------------------------------------------------------
// host-side launchers

template<class Leaf>
static cudaError_t
launch_curve(const Leaf& leaf, uint32_t n, const BuildBuffers& b, cudaStream_t s)
{
  k_bounds<Leaf><<<b.bounds_blocks, kBoundsThreads, 0, s>>>(leaf, n, reinterpret_cast<ArgBox*>(b.partials), b.state);
  k_morton<Leaf><<<b.morton_blocks, kMortonThreads, 0, s>>>(leaf, n, b.keys_a, b.state);
  return cudaGetLastError();
}

cudaError_t
launch_sort(uint32_t n, bool pairs, uint32_t epoch_base, const BuildBuffers& b, cudaStream_t s)
{
  const uint32_t tiles = ceil_div_u32(n, kSortTile);
  uint32_t* ka = b.keys_a;
  uint32_t* kb = b.keys_b;
  uint32_t* va = b.vals_a;
  uint32_t* vb = b.vals_b;
  for (uint32_t pass = 0; pass < 4; pass++) {
    const uint32_t epoch = epoch_base + pass;
    if (pairs) {
      if (pass == 0)
        k_onesweep<true, true><<<tiles, kSortThreads, 0, s>>>(ka, kb, nullptr, vb, n, pass, epoch, b.lookback, b.state);
      else
        k_onesweep<true, false><<<tiles, kSortThreads, 0, s>>>(ka, kb, va, vb, n, pass, epoch, b.lookback, b.state);
    } else {
      k_onesweep<false, false><<<tiles, kSortThreads, 0, s>>>(ka, kb, nullptr, nullptr, n, pass, epoch, b.lookback, b.state);
    }
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  // four passes: sorted keys (and values) are back in keys_a / vals_a
  return cudaGetLastError();
}

template<class Leaf>
static cudaError_t
launch_topology_and_fit(const Leaf& leaf, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  k_split<<<ceil_div_u32(n - 1, kSplitThreads), kSplitThreads, 0, s>>>(b.keys_a, n, b.child, b.leaf_parent, b.node_parent);
  k_fit<Leaf><<<ceil_div_u32(n, kFitThreads), kFitThreads, 0, s>>>(
    leaf, n, b.child, b.leaf_parent, b.node_parent, b.flags, nodes, b.state);
  return cudaGetLastError();
}

cudaError_t
launch_make_triangles(const float* verts, uint32_t n, Tri* out, cudaStream_t s)
{
  if (n == 0)
    return cudaSuccess;
  k_make_triangles<<<ceil_div_u32(n, 256), 256, 0, s>>>(verts, n, out);
  return cudaGetLastError();
}

cudaError_t
launch_curve_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, cudaStream_t s)
{
  return launch_curve(TriLeaf{ tris }, n, b, s);
}

cudaError_t
launch_curve_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, cudaStream_t s)
{
  return launch_curve(BoxLeaf{ boxes }, n, b, s);
}

cudaError_t
launch_fit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  return launch_topology_and_fit(TriLeaf{ tris }, n, b, nodes, s);
}

cudaError_t
launch_fit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  return launch_topology_and_fit(BoxLeaf{ boxes }, n, b, nodes, s);
}

cudaError_t
launch_gather_tris(const Tri* tris, const uint32_t* perm, uint32_t n, Tri* out, cudaStream_t s)
{
  k_gather_tris<<<ceil_div_u32(n, 256), 256, 0, s>>>(tris, perm, n, out);
  return cudaGetLastError();
}

cudaError_t
launch_gather_boxes(const Box* boxes, const uint32_t* perm, uint32_t n, Box* out, cudaStream_t s)
{
  k_gather_boxes<<<ceil_div_u32(n, 256), 256, 0, s>>>(boxes, perm, n, out);
  return cudaGetLastError();
}

template<class Leaf>
static cudaError_t
launch_refit(const Leaf& leaf, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  k_links_from_nodes<<<ceil_div_u32(n - 1, 256), 256, 0, s>>>(nodes, n - 1, b.child, b.leaf_parent, b.node_parent);
  k_fit<Leaf><<<ceil_div_u32(n, kFitThreads), kFitThreads, 0, s>>>(
    leaf, n, b.child, b.leaf_parent, b.node_parent, b.flags, nodes, b.state);
  return cudaGetLastError();
}

cudaError_t
launch_refit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  return launch_refit(TriLeaf{ tris }, n, b, nodes, s);
}

cudaError_t
launch_refit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, cudaStream_t s)
{
  return launch_refit(BoxLeaf{ boxes }, n, b, nodes, s);
}

} // namespace lbvh_gb300
