// LBVH build kernels for sm_103a: centroid bounds, Morton codes + radix
// histograms, onesweep LSD radix sort, bottom-up tree construction fused with
// the box fit, and refit.
//
// Reference: tay10r/lbvh `lbvh.h`, builder<float>::operator() (lbvh.h:1793-1822).
// Every kernel reproduces the reference's outputs bit for bit; the comments on
// each kernel cite the reference code it replaces.
#include "build.cuh"
#include "device_util.cuh"

#include <atomic>

#include <cooperative_groups.h>

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

template<class Leaf>
__global__ __launch_bounds__(kBoundsThreads) void
k_bounds(Leaf leaf, uint32_t n, ArgBox* __restrict__ partials, BuildState* __restrict__ st, Box* __restrict__ box_out)
{
  pdl_begin(); // the predecessor in the stream has finished
  __shared__ ArgBox s_part[kBoundsThreads / 32];
  __shared__ bool s_last;
  const uint32_t chunk = ceil_div_u32(n, gridDim.x);
  const uint32_t b = blockIdx.x * chunk;
  const uint32_t e = min(n, b + chunk);
  ArgBox a = empty_arg();
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const Box bx = leaf(i);
    if (box_out) { // stage the leaf box: later passes read 24 bytes, not 48
      float2* o = reinterpret_cast<float2*>(box_out + i);
      o[0] = make_float2(bx.lo[0], bx.lo[1]);
      o[1] = make_float2(bx.lo[2], bx.hi[0]);
      o[2] = make_float2(bx.hi[1], bx.hi[2]);
    }
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
    st->tree_fallback = 0;
    st->bucket_next = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      st->tile_counter[k] = 0;
  }
  for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x)
    (&st->hist[0][0])[k] = 0;
  for (uint32_t k = threadIdx.x; k < kTopBuckets; k += blockDim.x)
    st->top_hist[k] = 0;
}

// ---------------------------------------------------------------------------
// Morton codes (morton_curve_kernel, lbvh.h:1422-1475 with morton_encoder<4>,
// lbvh.h:1345-1359): q = u32((center - min) * scale), code = x<<2 | y<<1 | z.
// Also accumulates the four 8-bit digit histograms the radix sort needs, so
// the sort never re-reads the codes just to count them. With kTop (the bucket
// sort of large keys-only builds) CTA b takes the codes [b * range, +range)
// and also writes their counts per bucket of the top 12 bits to row b of
// `rows`.
__device__ __forceinline__ uint32_t
morton_of(const Box& bx, float lo0, float lo1, float lo2, float s0, float s1, float s2)
{
  const float cx = fmul(fadd(bx.lo[0], bx.hi[0]), 0.5f);
  const float cy = fmul(fadd(bx.lo[1], bx.hi[1]), 0.5f);
  const float cz = fmul(fadd(bx.lo[2], bx.hi[2]), 0.5f);
  const uint32_t x = __float2uint_rz(fmul(fsub(cx, lo0), s0));
  const uint32_t y = __float2uint_rz(fmul(fsub(cy, lo1), s1));
  const uint32_t z = __float2uint_rz(fmul(fsub(cz, lo2), s2));
  return (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
}

template<class Leaf, bool kTop>
__global__ __launch_bounds__(kMortonThreads) void
k_morton(Leaf leaf, uint32_t n, uint32_t* __restrict__ codes, BuildState* __restrict__ st, uint32_t range,
         uint32_t* __restrict__ rows)
{
  pdl_begin(); // the predecessor in the stream has finished
  __shared__ uint32_t s_hist[4 * 256];
  __shared__ uint32_t s_top[kTop ? kTopBuckets : 1]; // buckets of the top 12 bits, for the bucket sort
  for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x)
    s_hist[k] = 0;
  if (kTop)
    for (uint32_t k = threadIdx.x; k < kTopBuckets; k += blockDim.x)
      s_top[k] = 0;
  __syncthreads();
  const float lo0 = st->lo[0], lo1 = st->lo[1], lo2 = st->lo[2];
  const float s0 = st->scale[0], s1 = st->scale[1], s2 = st->scale[2];
  const uint32_t stride = kTop ? blockDim.x : gridDim.x * blockDim.x;
  const uint32_t end = kTop ? (n - blockIdx.x * range < range ? n : blockIdx.x * range + range) : n;
  for (uint32_t i = (kTop ? blockIdx.x * range : blockIdx.x * blockDim.x) + threadIdx.x; i < end; i += stride) {
    const uint32_t code = morton_of(leaf(i), lo0, lo1, lo2, s0, s1, s2);
    codes[i] = code;
    atomicAdd(&s_hist[0 * 256 + (code & 255u)], 1u);
    atomicAdd(&s_hist[1 * 256 + ((code >> 8) & 255u)], 1u);
    atomicAdd(&s_hist[2 * 256 + ((code >> 16) & 255u)], 1u);
    atomicAdd(&s_hist[3 * 256 + (code >> 24)], 1u);
    if (kTop)
      atomicAdd(&s_top[code >> (30 - kTopBits)], 1u); // codes are 30 bits
  }
  __syncthreads();
  if (kTop)
    for (uint32_t k = threadIdx.x; k < kTopBuckets; k += blockDim.x) {
      const uint32_t c = s_top[k];
      rows[size_t(blockIdx.x) * kTopBuckets + k] = c;
      if (c)
        atomicAdd(&st->top_hist[k], c);
    }
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

template<bool kPairs, bool kIotaVals, int kItems = kSortItems>
__global__ __launch_bounds__(kSortThreads, kPairs ? 3 : 4) void
k_onesweep(const uint32_t* __restrict__ kin,
           uint32_t* __restrict__ kout,
           const uint32_t* __restrict__ vin,
           uint32_t* __restrict__ vout,
           uint32_t n,
           uint32_t pass,
           uint32_t epoch,
           unsigned long long* __restrict__ lookback,
           BuildState* __restrict__ st,
           bool skip_if_msd,
           uint32_t spin_limit,
           uint32_t wait_xor,
           uint32_t tiles)
{
  pdl_begin(); // the predecessor in the stream has finished
  constexpr int kTile = kSortThreads * kItems;
  if (skip_if_msd && st->use_msd)
    return; // the bucket sort did this build's sorting
  __shared__ uint32_t s_keys[kTile];
  __shared__ uint32_t s_vals[kPairs ? kTile : 1];
  __shared__ uint32_t s_whist[kSortWarps][256];
  __shared__ uint32_t s_tile_start[256];
  __shared__ uint32_t s_gbase[256];
  __shared__ uint32_t s_warp[kSortWarps];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // A grid smaller than the tile count (the fallback passes of a bucket
  // sort, which usually return at once) takes tiles until none is left;
  // tiles are dispensed in order, so every look-back waits only on tiles
  // that running CTAs hold.
  const bool looping = gridDim.x < tiles;
  for (;;) {
  if (tid == 0)
    s_tile = atomicAdd(&st->tile_counter[pass], 1u);
  for (int i = tid; i < kSortWarps * 256; i += kSortThreads)
    (&s_whist[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  if (tile >= tiles)
    break; // uniform: every tile is taken
  const uint32_t base = tile * uint32_t(kTile);
  const uint32_t shift = pass * 8;

  // digits are recomputed from the keys where needed (fewer live registers)
  const uint32_t first = base + uint32_t(warp) * (32 * kItems) + lane;
  // the top pass of 30-bit codes has 6-bit digits; ranking, counters and
  // positions all use the same masked digit, so the tile's positions stay
  // inside the tile whatever words it is given
  const uint32_t dmask = pass == 3 ? 63u : 255u;
  auto digit = [&](uint32_t kv, int k) -> uint32_t {
    return first + uint32_t(k) * 32 < n ? (kv >> shift) & dmask : 256u; // 256: not a key, in no bucket
  };
  uint32_t key[kItems], val[kPairs ? kItems : 1], rank[kItems];
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const uint32_t idx = first + uint32_t(k) * 32;
    key[k] = idx < n ? kin[idx] : 0u;
    if (kPairs)
      val[kPairs ? k : 0] = idx < n ? (kIotaVals ? idx : vin[idx]) : 0u;
  }

  // warp-level stable ranking: items in (k, lane) order are in index order.
  // Lanes with the same digit are found with one ballot per digit bit (a
  // cost that does not grow with the number of distinct digits in the warp;
  // the top pass has 6-bit digits); a partial tile also masks out its
  // non-keys.
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t digit_bits = pass == 3 ? 6u : 8u; // the bits of dmask
  const bool full_tile = base + uint32_t(kTile) <= n;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const uint32_t d = digit(key[k], k);
    uint32_t peers = full_tile ? 0xffffffffu : __ballot_sync(0xffffffffu, d < 256);
#pragma unroll
    for (uint32_t b = 0; b < 8; b++) {
      if (b < digit_bits) {
        const uint32_t bit = (d >> b) & 1u;
        const uint32_t m = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? m : ~m;
      }
    }
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

  // Decoupled look-back over earlier tiles, kLookbackWindow words per poll:
  // add aggregates until an inclusive prefix; stop at a word not yet published
  // and poll again from there.
  uint32_t excl = 0;
  if (tile > 0) {
    const uint32_t want = epoch ^ wait_xor; // the tag earlier tiles publish (wait_xor: 0)
    uint32_t p = tile - 1; // next tile to read
    uint32_t spins = 0;
    bool done = false;
    while (!done) {
      unsigned long long e[kLookbackWindow];
#pragma unroll
      for (int w = 0; w < kLookbackWindow; w++)
        e[w] = (uint32_t(w) <= p) ? ld_relaxed_u64(lookback + size_t(p - w) * 256 + tid) : 0ull;
      uint32_t used = 0;
#pragma unroll
      for (int w = 0; w < kLookbackWindow; w++) {
        if (done || used != uint32_t(w) || uint32_t(w) > p)
          continue;
        const uint32_t lo = uint32_t(e[w]);
        const uint32_t status = lo >> 30;
        if (uint32_t(e[w] >> 32) != want || status == 0)
          continue; // not yet published: poll again from here
        excl += lo & 0x3fffffffu;
        used++;
        done = status == 2 || p - w == 0;
      }
      if (done)
        break;
      if (used) {
        p -= used;
        spins = 0;
      } else if (++spins > spin_limit) {
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
  for (int k = 0; k < kItems; k++) {
    const uint32_t d = digit(key[k], k);
    if (d < 256) {
      const uint32_t pos = s_tile_start[d] + s_whist[warp][d] + rank[k];
      s_keys[pos] = key[k];
      if (kPairs)
        s_vals[pos] = val[kPairs ? k : 0];
    }
  }
  __syncthreads();

  // write out: consecutive positions of one digit go to consecutive addresses
  const uint32_t tile_n = min(uint32_t(kTile), n - base);
  for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t d = (k >> shift) & dmask;
    const uint32_t o = s_gbase[d] + i - s_tile_start[d];
    if (o < n) { // always true unless a look-back wait gave up
      kout[o] = k;
      if (kPairs)
        vout[o] = s_vals[i];
    }
  }
  if (!looping)
    break;
  __syncthreads(); // the next tile reuses the shared arrays
  }
}

// ---------------------------------------------------------------------------
// Keys-only sort of large builds by buckets. Only the sorted code sequence
// reaches the tree (leaf p is primitive p), so equal codes may land in any
// order. The codes are partitioned by their top 12 bits into 4,096 buckets,
// then each bucket is sorted by its low 18 bits in shared memory by one CTA.
//
//   k_morton (kTop)  one CTA per range of `range` consecutive codes: writes
//                    the range's bucket counts as one row of `rows`
//                    [ranges][4096] and adds them to st->top_hist;
//   k_top_scan       bucket starts (st->top_base), the choice of path, and
//                    each range's start in each bucket (column prefix sums of
//                    `rows`, in place);
//   k_partition      one CTA per range: places its codes at those starts
//                    (shared-memory atomics rank the codes of a tile, so no
//                    global atomics);
//   k_bucket_sort    one CTA per bucket: an unstable pass by bits 0-8 into
//                    shared memory, then a stable pass by bits 9-17 into the
//                    output; the first pass may be unstable because codes
//                    equal in all 30 bits are interchangeable.
//
// k_top_scan chooses this path when every bucket holds at most kBucketMax
// codes, the four onesweep passes otherwise; both are launched and the
// unchosen kernels return at once, so the choice needs no host read-back.

// Exclusive scan of one value per thread over a block of kWarps warps.
template<int kWarps>
__device__ __forceinline__ uint32_t
block_excl_scan(uint32_t v, uint32_t* s_warp)
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
    const uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
    uint32_t t = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o)
        t += y;
    }
    if (lane < kWarps)
      s_warp[lane] = t - w;
  }
  __syncthreads();
  const uint32_t r = x - v + s_warp[warp];
  __syncthreads();
  return r;
}

// kTopBuckets / 32 CTAs of 1,024 threads; CTA b owns buckets [32b, 32b + 32)
// (lane = bucket): warp w sums its block of rows, the warps' sums are
// scanned through shared memory, and warp w rewrites its rows as starts.
// Every access to `rows` is one 128-byte line per warp.
__global__ __launch_bounds__(1024) void
k_top_scan(uint32_t* __restrict__ rows, uint32_t nrows, BuildState* __restrict__ st)
{
  pdl_begin(); // the predecessor in the stream has finished
  constexpr int kPer = kTopBuckets / 1024;
  constexpr uint32_t kBatch = 8;
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_max;
  __shared__ uint32_t s_base[kTopBuckets];
  __shared__ uint32_t s_part[32][33];
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0)
    s_max = 0;
  __syncthreads();
  // every CTA scans the bucket totals (16 KB); CTA 0 publishes them
  uint32_t c[kPer], sum = 0, mx = 0;
#pragma unroll
  for (int j = 0; j < kPer; j++) {
    c[j] = st->top_hist[kPer * t + j];
    sum += c[j];
    mx = max(mx, c[j]);
  }
  atomicMax(&s_max, mx);
  uint32_t ex = block_excl_scan<32>(sum, s_warp);
#pragma unroll
  for (int j = 0; j < kPer; j++) {
    s_base[kPer * t + j] = ex;
    if (blockIdx.x == 0)
      st->top_base[kPer * t + j] = ex;
    ex += c[j];
  }
  const bool use = s_max <= kBucketMax;
  if (blockIdx.x == 0) {
    if (t == 1023)
      st->top_base[kTopBuckets] = ex; // == n
    if (t == 0)
      st->use_msd = use ? 1u : 0u;
    // the non-empty buckets in ascending order, for the bucket sort's CTAs
    uint32_t nz = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++)
      nz += c[j] != 0;
    uint32_t at = block_excl_scan<32>(nz, s_warp);
#pragma unroll
    for (int j = 0; j < kPer; j++)
      if (c[j] != 0)
        st->top_list[at++] = kPer * t + j;
    if (t == 1023)
      st->top_nonempty = at;
  }
  if (!use)
    return; // uniform over the CTA
  const uint32_t d = blockIdx.x * 32 + lane;
  const uint32_t per = (nrows + 31) / 32;
  const uint32_t r_lo = min(nrows, warp * per);
  const uint32_t r_hi = min(nrows, r_lo + per);
  uint32_t part = 0;
#pragma unroll 1
  for (uint32_t r0 = r_lo; r0 < r_hi; r0 += kBatch) {
    uint32_t v[kBatch];
#pragma unroll
    for (uint32_t u = 0; u < kBatch; u++)
      v[u] = r0 + u < r_hi ? rows[size_t(r0 + u) * kTopBuckets + d] : 0u;
#pragma unroll
    for (uint32_t u = 0; u < kBatch; u++)
      part += v[u];
  }
  s_part[warp][lane] = part;
  __syncthreads();
  uint32_t run = s_base[d];
  for (uint32_t w = 0; w < warp; w++)
    run += s_part[w][lane];
#pragma unroll 1
  for (uint32_t r0 = r_lo; r0 < r_hi; r0 += kBatch) {
    uint32_t v[kBatch];
#pragma unroll
    for (uint32_t u = 0; u < kBatch; u++)
      v[u] = r0 + u < r_hi ? rows[size_t(r0 + u) * kTopBuckets + d] : 0u;
#pragma unroll
    for (uint32_t u = 0; u < kBatch; u++)
      if (r0 + u < r_hi) {
        rows[size_t(r0 + u) * kTopBuckets + d] = run;
        run += v[u];
      }
  }
}

// One CTA per range [blockIdx.x * range, +range) of the unsorted codes
// (`group` consecutive ranges of the Morton pass, so its starts are the
// first of their rows), in tiles of kPartTile: each tile's codes are ranked within their bucket by
// shared-memory atomics, grouped by bucket in shared memory and written at
// the range's running position in each bucket (runs of consecutive codes).
// Tiles arrive by cp.async into two shared buffers: the next tile is in
// flight while the current one is ranked, and a tile's buffer then holds its
// regrouped codes.
__global__ __launch_bounds__(kPartThreads) void
k_partition(const uint32_t* __restrict__ kin, uint32_t* __restrict__ kout, uint32_t n, uint32_t range,
            uint32_t group, const uint32_t* __restrict__ rows, const BuildState* __restrict__ st)
{
  pdl_begin(); // the predecessor in the stream has finished
  if (!st->use_msd)
    return;
  constexpr int kPer = kTopBuckets / kPartThreads; // buckets per thread in the scans
  constexpr uint32_t kChunks = kPartTile / 4 / kPartThreads; // 16-byte copies per thread per tile
  extern __shared__ __align__(16) uint32_t smem_p[];
  uint32_t* s_cur = smem_p;                   // [kTopBuckets] the range's next output position per bucket
  uint32_t* s_start = s_cur + kTopBuckets;    // [kTopBuckets] counts, then the tile's bucket starts
  uint32_t* s_stage = s_start + kTopBuckets;  // [2][kPartTile] tiles as loaded, then regrouped
  __shared__ uint32_t s_warp[32];
  const uint32_t tid = threadIdx.x;
  const uint32_t lo = blockIdx.x * range;     // a multiple of 256 codes: 16-byte aligned
  const uint32_t hi = n - lo < range ? n : lo + range;
  // tile `base` -> s_stage[buf]; a copy past hi reads only the codes below hi
  auto fetch = [&](uint32_t base, uint32_t buf) {
#pragma unroll
    for (uint32_t j = 0; j < kChunks; j++) {
      const uint32_t c = j * kPartThreads + tid; // 16-byte chunk within the tile
      const uint32_t i = base + 4 * c;
      const uint32_t bytes = i < hi ? min(16u, 4 * (hi - i)) : 0u;
      copy16_async(s_stage + buf * kPartTile + 4 * c, bytes ? kin + i : kin, bytes);
    }
  };
  for (uint32_t k = tid; k < kTopBuckets; k += kPartThreads)
    s_cur[k] = rows[size_t(blockIdx.x) * group * kTopBuckets + k]; // the range's first row
  fetch(lo, 0);
  copy_async_commit();
  uint32_t buf = 0;
#pragma unroll 1
  for (uint32_t base = lo; base < hi; base += kPartTile, buf ^= 1u) {
    if (base + kPartTile < hi)
      fetch(base + kPartTile, buf ^ 1u);
    copy_async_commit();
    for (uint32_t k = tid; k < kTopBuckets; k += kPartThreads)
      s_start[k] = 0;
    copy_async_wait<1>(); // this tile's copies (all but the newest group)
    __syncthreads();
    uint32_t* tile = s_stage + buf * kPartTile;
    uint32_t key[kPartItems], pk[kPartItems]; // pk: rank in the tile's bucket << 12 | bucket
#pragma unroll
    for (int k = 0; k < kPartItems; k++)
      key[k] = tile[uint32_t(k) * kPartThreads + tid];
#pragma unroll
    for (int k = 0; k < kPartItems; k++) {
      const uint32_t idx = base + uint32_t(k) * kPartThreads + tid;
      pk[k] = 0xffffffffu;
      if (idx < hi) {
        const uint32_t d = key[k] >> (30 - kTopBits); // codes are 30 bits
        pk[k] = (atomicAdd(&s_start[d], 1u) << kTopBits) | d;
      }
    }
    __syncthreads();
    uint32_t c[kPer], sum = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      c[j] = s_start[kPer * tid + j];
      sum += c[j];
    }
    uint32_t ex = block_excl_scan<kPartThreads / 32>(sum, s_warp);
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      s_start[kPer * tid + j] = ex;
      ex += c[j];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPartItems; k++)
      if (pk[k] != 0xffffffffu)
        tile[s_start[pk[k] & (kTopBuckets - 1)] + (pk[k] >> kTopBits)] = key[k];
    __syncthreads();
    const uint32_t tile_n = min(uint32_t(kPartTile), hi - base);
    for (uint32_t i = tid; i < tile_n; i += kPartThreads) {
      const uint32_t k = tile[i];
      const uint32_t d = k >> (30 - kTopBits);
      kout[s_cur[d] + (i - s_start[d])] = k;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPer; j++)
      s_cur[kPer * tid + j] += c[j];
  }
  copy_async_wait<0>();
}

// Persistent CTAs of 1,024 threads (one per SM) take the non-empty buckets
// from st->top_list in turn. Per bucket: the codes are read once (into
// shared buffer A, counted on the way); an unstable counting pass by bits
// 0-12 (shared-memory atomics) scatters them into shared buffer B; a stable pass by bits 13-17 ranks them
// per warp (one ballot per digit bit, up to kBucketChunk codes per step,
// spread evenly over the warps) into shared buffer A, which is written out
// in order.
__global__ __launch_bounds__(kBucketThreads, 1) void
k_bucket_sort(const uint32_t* __restrict__ kin, uint32_t* __restrict__ kout, BuildState* __restrict__ st)
{
  pdl_begin(); // the predecessor in the stream has finished
  if (!st->use_msd)
    return;
  constexpr int kWarps = kBucketThreads / 32;
  constexpr uint32_t kPerThread = kBucketMax / kBucketThreads;
  constexpr int kFirstPer = kFirstDigits / kBucketThreads;
  constexpr uint32_t kFirstMask = kFirstDigits - 1, kSecondMask = kSecondDigits - 1;
  constexpr uint32_t kInvalid = 0xffffffffu; // codes are 30 bits
  static_assert(kBucketMax % kBucketThreads == 0, "whole codes per thread");
  static_assert(kFirstDigits % kBucketThreads == 0, "whole first-pass digits per thread");
  static_assert(kSecondDigits == kWarps, "one second-pass digit per warp in the offset scan");
  static_assert(kFirstBits + kSecondBits == 30 - kTopBits, "the passes cover the bits below the bucket");
  extern __shared__ __align__(16) uint32_t smem_b[];
  uint32_t* A = smem_b;                                                     // [kBucketMax]
  uint32_t* B = A + kBucketMax;                                             // [kBucketMax]
  uint32_t* s_first = B + kBucketMax;                                       // [kFirstDigits]
  uint32_t* s_run = s_first + kFirstDigits;                                 // [kSecondDigits]
  uint16_t* whist = reinterpret_cast<uint16_t*>(s_run + kSecondDigits);     // [kWarps][kSecondDigits]
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_take;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t buckets = st->top_nonempty;

#pragma unroll 1
  for (;;) {
    if (tid == 0)
      s_take = atomicAdd(&st->bucket_next, 1u);
    __syncthreads();
    const uint32_t take = s_take;
    if (take >= buckets)
      break; // uniform over the CTA
    const uint32_t bkt = st->top_list[take];
    const uint32_t cnt = st->top_hist[bkt]; // <= kBucketMax when use_msd is set
    const uint32_t start = st->top_base[bkt];
    const uint32_t* src = kin + start;

#pragma unroll
    for (int j = 0; j < kFirstPer; j++)
      s_first[kFirstPer * tid + j] = 0;
    if (tid < kSecondDigits)
      s_run[tid] = 0;
    uint32_t v[kPerThread];
#pragma unroll
    for (uint32_t u = 0; u < kPerThread; u++) {
      const uint32_t i = u * kBucketThreads + tid;
      v[u] = i < cnt ? __ldcs(src + i) : kInvalid;
    }
    __syncthreads(); // also: every thread has read s_take
#pragma unroll
    for (uint32_t u = 0; u < kPerThread; u++)
      if (u * kBucketThreads < cnt && v[u] != kInvalid) {
        A[u * kBucketThreads + tid] = v[u];
        atomicAdd(&s_first[v[u] & kFirstMask], 1u);
        atomicAdd(&s_run[(v[u] >> kFirstBits) & kSecondMask], 1u);
      }
    __syncthreads();
    {
      uint32_t sum = 0;
#pragma unroll
      for (int j = 0; j < kFirstPer; j++)
        sum += s_first[kFirstPer * tid + j];
      // warp 0 scans the second-pass histogram (one digit per lane) meanwhile
      uint32_t h = 0, hx = 0;
      if (warp == 0) {
        h = s_run[lane];
        uint32_t x = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o)
            x += y;
        }
        hx = x - h;
      }
      uint32_t ex = block_excl_scan<kWarps>(sum, s_warp);
#pragma unroll
      for (int j = 0; j < kFirstPer; j++) {
        const uint32_t cj = s_first[kFirstPer * tid + j]; // this thread's own digits
        s_first[kFirstPer * tid + j] = ex;
        ex += cj;
      }
      if (warp == 0)
        s_run[lane] = hx;
    }
    __syncthreads();
    // unstable pass by bits 0-12: A -> B
#pragma unroll 4
    for (uint32_t i = tid; i < cnt; i += kBucketThreads) {
      const uint32_t k = A[i];
      B[atomicAdd(&s_first[k & kFirstMask], 1u)] = k;
    }
    __syncthreads();
    // stable pass by bits 13-17: B -> A
#pragma unroll 1
    for (uint32_t c0 = 0; c0 < cnt; ) {
      const uint32_t ipw = min(uint32_t(kBucketItems), (cnt - c0 + kBucketThreads - 1) / kBucketThreads);
      const uint32_t step = ipw * kBucketThreads;
      const bool full = c0 + step <= cnt;
      if (tid < kWarps * kSecondDigits / 2)
        reinterpret_cast<uint32_t*>(whist)[tid] = 0;
      __syncthreads();
      const uint32_t first = c0 + warp * ipw * 32 + lane;
      uint32_t key[kBucketItems], rank[kBucketItems];
      // the lanes holding the same digit, for every item first (independent
      // ballots), then the items' counts in order through the warp's histogram
#pragma unroll
      for (int k = 0; k < kBucketItems; k++) {
        if (uint32_t(k) < ipw) {
          const uint32_t idx = first + uint32_t(k) * 32;
          key[k] = (full || idx < cnt) ? B[idx] : kInvalid;
          const uint32_t d = (key[k] >> kFirstBits) & kSecondMask; // invalid: matches no valid lane
          uint32_t peers = full ? 0xffffffffu : __ballot_sync(0xffffffffu, key[k] != kInvalid);
#pragma unroll
          for (uint32_t b = 0; b < kSecondBits; b++) {
            const uint32_t bit = (d >> b) & 1u;
            const uint32_t m = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? m : ~m;
          }
          rank[k] = peers;
        }
      }
#pragma unroll
      for (int k = 0; k < kBucketItems; k++) {
        if (uint32_t(k) < ipw) {
          const bool valid = key[k] != kInvalid;
          const uint32_t d = (key[k] >> kFirstBits) & kSecondMask;
          const uint32_t peers = rank[k];
          const uint32_t pre = __popc(peers & lt_mask);
          uint32_t before = 0;
          if (valid)
            before = whist[warp * kSecondDigits + d];
          __syncwarp();
          if (valid && pre == 0)
            whist[warp * kSecondDigits + d] = uint16_t(before + __popc(peers));
          __syncwarp();
          rank[k] = before + pre;
        }
      }
      __syncthreads();
      // per digit, exclusive offsets over the warps: warp w scans digit w
      // with lane = the warp whose count it holds
      uint32_t tot;
      {
        const uint32_t i0 = lane * kSecondDigits + warp;
        const uint32_t cw = whist[i0];
        uint32_t x = cw;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o)
            x += y;
        }
        whist[i0] = uint16_t(x - cw);
        tot = __shfl_sync(0xffffffffu, x, 31);
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kBucketItems; k++) {
        if (uint32_t(k) < ipw && key[k] != kInvalid) {
          const uint32_t d = (key[k] >> kFirstBits) & kSecondMask;
          A[s_run[d] + whist[warp * kSecondDigits + d] + rank[k]] = key[k];
        }
      }
      __syncthreads();
      if (lane == 0)
        s_run[warp] += tot;
      c0 += step;
    }
    __syncthreads();
    uint32_t* dst = kout + start;
    for (uint32_t i = tid; i < cnt; i += kBucketThreads)
      dst[i] = A[i];
    // the next bucket's first writes to s_first / s_run / B / A all follow
    // at least one more barrier; A is read here, written after three
  }
}

// ---------------------------------------------------------------------------
// Tree construction fused with the box fit. Replaces the reference's
// per-node split search (divide_node + builder_kernel, lbvh.h:1588-1731) and
// its serial fit (builder::fit_boxes, lbvh.h:1826-1867) with one bottom-up
// pass that produces the identical node array.
//
// The reference's tree is the binary radix tree over the sorted codes made
// distinct by their positions: delta(i, j) = clz(code_i ^ code_j), or
// clz(i ^ j) + 32 on equal codes, -1 out of range (lbvh.h:1602-1621). Node
// i's range has i at one end and is split at gamma; its children are gamma
// (range ending at gamma) and gamma + 1 (range starting there), with the leaf
// bit when a child range is a single slot (lbvh.h:1718-1729). So a node that
// is its parent's left child is stored at its range's right end, a right
// child at its left end, and the root [0, n-1] at 0.
//
// Bottom-up: a node [L, R] is its parent's left child exactly when
// delta(R, R+1) > delta(L-1, L) (the two can never be equal), and the
// parent's split is then R, else L - 1. One thread starts at every leaf slot;
// at each node it knows its range, hence its own index, writes its record,
// and arrives at its parent's slot. The first of the two children to arrive
// leaves its far range end in the slot and stops; the second reads it, has
// the parent's range, split and children, fits the parent's box (left box,
// then union with the right, as the reference does) and carries on upwards.
//
// A slot is one 64-bit word {epoch, far end} swapped atomically: a word from
// an earlier build carries another epoch, so slots are never cleared. A
// child's node record is published with a fence before the swap, and read
// after one, only when that child is an internal node; leaf boxes are
// recomputed from the primitives.

// Two phases.
//
// Local phase (k_tree_local), one CTA per kTreeBlock consecutive leaf slots:
// every node whose range lies inside the CTA's slots finds its parent's
// arrival slot and its sibling's record in shared memory, and threads walk up
// with block-scope acquire-release exchanges on shared memory only. Lanes take leaf
// slots from a CTA queue (one shared atomic per warp refill), so a lane whose
// walk ended starts the next one instead of idling while its warp finishes.
// A walk ends at a first arrival, or at a node whose parent's split lies on
// the CTA's edge (a "CTA root"). After a barrier, a slot holding a single
// arrival marks a node whose sibling range leaves the CTA. Those nodes and the
// CTA roots -- the canonical pieces of the CTA's slot range, at most two per
// tree level, which together cover the range -- are written out in leaf
// order; the CTA's finished records are written out coalesced.
//
// Merge phase (k_tree_merge, below): the nodes above the pieces, built window
// by window in shared memory. (With LBVH_PARAM_TREE_WALK_FUSED the local
// phase's own threads walk its pieces up through the global epoch-tagged
// slots instead; every record such a thread writes is published by the
// release half of its next global arrival, an acq_rel exchange.)

struct PendingNode
{
  uint32_t L, R;
  Box box;
};
static_assert(sizeof(PendingNode) == 32, "pending record layout");

// A piece record as two 16-byte stores / loads (records start on 32 bytes).
__device__ __forceinline__ void
store_piece(PieceRec* p, uint32_t R, int dR, const Box& b)
{
  float4* dst = reinterpret_cast<float4*>(p);
  dst[0] = make_float4(__uint_as_float(R), __int_as_float(dR), b.lo[0], b.lo[1]);
  dst[1] = make_float4(b.lo[2], b.hi[0], b.hi[1], b.hi[2]);
}

__device__ __forceinline__ Box
load_piece_box(const PieceRec* p)
{
  const float4 a = __ldcg(reinterpret_cast<const float4*>(p)), c = __ldcg(reinterpret_cast<const float4*>(p) + 1);
  return Box{ { a.z, a.w, c.x }, { c.y, c.z, c.w } };
}

constexpr uint32_t kSlotEmpty = 0xffffffffu;    // no arrival yet
constexpr uint32_t kSlotComplete = 0xfffffffeu; // both children arrived

// The walk of one pending node [L, R] (box `box`) up through the global
// epoch-tagged arrival slots: at each parent the first of the two children
// to arrive parks its far range end and stops, the second completes the
// parent (its record is published by the release half of this thread's next
// arrival) and climbs on. Node records the sibling's walk wrote are read
// after the acquire half of this thread's arrival. kOneCta: every walk of
// the tree runs in one CTA, so the arrivals are ordered at block scope.
template<class Leaf, bool kOneCta = false>
__device__ __forceinline__ void
walk_global(const Leaf& leaf, uint32_t n, const uint32_t* __restrict__ codes, unsigned long long* __restrict__ slots,
            Node* __restrict__ nodes, BuildState* __restrict__ st, uint32_t epoch, uint32_t L, uint32_t R, Box box)
{
  const unsigned long long tag = (unsigned long long)epoch << 32;
  bool is_left = boundary_delta(codes, n, R) > boundary_delta(codes, n, L - 1);
  for (uint32_t depth = 0;; depth++) {
    if (depth > kMaxTreeDepth + 2) {
      atomicOr(&st->error, kErrBadTopology);
      return;
    }
    const uint32_t s = is_left ? R : L - 1;
    const unsigned long long v = tag | (is_left ? L : R);
    const unsigned long long old = kOneCta ? arrive_acq_rel_cta_global(slots + s, v) : arrive_acq_rel(slots + s, v);
    if (uint32_t(old >> 32) != epoch)
      return; // first arrival: the sibling completes the parent
    const uint32_t far = uint32_t(old);
    const uint32_t LP = is_left ? L : far, RP = is_left ? far : R;
    const uint32_t cl = (LP == s) ? (s | kLeafBit) : s;
    const uint32_t cr = (RP == s + 1) ? ((s + 1) | kLeafBit) : (s + 1);
    const uint32_t sib = is_left ? cr : cl;
    Box other;
    if (sib & kLeafBit)
      other = leaf(sib & ~kLeafBit);
    else
      other = load_node_box(nodes, sib); // published before the sibling's swap, seen after ours
    box = is_left ? join(box, other) : join(other, box);
    L = LP;
    R = RP;
    if (L == 0 && R == n - 1) {
      store_node(nodes, 0, box, cl, cr);
      return;
    }
    is_left = boundary_delta(codes, n, R) > boundary_delta(codes, n, L - 1);
    store_node(nodes, is_left ? R : L, box, cl, cr);
  }
}

// The local phase's walks over one CTA's kSlots leaf slots [b0, b0 + count):
// s_delta holds the boundaries b0 - 1 .. b0 + kSlots - 1, s_slot / s_rec
// start empty, *s_next / *s_npend at 0. Records of the nodes completed here
// go to s_rec (by Karras index - b0), the CTA roots to s_pend.
template<uint32_t kSlots, class Leaf>
__device__ __forceinline__ void
local_walks(const Leaf& leaf, uint32_t n, uint32_t b0, uint32_t count, const int* s_delta, uint32_t* s_slot,
            Node* s_rec, PendingNode* s_pend, uint32_t* s_next, uint32_t* s_npend)
{
  const uint32_t lane = threadIdx.x & 31;
  bool active = false, internal = false;
  uint32_t L = 0, R = 0, lref = 0, rref = 0;
  Box box{};
  const uint32_t lt_mask = (1u << lane) - 1u;
  bool drained = false; // warp-uniform: the queue had no slot left at this warp's last refill
  for (;;) {
    // ---- lanes without a walk take the next leaf slots of the CTA ----
    const uint32_t idle = __ballot_sync(0xffffffffu, !active);
    if (idle && !drained) {
      uint32_t first = 0;
      if ((idle & lt_mask) == 0 && !active)
        first = atomicAdd(s_next, uint32_t(__popc(idle)));
      first = __shfl_sync(0xffffffffu, first, __ffs(idle) - 1);
      drained = first + __popc(idle) >= count;
      if (!active) {
        const uint32_t j = first + __popc(idle & lt_mask);
        if (j < count) {
          L = R = b0 + j;
          box = leaf(L);
          internal = false;
          active = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, active))
      break; // the queue is empty and every walk has ended
    if (!active)
      continue;

    // ---- one step of the walk ----
    const bool is_left = s_delta[R - b0 + 1] > s_delta[L - b0]; // delta(R) vs delta(L - 1)
    const uint32_t s = is_left ? R : L - 1;
    if (internal)
      stage_record_at(s_rec, (is_left ? R : L) - b0, box, lref, rref);
    if (s < b0 || s + 1 >= b0 + kSlots) { // split on the CTA's edge
      const uint32_t k = atomicAdd(s_npend, 1u);
      if (k < kTreePendingPerBlock)
        s_pend[k] = PendingNode{ L, R, box };
      active = false;
      continue;
    }
    // release publishes this thread's staged record, acquire makes the
    // sibling's visible
    const uint32_t old = arrive_acq_rel_cta(s_slot + (s - b0), is_left ? L : R);
    if (old == kSlotEmpty) {
      active = false; // first arrival: recoverable from the slot if unmatched
      continue;
    }
    s_slot[s - b0] = kSlotComplete; // read only after the block barrier below
    const uint32_t LP = is_left ? L : old, RP = is_left ? old : R;
    const uint32_t cl = (LP == s) ? (s | kLeafBit) : s;
    const uint32_t cr = (RP == s + 1) ? ((s + 1) | kLeafBit) : (s + 1);
    const uint32_t sib = is_left ? cr : cl;
    Box other;
    if (sib & kLeafBit) {
      other = leaf(sib & ~kLeafBit);
    } else {
      other = staged_box_at(s_rec, sib - b0);
    }
    box = is_left ? join(box, other) : join(other, box);
    L = LP;
    R = RP;
    lref = cl;
    rref = cr;
    internal = true;
    if (L == 0 && R == n - 1) { // the root: the whole tree fits in this CTA
      stage_record_at(s_rec, 0, box, lref, rref);
      active = false;
    }
  }
}

// After the walks and a barrier: the coalesced write-out of the records
// finished in the CTA, and the first arrivals that were never matched (nodes
// whose sibling range leaves the CTA) added to s_pend.
template<uint32_t kSlots, class Leaf>
__device__ __forceinline__ void
local_write_out(const Leaf& leaf, uint32_t n, uint32_t b0, Node* __restrict__ nodes, const uint32_t* s_slot,
                const Node* s_rec, PendingNode* s_pend, uint32_t* s_npend)
{
  for (uint32_t j = threadIdx.x; j < kSlots; j += blockDim.x) {
    const float4 ra = *rec_half(s_rec, j, 0), rb = *rec_half(s_rec, j, 1);
    const uint32_t rl = __float_as_uint(rb.z), rr = __float_as_uint(rb.w);
    if (rl != 0 && b0 + j + 1 < n)
      store_node(nodes, b0 + j, Box{ { ra.x, ra.y, ra.z }, { ra.w, rb.x, rb.y } }, rl, rr);
    const uint32_t v = s_slot[j];
    if (v != kSlotEmpty && v != kSlotComplete) {
      const uint32_t sj = b0 + j;
      // the waiter was the left child [v, s] (v <= s) or the right [s + 1, v]
      const uint32_t wl = v <= sj ? v : sj + 1, wr = v <= sj ? sj : v;
      Box wb;
      if (wl == wr) {
        wb = leaf(wl);
      } else {
        wb = staged_box_at(s_rec, (v <= sj ? wr : wl) - b0);
      }
      const uint32_t k = atomicAdd(s_npend, 1u);
      if (k < kTreePendingPerBlock)
        s_pend[k] = PendingNode{ wl, wr, wb };
    }
  }
}

template<class Leaf>
__global__ __launch_bounds__(kTreeThreads) void
k_tree_local(Leaf leaf,
             uint32_t n,
             const uint32_t* __restrict__ codes,
             Node* __restrict__ nodes,
             PieceRec* __restrict__ pieces_out,
             PieceHdr* __restrict__ hdr_out,
             BuildState* __restrict__ st,
             unsigned long long* __restrict__ slots,
             uint32_t epoch,
             bool walk_on)
{
  pdl_begin(); // the predecessor in the stream has finished
  extern __shared__ __align__(32) unsigned char smem[];
  int* s_delta = reinterpret_cast<int*>(smem);                               // kTreeBlock + 1
  uint32_t* s_slot = reinterpret_cast<uint32_t*>(s_delta + kTreeBlock + 8);   // kTreeBlock
  Node* s_rec = reinterpret_cast<Node*>(s_slot + kTreeBlock);                 // kTreeBlock
  __shared__ PendingNode s_pend[kTreePendingPerBlock];
  __shared__ uint32_t s_next, s_npend;

  const uint32_t tid = threadIdx.x;
  const uint32_t b0 = blockIdx.x * kTreeBlock;
  const uint32_t count = min(kTreeBlock, n - b0);
  // A sort that gave up leaves codes in no order, over which a walk could
  // leave its CTA's ranges: then no tree is built (the error is reported).
  // The sort kernels have finished, so every thread reads the same bit.
  const uint32_t sort_failed = __ldcg(&st->error) & kErrLookbackTimeout;

  // boundaries k = b0 - 1 .. b0 + kTreeBlock - 1 at s_delta[k - (b0 - 1)]
  for (uint32_t j = tid; j <= kTreeBlock; j += kTreeThreads)
    s_delta[j] = boundary_delta(codes, n, b0 - 1 + j);
  // the walks' first leaf-box loads wait on DRAM otherwise: start them now
  leaf.prefetch(b0, count);
  for (uint32_t j = tid; j < kTreeBlock; j += kTreeThreads) {
    s_slot[j] = kSlotEmpty;
    *staged_left_at(s_rec, j) = 0.0f; // no record (node 0, the root, is never a child)
  }
  if (tid == 0) {
    s_next = 0;
    s_npend = 0;
  }
  __syncthreads();
  if (sort_failed)
    return;

  local_walks<kTreeBlock>(leaf, n, b0, count, s_delta, s_slot, s_rec, s_pend, &s_next, &s_npend);
  __syncthreads();
  local_write_out<kTreeBlock>(leaf, n, b0, nodes, s_slot, s_rec, s_pend, &s_npend);
  __syncthreads();
  const uint32_t np = s_npend;
  if (walk_on) {
    // The walks above this CTA's pieces start here: each piece walks up
    // through the global arrival slots at once, so chains across CTA edges
    // overlap the local phases of the CTAs still to run. This CTA's records were all
    // written before the barrier above; the fence orders them before the
    // walk's first release.
    if (tid == 0 && np > kTreePendingPerBlock)
      atomicOr(&st->error, kErrBadTopology); // more canonical pieces than a tree can have
    if (tid < min(np, kTreePendingPerBlock)) {
      __threadfence();
      const PendingNode pn = s_pend[tid];
      walk_global(leaf, n, codes, slots, nodes, st, epoch, pn.L, pn.R, pn.box);
    }
    return;
  }
  // the CTA's pieces in leaf order, after its header, for the merge phase
  const uint32_t m = min(np, kTreePendingPerBlock);
  if (tid == 0) {
    if (np > kTreePendingPerBlock)
      atomicOr(&st->error, kErrBadTopology); // more canonical pieces than a tree can have
    hdr_out[blockIdx.x] = PieceHdr{ m, b0, s_delta[0], 0 };
  }
  PieceRec* out = pieces_out + size_t(blockIdx.x) * kMergeOut;
  for (uint32_t k = tid; k < m; k += kTreeThreads) {
    const PendingNode pn = s_pend[k];
    uint32_t rank = 0; // the pieces partition the CTA's range: their first leaves differ
    for (uint32_t j = 0; j < m; j++)
      rank += s_pend[j].L < pn.L;
    store_piece(out + rank, pn.R, s_delta[pn.R - b0 + 1], pn.box);
  }
}

// Merge phase: one CTA per window of `window` consecutive groups of the level
// below. The window's P pieces are numbered in leaf order; boundary k lies
// between pieces k and k + 1, at split position R_k. A node covering pieces
// [a, b] is a left child, with its parent's split at boundary b, when
// delta(R_b) > delta(L_a - 1), else a right child with the split at boundary
// a - 1: the reference's rule over the same deltas, so these are the nodes a
// walk from the leaves finds. An arrival stores its box in its side of the
// boundary's box pair and swaps its far piece index into the boundary's slot
// (block-scope acquire-release exchange on shared memory); the first arrival
// stops, the second reads its sibling's box and far end, marks the slot
// complete with the parent's piece range and climbs on, so each step of a
// chain is a few shared-memory round trips. (No record is stored to global
// memory during a walk: the release half of the next exchange would wait for
// it.) A walk stops at the window's edge (boundary -1 or P - 1). After a
// barrier every complete slot yields its node's record -- the two child boxes
// are still in the pair, joined left then right -- and a slot still holding
// one arrival marks a node whose sibling leaves the window. Those nodes are
// the window's pieces for the next level. The last level is one window over
// everything and ends at the root.
//
// A window with more than `cap` pieces (kMergeCap: ~11 pieces come per
// local-phase CTA, ~15-20 per window, so this is far from reached) sets
// tree_fallback; the later levels see it and return, and the last one walks
// every local-phase piece up through the global epoch-tagged slots instead
// (walk_global at block scope), which holds for any number of pieces.
constexpr uint32_t kMergeDone = 0x80000000u; // slot: both arrived; bits 30-16 / 15-0 the parent's pieces
static_assert(kMergeCap <= 0x7fffu, "piece indices of a complete slot take 15 bits");

struct MergeOut
{
  uint32_t L, R;
  int32_t dR;
  Box box;
};

// Largest g < ng with pre[g] <= i (pre[0] = 0 <= i < pre[ng]): the group of piece i.
__device__ __forceinline__ uint32_t
group_of(const uint32_t* pre, uint32_t ng, uint32_t i)
{
  uint32_t lo = 0, hi = ng;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (pre[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The merge's walks over P pieces numbered in leaf order (first leaf L0,
// delta(L0 - 1) = dL0): s_R / s_d hold each piece's last leaf and the delta
// after it, s_slot starts empty, piece_box(i) gives piece i's box. Nodes whose
// parent's split is on the edge (boundary -1 or P - 1) go to s_out.
template<class PieceBox>
__device__ __forceinline__ void
merge_walks(const PieceBox& piece_box, uint32_t n, uint32_t P, uint32_t L0, int dL0, const uint32_t* s_R,
            const int8_t* s_d, uint32_t* s_slot, Box* s_box, MergeOut* s_out, uint32_t* s_nout,
            BuildState* __restrict__ st)
{
  for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
    Box box = piece_box(i);
    uint32_t a = i, b = i;
    uint32_t L = i == 0 ? L0 : s_R[i - 1] + 1, R = s_R[i];
    int dl = i == 0 ? dL0 : s_d[i - 1], dr = s_d[i];
    for (uint32_t depth = 0;; depth++) {
      if (depth > kMaxTreeDepth + 2) {
        atomicOr(&st->error, kErrBadTopology);
        break;
      }
      const bool is_left = dr > dl; // delta(R) > delta(L - 1)
      if (is_left ? b + 1 >= P : a == 0) { // the parent's split is on the window's edge
        const uint32_t j = atomicAdd(s_nout, 1u);
        if (j < kMergeOut)
          s_out[j] = MergeOut{ L, R, dr, box };
        break;
      }
      const uint32_t k = is_left ? b : a - 1;
      store_box8(s_box + 2 * k + (is_left ? 0 : 1), box);
      // release publishes this box, acquire makes the sibling's visible
      const uint32_t old = arrive_acq_rel_cta(s_slot + k, is_left ? a : b);
      if (old == kSlotEmpty)
        break; // first arrival: the sibling completes the parent
      const Box other = load_box8(s_box + 2 * k + (is_left ? 1 : 0));
      box = is_left ? join(box, other) : join(other, box);
      if (is_left)
        b = old;
      else
        a = old;
      s_slot[k] = kMergeDone | (a << 16) | b; // read only after the barrier below
      L = a == 0 ? L0 : s_R[a - 1] + 1;
      R = s_R[b];
      if (L == 0 && R == n - 1)
        break; // the root
      dl = a == 0 ? dL0 : s_d[a - 1];
      dr = s_d[b];
    }
  }
}

// After the walks and a barrier: the records of the nodes completed by the
// walks, and the single arrivals (nodes whose sibling leaves the window) added
// to s_out.
__device__ __forceinline__ void
merge_write_out(uint32_t n, uint32_t P, uint32_t L0, int dL0, const uint32_t* s_R, const int8_t* s_d,
                const uint32_t* s_slot, const Box* s_box, Node* __restrict__ nodes, MergeOut* s_out, uint32_t* s_nout)
{
  for (uint32_t k = threadIdx.x; k + 1 < P; k += blockDim.x) {
    const uint32_t v = s_slot[k];
    if (v == kSlotEmpty)
      continue;
    if (v & kMergeDone) { // the record of the node completed here
      const uint32_t a = (v >> 16) & 0x7fffu, b = v & 0xffffu, s = s_R[k];
      const uint32_t L = a == 0 ? L0 : s_R[a - 1] + 1, R = s_R[b];
      const uint32_t cl = (L == s) ? (s | kLeafBit) : s;
      const uint32_t cr = (R == s + 1) ? ((s + 1) | kLeafBit) : (s + 1);
      const int dl = a == 0 ? dL0 : s_d[a - 1];
      const uint32_t idx = (L == 0 && R == n - 1) ? 0 : (s_d[b] > dl ? R : L);
      store_node(nodes, idx, join(load_box8(s_box + 2 * k), load_box8(s_box + 2 * k + 1)), cl, cr);
      continue;
    }
    // a single arrival: a node whose sibling range leaves the window
    const bool left = v <= k; // the waiter covers pieces [v, k] (a left child) or [k + 1, v]
    const uint32_t a = left ? v : k + 1, b = left ? k : v;
    const uint32_t j = atomicAdd(s_nout, 1u);
    if (j < kMergeOut)
      s_out[j] = MergeOut{ a == 0 ? L0 : s_R[a - 1] + 1, s_R[b], s_d[b], s_box[2 * k + (left ? 0 : 1)] };
  }
}

template<class Leaf>
__global__ __launch_bounds__(kMergeThreads) void
k_tree_merge(Leaf leaf,
             uint32_t n,
             const uint32_t* __restrict__ codes,
             unsigned long long* __restrict__ slots,
             uint32_t epoch,
             Node* __restrict__ nodes,
             BuildState* __restrict__ st,
             const PieceRec* __restrict__ in,
             const PieceHdr* __restrict__ in_hdr,
             uint32_t groups,
             uint32_t window,
             PieceRec* __restrict__ out,
             PieceHdr* __restrict__ out_hdr,
             const PieceRec* __restrict__ first,
             const PieceHdr* __restrict__ first_hdr,
             uint32_t first_groups,
             uint32_t cap,
             bool last)
{
  pdl_begin(); // the predecessor in the stream has finished
  extern __shared__ __align__(32) unsigned char smem[];
  Box* s_box = reinterpret_cast<Box*>(smem);                                   // 2 x kMergeCap
  uint32_t* s_R = reinterpret_cast<uint32_t*>(s_box + 2 * kMergeCap);          // kMergeCap
  uint32_t* s_slot = s_R + kMergeCap;                                          // kMergeCap
  uint32_t* s_pre = s_slot + kMergeCap;                                        // kMergeMaxGroups + 1
  MergeOut* s_out = reinterpret_cast<MergeOut*>(s_pre + kMergeMaxGroups + 1);  // kMergeOut
  int8_t* s_d = reinterpret_cast<int8_t*>(s_out + kMergeOut);                  // kMergeCap
  __shared__ uint32_t s_nout, s_fallback;

  if (__ldcg(&st->error) & kErrLookbackTimeout)
    return; // the sort gave up: no tree (the error is reported); uniform over the CTA
  const uint32_t tid = threadIdx.x;
  const uint32_t g0 = blockIdx.x * window, ng = min(window, groups - g0);
  if (tid == 0) {
    s_nout = 0;
    s_fallback = __ldcg(&st->tree_fallback); // set by an earlier level only
    s_pre[0] = 0;
  }
  for (uint32_t g = tid; g < ng; g += kMergeThreads)
    s_pre[g + 1] = min(__ldcg(&in_hdr[g0 + g].count), kMergeOut);
  __syncthreads();
  if (tid < 32) { // running sum of the group counts
    uint32_t carry = 0;
    for (uint32_t base = 0; base < ng; base += 32) {
      const uint32_t g = base + tid;
      uint32_t v = g < ng ? s_pre[g + 1] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (int(tid) >= o)
          v += t;
      }
      if (g < ng)
        s_pre[g + 1] = v + carry;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
  }
  __syncthreads();
  const uint32_t P = s_pre[ng];
  const uint32_t L0 = __ldcg(&in_hdr[g0].L0);
  const int dL0 = __ldcg(&in_hdr[g0].dL);

  if (s_fallback || P > cap) { // uniform over the CTA
    if (!last) {
      if (tid == 0)
        atomicExch(&st->tree_fallback, 1u);
      return;
    }
    for (size_t idx = tid; idx < size_t(first_groups) * kMergeOut; idx += kMergeThreads) {
      const uint32_t c = uint32_t(idx / kMergeOut), k = uint32_t(idx % kMergeOut);
      if (k >= min(__ldcg(&first_hdr[c].count), kMergeOut))
        continue;
      const PieceRec* p = first + idx;
      const uint32_t L = k == 0 ? __ldcg(&first_hdr[c].L0) : __ldcg(&p[-1].R) + 1;
      walk_global<Leaf, true>(leaf, n, codes, slots, nodes, st, epoch, L, __ldcg(&p->R), load_piece_box(p));
    }
    return;
  }

  for (uint32_t i = tid; i < P; i += kMergeThreads) {
    const uint32_t g = group_of(s_pre, ng, i);
    const uint2 rd = __ldcg(reinterpret_cast<const uint2*>(in + size_t(g0 + g) * kMergeOut + (i - s_pre[g])));
    s_R[i] = rd.x;
    s_d[i] = int8_t(int(rd.y));
    s_slot[i] = kSlotEmpty;
  }
  __syncthreads();

  merge_walks(
    [&](uint32_t i) {
      const uint32_t g = group_of(s_pre, ng, i);
      return load_piece_box(in + size_t(g0 + g) * kMergeOut + (i - s_pre[g]));
    },
    n, P, L0, dL0, s_R, s_d, s_slot, s_box, s_out, &s_nout, st);
  __syncthreads();
  merge_write_out(n, P, L0, dL0, s_R, s_d, s_slot, s_box, nodes, s_out, &s_nout);
  __syncthreads();
  const uint32_t nout = s_nout;
  if (last) {
    if (tid == 0 && nout != 0)
      atomicOr(&st->error, kErrBadTopology); // the root was not reached
    return;
  }
  const uint32_t m = min(nout, kMergeOut);
  if (tid == 0) {
    if (nout > kMergeOut)
      atomicOr(&st->error, kErrBadTopology); // more canonical pieces than a tree can have
    out_hdr[blockIdx.x] = PieceHdr{ m, L0, dL0, 0 };
  }
  for (uint32_t k = tid; k < m; k += kMergeThreads) {
    const MergeOut o = s_out[k];
    uint32_t rank = 0;
    for (uint32_t j = 0; j < m; j++)
      rank += s_out[j].L < o.L;
    store_piece(out + size_t(blockIdx.x) * kMergeOut + rank, o.R, o.dR, o.box);
  }
}

// ---------------------------------------------------------------------------
// Small keys-only builds in one launch (k_small_build). One thread-block
// cluster of C = ceil(n / 1024) CTAs (C <= 16); CTA r holds primitives and
// leaf slots [1024 r, 1024 r + 1024) -- in parity mode leaf slot p is
// primitive p, so a CTA's leaf boxes are the boxes it computes. Every phase
// is the multi-kernel build's arithmetic, in shared memory:
//   1. the leaf boxes and the centroid bounds with the index tie rule
//      (k_bounds); the CTAs' partial bounds are combined through distributed
//      shared memory;
//   2. the Morton codes (k_morton);
//   3. a sort over the cluster: each CTA sorts its codes with a bitonic
//      network and tabulates where each value of the codes' top 10 bits
//      starts in its sorted run; a code's global position is its rank in its
//      own run plus, for every other CTA, the start of its bucket there and a
//      binary search inside that bucket (ties go to the lower CTA, so every
//      position is taken once); each code is stored into the shared memory
//      of the CTA that owns its position;
//   4. the local tree phase over the CTA's 1,024 slots (local_walks), with the
//      neighbours' edge codes read remotely, its pieces kept in shared memory;
//   5. CTA 0 gathers every CTA's pieces and merges them to the root
//      (merge_walks), as the last merge level does.
// A cluster barrier separates the phases that read other CTAs' shared memory.
namespace cg = cooperative_groups;

struct SmemLeaf
{
  const Box* boxes;
  uint32_t b0;
  __device__ __forceinline__ Box operator()(uint32_t i) const { return load_box8(boxes + (i - b0)); }
};

template<class Leaf>
__global__ __launch_bounds__(kSmallThreads, 1) void
k_small_build(Leaf leaf, uint32_t n, uint32_t* __restrict__ codes_out, Node* __restrict__ nodes,
              BuildState* __restrict__ st)
{
  pdl_begin(); // the predecessor in the stream has finished
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(32) unsigned char smem[];
  Box* s_box = reinterpret_cast<Box*>(smem + kSmBox);
  uint32_t* s_key = reinterpret_cast<uint32_t*>(smem + kSmKey);
  __shared__ uint16_t s_tab[1025]; // the CTA's sorted run by bucket (step 3)
  PieceRec* s_piece = reinterpret_cast<PieceRec*>(smem + kSmPiece);
  unsigned char* u = smem + kSmUnion;
  __shared__ ArgBox s_part[kSmallThreads / 32];
  __shared__ ArgBox s_cpart;
  __shared__ float s_lo[3], s_scale[3];
  __shared__ uint32_t s_next, s_npend, s_npieces, s_nout;
  __shared__ uint32_t s_pre[kSmallMaxCtas + 1];

  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t r = blockIdx.x, C = gridDim.x; // the grid is one cluster
  const uint32_t b0 = r * kSmallSlots, cnt = min(kSmallSlots, n - b0);
  const bool valid = tid < cnt;

  // ---- 1. leaf boxes and centroid bounds (k_bounds) ----
  ArgBox a = empty_arg();
  Box bx{};
  if (valid) {
    const uint32_t i = b0 + tid;
    bx = leaf(i);
    store_box8(s_box + tid, bx);
    const float c[3] = { fmul(fadd(bx.lo[0], bx.hi[0]), 0.5f), fmul(fadd(bx.lo[1], bx.hi[1]), 0.5f),
                         fmul(fadd(bx.lo[2], bx.hi[2]), 0.5f) };
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
  if (tid == 0)
    s_cpart = a;
  cluster.sync();
  if (warp == 0) { // lane q takes CTA q's partial; the combine is order-free
    ArgBox t = lane < C ? *cluster.map_shared_rank(&s_cpart, lane) : empty_arg();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ArgBox o2;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        o2.v[k] = __shfl_down_sync(0xffffffffu, t.v[k], o);
        o2.i[k] = __shfl_down_sync(0xffffffffu, t.i[k], o);
      }
      combine(t, o2);
    }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        s_lo[k] = t.v[k];
        s_scale[k] = fdiv(1024.0f, fadd(fsub(t.v[k + 3], t.v[k]), 1.0f)); // lbvh.h:1437-1441
      }
  }
  __syncthreads();

  // ---- 2. Morton codes (k_morton) ----
  uint32_t* key_cur = s_key;
  uint32_t* key_nxt = s_key + kSmallSlots;
  if (valid)
    key_cur[tid] = morton_of(bx, s_lo[0], s_lo[1], s_lo[2], s_scale[0], s_scale[1], s_scale[2]);

  // ---- 3. the sort: each CTA sorts its codes, then every code finds its
  //      position among all CTAs' sorted runs ----
  // 3a. bitonic sort of the CTA's codes (only the codes are kept, so equal
  //     codes are interchangeable; exchanges of distance >= 32 through
  //     shared memory, two buffers; the rest by shuffles); past-the-end
  //     lanes carry ~0, above every 30-bit code, and sort last
  uint32_t* s_bit = reinterpret_cast<uint32_t*>(u); // [2][kSmallSlots]
  {
    uint32_t v = valid ? key_cur[tid] : ~0u;
    int buf = 0;
    for (uint32_t k = 2; k <= kSmallSlots; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        uint32_t o;
        if (j >= 32) {
          s_bit[buf * kSmallSlots + tid] = v;
          __syncthreads();
          o = s_bit[buf * kSmallSlots + (tid ^ j)];
          buf ^= 1;
        } else {
          o = __shfl_xor_sync(0xffffffffu, v, j);
        }
        const bool keep_min = ((tid & j) == 0) == ((tid & k) == 0);
        v = keep_min ? min(o, v) : max(o, v);
      }
    if (valid)
      key_nxt[tid] = v; // the CTA's run, in order
  }
  __syncthreads();
  // 3b. the run's bucket table: s_tab[t] = the run's codes below bucket t
  //     (t = the top 10 code bits), for t = 0..1024
  for (uint32_t t = tid; t <= 1024; t += kSmallThreads) {
    uint32_t lo = 0, hi = cnt; // first run index whose bucket is >= t
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if ((key_nxt[mid] >> 20) < t)
        lo = mid + 1;
      else
        hi = mid;
    }
    s_tab[t] = uint16_t(lo);
  }
  cluster.sync(); // every CTA's run and table are complete
  // 3c. a code's position: its rank in its own run plus, in each other run,
  //     the codes before it -- below its bucket from the table, then inside
  //     the bucket by binary search: codes <= its own in runs of lower index,
  //     codes < its own in later runs (equal codes thus take distinct places)
  if (valid) {
    const uint32_t code = key_nxt[tid];
    const uint32_t t = code >> 20;
    uint32_t pos = tid;
#pragma unroll
    for (uint32_t q = 0; q < kSmallMaxCtas; q++) {
      if (q >= C || q == r)
        continue;
      const uint16_t* tab = cluster.map_shared_rank(s_tab, q);
      const uint32_t* run = cluster.map_shared_rank(key_nxt, q);
      uint32_t lo = tab[t], hi = tab[t + 1];
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t c = run[mid];
        if (q < r ? c <= code : c < code)
          lo = mid + 1;
        else
          hi = mid;
      }
      pos += lo;
    }
    if (pos < n)
      cluster.map_shared_rank(key_cur, pos / kSmallSlots)[pos % kSmallSlots] = code;
    else
      atomicOr(&st->error, kErrBadTopology); // < n by construction
  }
  cluster.sync(); // every code has landed; every run and table has been read

  // ---- 4. local tree phase over the CTA's slots ----
  int* s_delta = reinterpret_cast<int*>(u);
  uint32_t* s_slot = reinterpret_cast<uint32_t*>(u + kSmTreeSlot);
  Node* s_rec = reinterpret_cast<Node*>(u + kSmTreeRec);
  PendingNode* s_pend = reinterpret_cast<PendingNode*>(u + kSmTreePend);
  {
    // boundary b0 - 1 + tid, and (thread 0) b0 + 1023; codes beyond the CTA
    // are the neighbours' edge codes
    const auto code_at = [&](uint32_t k) -> uint32_t {
      if (k < b0)
        return *cluster.map_shared_rank(key_cur + (kSmallSlots - 1), r - 1);
      if (k >= b0 + kSmallSlots)
        return *cluster.map_shared_rank(key_cur, r + 1);
      return key_cur[k - b0];
    };
    for (uint32_t j = tid; j <= kSmallSlots; j += kSmallThreads) {
      const uint32_t k = b0 - 1 + j;
      int dv = -1; // k = L - 1 wraps for L = 0; k >= n - 1 is past the end
      if (k < n - 1) {
        const uint32_t x = code_at(k), y = code_at(k + 1);
        dv = x == y ? int(__clz(k ^ (k + 1))) + 32 : int(__clz(x ^ y));
      }
      s_delta[j] = dv;
    }
    s_slot[tid] = kSlotEmpty;
    *staged_left_at(s_rec, tid) = 0.0f; // no record (node 0, the root, is never a child)
    if (tid == 0) {
      s_next = 0;
      s_npend = 0;
    }
  }
  __syncthreads();
  const SmemLeaf sl{ s_box, b0 };
  local_walks<kSmallSlots>(sl, n, b0, cnt, s_delta, s_slot, s_rec, s_pend, &s_next, &s_npend);
  __syncthreads();
  local_write_out<kSmallSlots>(sl, n, b0, nodes, s_slot, s_rec, s_pend, &s_npend);
  __syncthreads();
  {
    const uint32_t np = s_npend, m = min(np, kMergeOut);
    if (tid == 0) {
      if (np > kMergeOut)
        atomicOr(&st->error, kErrBadTopology); // more canonical pieces than a tree can have
      s_npieces = m;
    }
    for (uint32_t k = tid; k < m; k += kSmallThreads) {
      const PendingNode pn = s_pend[k];
      uint32_t rank = 0; // the pieces partition the CTA's slots: their first leaves differ
      for (uint32_t j = 0; j < m; j++)
        rank += s_pend[j].L < pn.L;
      store_piece(s_piece + rank, pn.R, s_delta[pn.R - b0 + 1], pn.box);
    }
  }
  cluster.sync(); // every CTA's pieces are complete

  // ---- 5. CTA 0 gathers the pieces and merges them to the root ----
  Box* m_box = reinterpret_cast<Box*>(u);
  uint32_t* m_R = reinterpret_cast<uint32_t*>(u + kSmMergeR);
  uint32_t* m_slot = reinterpret_cast<uint32_t*>(u + kSmMergeSlot);
  int8_t* m_d = reinterpret_cast<int8_t*>(u + kSmMergeD);
  MergeOut* m_out = reinterpret_cast<MergeOut*>(u + kSmMergeOut);
  const bool merging = r == 0 && C > 1;
  if (merging) { // this CTA's tree scratch is dead: its write-out ended before the barrier
    if (warp == 0) { // lane q reads CTA q's piece count; a running sum gives the starts
      uint32_t v = lane < C ? *cluster.map_shared_rank(&s_npieces, lane) : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= uint32_t(o))
          v += y;
      }
      if (lane < C)
        s_pre[lane + 1] = v;
      if (lane == 0) {
        s_pre[0] = 0;
        s_nout = 0;
      }
    }
    __syncthreads();
    const uint32_t P = s_pre[C];
    for (uint32_t i = tid; i < P; i += kSmallThreads) {
      const uint32_t q = group_of(s_pre, C, i);
      const PieceRec* pr = cluster.map_shared_rank(s_piece, q) + (i - s_pre[q]);
      const float4 pa = reinterpret_cast<const float4*>(pr)[0], pb = reinterpret_cast<const float4*>(pr)[1];
      m_R[i] = __float_as_uint(pa.x);
      m_d[i] = int8_t(__float_as_int(pa.y));
      m_slot[i] = kSlotEmpty;
      // piece i's box: only a node containing piece i writes there later
      store_box8(m_box + 2 * i, Box{ { pa.z, pa.w, pb.x }, { pb.y, pb.z, pb.w } });
    }
  }
  cluster.sync(); // CTA 0 has read every CTA's pieces: the others may exit
  if (valid) // the sorted codes, for refits (stored last: no store is in flight during the walks)
    codes_out[b0 + tid] = key_cur[tid];
  if (!merging)
    return;
  const uint32_t P = s_pre[C];
  merge_walks([&](uint32_t i) { return load_box8(m_box + 2 * i); }, n, P, 0u, -1, m_R, m_d, m_slot, m_box, m_out, &s_nout,
              st);
  __syncthreads();
  merge_write_out(n, P, 0u, -1, m_R, m_d, m_slot, m_box, nodes, m_out, &s_nout);
  __syncthreads();
  if (tid == 0 && s_nout != 0)
    atomicOr(&st->error, kErrBadTopology); // the root was not reached
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

// Validation of a node array from outside this library (the check_bvh
// invariants of lbvh_test.cpp:369-446): every child index in range, the root
// unreferenced, every other internal node and every leaf referenced exactly
// once. Such an array is a tree below the root, so a traversal from the root
// visits each node at most once.
__global__ void
k_count_refs(const Node* __restrict__ nodes,
             uint32_t n_nodes,
             uint32_t* __restrict__ node_refs,
             uint32_t* __restrict__ leaf_refs,
             BuildState* __restrict__ st)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes)
    return;
  const uint4 lr = *reinterpret_cast<const uint4*>(&nodes[i].hi[1]);
  const uint32_t c[2] = { lr.z, lr.w };
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const uint32_t x = c[k] & ~kLeafBit;
    if (c[k] & kLeafBit) {
      if (x > n_nodes)
        atomicOr(&st->error, kErrBadTopology);
      else
        atomicAdd(leaf_refs + x, 1u);
    } else {
      if (x >= n_nodes)
        atomicOr(&st->error, kErrBadTopology);
      else
        atomicAdd(node_refs + x, 1u);
    }
  }
}

__global__ void
k_check_refs(uint32_t n_nodes, const uint32_t* __restrict__ node_refs, const uint32_t* __restrict__ leaf_refs,
             BuildState* __restrict__ st)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_nodes && node_refs[i] != (i == 0 ? 0u : 1u))
    atomicOr(&st->error, kErrBadTopology);
  if (i <= n_nodes && leaf_refs[i] != 1u)
    atomicOr(&st->error, kErrBadTopology);
}

// Refit: the box fit alone over a given topology (child and parent links),
// with the same arrival slots as k_build_tree. Equal to the reference's
// fit_boxes over the existing nodes.
template<class Leaf>
__global__ __launch_bounds__(kFitThreads) void
k_refit(Leaf leaf,
        uint32_t n,
        const uint2* __restrict__ child,
        const uint32_t* __restrict__ leaf_parent,
        const uint32_t* __restrict__ node_parent,
        unsigned long long* __restrict__ slots,
        Node* __restrict__ nodes,
        BuildState* __restrict__ st,
        uint32_t epoch)
{
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n)
    return;
  Box box = leaf(p);
  uint32_t self = p | kLeafBit;
  uint32_t q = __ldg(leaf_parent + p);
  const unsigned long long tag = (unsigned long long)epoch << 32;
  for (uint32_t depth = 0;; depth++) {
    if (q >= n - 1 || depth > 2 * kMaxTreeDepth) {
      atomicOr(&st->error, kErrBadTopology);
      return;
    }
    // release: this thread's last record is published; acquire: the
    // sibling's record, published by its own arrival, is visible below
    const unsigned long long old = arrive_acq_rel(slots + q, tag);
    if (uint32_t(old >> 32) != epoch)
      return;
    const uint2 lr = __ldg(child + q);
    const uint32_t lx = lr.x & ~kLeafBit, ly = lr.y & ~kLeafBit;
    if (((lr.x & kLeafBit) ? lx >= n : lx >= n - 1) || ((lr.y & kLeafBit) ? ly >= n : ly >= n - 1)) {
      atomicOr(&st->error, kErrBadTopology);
      return;
    }
    const uint32_t sib = (lr.x == self) ? lr.y : lr.x;
    Box other;
    if (sib & kLeafBit)
      other = leaf(sib & ~kLeafBit);
    else
      other = load_node_box(nodes, sib);
    box = (lr.x == self) ? join(box, other) : join(other, box);
    store_node(nodes, q, box, lr.x, lr.y);
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
  pdl_begin(); // the predecessor in the stream has finished
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint32_t p = __ldg(perm + i);
  out[i] = tris[p < n ? p : 0]; // p >= n only after a sort that gave up (error reported)
}

__global__ void
k_gather_boxes(const Box* __restrict__ boxes,
               const uint32_t* __restrict__ perm,
               uint32_t n,
               Box* __restrict__ out)
{
  pdl_begin(); // the predecessor in the stream has finished
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint32_t p = __ldg(perm + i);
  out[i] = boxes[p < n ? p : 0]; // p >= n only after a sort that gave up (error reported)
}

// ---------------------------------------------------------------------------
// host-side launchers

#define CUDA_TRY(call)                                                                                                 \
  do {                                                                                                                 \
    const cudaError_t e_ = (call);                                                                                     \
    if (e_ != cudaSuccess)                                                                                             \
      return e_;                                                                                                       \
  } while (0)

template<class Leaf>
static cudaError_t
launch_curve(const Leaf& leaf, uint32_t n, const BuildBuffers& b, cudaStream_t s, Box* stage)
{
  CUDA_TRY(launch_pdl(k_bounds<Leaf>, b.bounds_blocks, kBoundsThreads, 0, s, leaf, n,
                      reinterpret_cast<ArgBox*>(b.partials), b.state, stage));
  if (stage) {
    if (b.msd)
      CUDA_TRY(launch_pdl(k_morton<BoxLeaf, true>, b.msd_ranges, kMortonThreads, 0, s, BoxLeaf{ stage }, n, b.keys_a,
                          b.state, b.msd_range, b.top_rows));
    else
      CUDA_TRY(launch_pdl(k_morton<BoxLeaf, false>, b.morton_blocks, kMortonThreads, 0, s, BoxLeaf{ stage }, n,
                          b.keys_a, b.state, 0, nullptr));
  } else {
    if (b.msd)
      CUDA_TRY(launch_pdl(k_morton<Leaf, true>, b.msd_ranges, kMortonThreads, 0, s, leaf, n, b.keys_a, b.state,
                          b.msd_range, b.top_rows));
    else
      CUDA_TRY(launch_pdl(k_morton<Leaf, false>, b.morton_blocks, kMortonThreads, 0, s, leaf, n, b.keys_a, b.state, 0,
                          nullptr));
  }
  return cudaGetLastError();
}

cudaError_t
launch_sort(uint32_t n, bool pairs, uint32_t epoch_base, const BuildBuffers& b, cudaStream_t s, uint32_t passes)
{
  const bool msd = b.msd && !pairs;
  if (msd) {
    static std::atomic<uint64_t> configured{ 0 }; // the shared-memory opt-in, once per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
      return e;
    const uint64_t bit = 1ull << (dev & 63);
    if (!(configured.load(std::memory_order_relaxed) & bit)) {
      e = cudaFuncSetAttribute(k_bucket_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBucketSmem));
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_partition, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kPartSmem));
      if (e != cudaSuccess)
        return e;
      configured.fetch_or(bit, std::memory_order_relaxed);
    }
    // the bucket sort (keys_a -> keys_b -> keys_a), or nothing if a bucket is too large
    CUDA_TRY(launch_pdl(k_top_scan, kTopBuckets / 32, 1024, 0, s, b.top_rows, b.msd_ranges, b.state));
    const uint32_t ctas = ceil_div_u32(b.msd_ranges, b.msd_group);
    CUDA_TRY(launch_pdl(k_partition, ctas, kPartThreads, kPartSmem, s, b.keys_a, b.keys_b, n, b.msd_range * b.msd_group,
                        b.msd_group, b.top_rows, b.state));
    CUDA_TRY(launch_pdl(k_bucket_sort, b.sort_ctas, kBucketThreads, kBucketSmem, s, b.keys_b, b.keys_a, b.state));
  }
  // the onesweep passes (they return at once when the bucket sort ran);
  // small keys-only sorts use smaller tiles, so that more SMs take part
  const bool small = !pairs && (b.tile_keys ? b.tile_keys == uint32_t(kSmallTile) : n <= kSmallTileMaxPrims);
  const uint32_t tiles = ceil_div_u32(n, small ? kSmallTile : kSortTile);
  uint32_t* ka = b.keys_a;
  uint32_t* kb = b.keys_b;
  uint32_t* va = b.vals_a;
  uint32_t* vb = b.vals_b;
  const uint32_t spin = b.spin_limit ? b.spin_limit : kSpinLimit;
  const uint32_t wx = b.wait_xor;
  // after a bucket sort the passes only run when it gave up: one wave of CTAs
  // looping over the tiles instead of one CTA per tile
  const uint32_t grid = (msd && b.sort_ctas && tiles > 4 * b.sort_ctas) ? 4 * b.sort_ctas : tiles;
  for (uint32_t pass = 0; pass < passes; pass++) {
    const uint32_t epoch = epoch_base + pass;
    if (pairs) {
      if (pass == 0)
        CUDA_TRY(launch_pdl(k_onesweep<true, true>, tiles, kSortThreads, 0, s, ka, kb, nullptr, vb, n, pass, epoch,
                            b.lookback, b.state, false, spin, wx, tiles));
      else
        CUDA_TRY(launch_pdl(k_onesweep<true, false>, tiles, kSortThreads, 0, s, ka, kb, va, vb, n, pass, epoch,
                            b.lookback, b.state, false, spin, wx, tiles));
    } else if (small) {
      CUDA_TRY(launch_pdl(k_onesweep<false, false, kSmallTileItems>, grid, kSortThreads, 0, s, ka, kb, nullptr,
                          nullptr, n, pass, epoch, b.lookback, b.state, msd, spin, wx, tiles));
    } else {
      CUDA_TRY(launch_pdl(k_onesweep<false, false>, grid, kSortThreads, 0, s, ka, kb, nullptr, nullptr, n, pass, epoch,
                          b.lookback, b.state, msd, spin, wx, tiles));
    }
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  // an even pass count leaves the sorted keys (and values) in keys_a / vals_a
  return cudaGetLastError();
}

template<class Leaf>
static cudaError_t
launch_topology_and_fit(const Leaf& leaf, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  // the shared-memory opt-in is per device; set it once on each
  static std::atomic<uint64_t> configured{ 0 };
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return e;
  const uint64_t bit = 1ull << (dev & 63);
  if (!(configured.load(std::memory_order_relaxed) & bit)) {
    e = cudaFuncSetAttribute(k_tree_local<Leaf>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTreeSmem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tree_merge<Leaf>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kMergeSmem));
    if (e != cudaSuccess)
      return e;
    configured.fetch_or(bit, std::memory_order_relaxed);
  }
  const uint32_t blocks = ceil_div_u32(n, kTreeBlock);
  const TreeScratch ts = tree_scratch(n);
  char* pend = static_cast<char*>(b.pending);
  auto pieces = [&](uint32_t lv) { return reinterpret_cast<PieceRec*>(pend + ts.pieces[lv]); };
  auto hdrs = [&](uint32_t lv) { return reinterpret_cast<PieceHdr*>(pend + ts.hdrs[lv]); };
  // trees beyond the fused-walk threshold walk their CTA edges from the local
  // phase's tail when the context asks; all others merge the local pieces
  const bool walk_on = blocks > 1 && n > kTreeGlobalCtaMaxPrims && b.walk_fused == 1;
  CUDA_TRY(launch_pdl(k_tree_local<Leaf>, blocks, kTreeThreads, kTreeSmem, s, leaf, n, b.keys_a, nodes, pieces(0),
                      hdrs(0), b.state, b.slots, epoch, walk_on));
  if (blocks == 1 || walk_on)
    return cudaGetLastError(); // the whole tree was built in the one CTA, or by the walks
  const uint32_t cap = (b.merge_cap && b.merge_cap < kMergeCap) ? b.merge_cap : kMergeCap;
  for (uint32_t lv = 0; lv < ts.merges; lv++) {
    const bool last = lv + 1 == ts.merges;
    CUDA_TRY(launch_pdl(k_tree_merge<Leaf>, ceil_div_u32(ts.groups[lv], ts.window[lv]), kMergeThreads, kMergeSmem, s,
                        leaf, n, b.keys_a, b.slots, epoch, nodes, b.state, pieces(lv), hdrs(lv), ts.groups[lv],
                        ts.window[lv], pieces(lv + 1), hdrs(lv + 1), pieces(0), hdrs(0), ts.groups[0], cap, last));
  }
  return cudaGetLastError();
}

template<class Leaf>
static cudaError_t
launch_small(const Leaf& leaf, uint32_t n, uint32_t* codes_out, Node* nodes, BuildState* st, cudaStream_t s)
{
  const uint32_t C = ceil_div_u32(n, kSmallSlots);
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kSmallThreads);
  cfg.dynamicSmemBytes = kSmallSmem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_small_build<Leaf>, leaf, n, codes_out, nodes, st);
}

// Per device: the shared-memory and cluster-size opt-ins of both
// instantiations, then the largest cluster (16, else 8 CTAs) the device can
// schedule with this much shared memory per CTA.
uint32_t
small_build_limit()
{
  static std::atomic<uint32_t> limit[64];
  static std::atomic<uint64_t> known{ 0 };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 0;
  }
  const uint64_t bit = 1ull << dev;
  if (known.load(std::memory_order_acquire) & bit)
    return limit[dev].load(std::memory_order_relaxed);
  uint32_t best = 0;
  auto setup = [](auto kernel) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmallSmem)) == cudaSuccess &&
           cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  };
  if (setup(k_small_build<TriLeaf>) && setup(k_small_build<BoxLeaf>)) {
    for (uint32_t c : { kSmallMaxCtas, 8u }) {
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = c;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kSmallThreads);
      cfg.dynamicSmemBytes = kSmallSmem;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int tri = 0, box = 0;
      if (cudaOccupancyMaxActiveClusters(&tri, k_small_build<TriLeaf>, &cfg) == cudaSuccess &&
          cudaOccupancyMaxActiveClusters(&box, k_small_build<BoxLeaf>, &cfg) == cudaSuccess && tri > 0 && box > 0) {
        best = c * kSmallSlots;
        break;
      }
    }
  }
  cudaGetLastError(); // a refused opt-in or query only disables this path
  limit[dev].store(best, std::memory_order_relaxed);
  known.fetch_or(bit, std::memory_order_release);
  return best;
}

cudaError_t
launch_small_build_tris(const Tri* tris, uint32_t n, uint32_t* codes_out, Node* nodes, BuildState* st, cudaStream_t s)
{
  return launch_small(TriLeaf{ tris }, n, codes_out, nodes, st, s);
}

cudaError_t
launch_small_build_boxes(const Box* boxes, uint32_t n, uint32_t* codes_out, Node* nodes, BuildState* st,
                         cudaStream_t s)
{
  return launch_small(BoxLeaf{ boxes }, n, codes_out, nodes, st, s);
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
  return launch_curve(TriLeaf{ tris }, n, b, s, b.boxes);
}

cudaError_t
launch_curve_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, cudaStream_t s)
{
  return launch_curve(BoxLeaf{ boxes }, n, b, s, nullptr);
}

cudaError_t
launch_fit_staged(uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  return launch_topology_and_fit(BoxLeaf{ b.boxes }, n, b, nodes, epoch, s);
}

cudaError_t
launch_fit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  return launch_topology_and_fit(TriLeaf{ tris }, n, b, nodes, epoch, s);
}

cudaError_t
launch_fit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  return launch_topology_and_fit(BoxLeaf{ boxes }, n, b, nodes, epoch, s);
}

cudaError_t
launch_gather_tris(const Tri* tris, const uint32_t* perm, uint32_t n, Tri* out, cudaStream_t s)
{
  CUDA_TRY(launch_pdl(k_gather_tris, ceil_div_u32(n, 256), 256, 0, s, tris, perm, n, out));
  return cudaGetLastError();
}

cudaError_t
launch_gather_boxes(const Box* boxes, const uint32_t* perm, uint32_t n, Box* out, cudaStream_t s)
{
  CUDA_TRY(launch_pdl(k_gather_boxes, ceil_div_u32(n, 256), 256, 0, s, boxes, perm, n, out));
  return cudaGetLastError();
}

template<class Leaf>
static cudaError_t
launch_refit(const Leaf& leaf, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  k_links_from_nodes<<<ceil_div_u32(n - 1, 256), 256, 0, s>>>(nodes, n - 1, b.child, b.leaf_parent, b.node_parent);
  k_refit<Leaf><<<ceil_div_u32(n, kFitThreads), kFitThreads, 0, s>>>(
    leaf, n, b.child, b.leaf_parent, b.node_parent, b.slots, nodes, b.state, epoch);
  return cudaGetLastError();
}

cudaError_t
launch_validate(const Node* nodes, uint32_t n_nodes, const BuildBuffers& b, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(b.node_parent, 0, 4 * size_t(n_nodes), s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(b.leaf_parent, 0, 4 * (size_t(n_nodes) + 1), s);
  if (e != cudaSuccess)
    return e;
  k_count_refs<<<ceil_div_u32(n_nodes, 256), 256, 0, s>>>(nodes, n_nodes, b.node_parent, b.leaf_parent, b.state);
  k_check_refs<<<ceil_div_u32(n_nodes + 1, 256), 256, 0, s>>>(n_nodes, b.node_parent, b.leaf_parent, b.state);
  return cudaGetLastError();
}

cudaError_t
launch_refit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  return launch_refit(TriLeaf{ tris }, n, b, nodes, epoch, s);
}

cudaError_t
launch_refit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s)
{
  return launch_refit(BoxLeaf{ boxes }, n, b, nodes, epoch, s);
}

} // namespace lbvh_gb300
