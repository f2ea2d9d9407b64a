// Closest-hit ray/triangle traversal for sm_103a.
//
// Replaces traverser<float, triangle<float>, triangle_intersection<float>>::
// operator() with triangle_intersector<float> (lbvh.h:1869-1942, 2055-2075)
// with the reference's exact visiting order, per ray:
//   * a 128-entry stack of {node, tmin} that drops pushes when full
//     (lbvh.h:1746-1789), seeded with {root, +inf};
//   * pop; skip if closest.t < entry.tmin;
//   * leaf children are intersected when their parent is popped, left first;
//     internal children are box-tested (octant form, lbvh.h:1071-1091);
//   * both hit: push the farther first (equal tmin: right popped first).
// All arithmetic uses explicit round-to-nearest ops, so hits (id, t, u, v)
// are bit-identical to the reference.
//
// GB300 mapping:
//   * a traversal copy of the tree in which each internal node carries both
//     children's boxes (64 bytes, two 32-byte loads from one line), built
//     once per build by k_repack;
//   * persistent warps: a lane whose ray has finished takes the next ray of
//     its warp's batch (ballot + shuffle), and a warp fetches a new batch of
//     32 rays with one atomic, so lanes do not idle while the longest ray of
//     a fixed group finishes.
#include "batch.cuh"
#include "trace.cuh"

namespace lbvh_gb300 {

struct RayCtx
{
  float px, py, pz, dx, dy, dz, tmin, tmax;
  float2 rxy, ixy;    // reciprocal direction and (-pos) * rcp, x and y
  float2 rzz, izz;    // the same for z, twice (paired slab math, see box_pair_fast)
  bool sx, sy, sz;    // dir > 0: near plane is the box minimum
  bool fast;          // no slab value can be NaN: min/max may use fminf/fmaxf
};

// 1 / x correctly rounded. IEEE 754 gives a correctly rounded reciprocal
// and a correctly rounded division of 1 by x the same bits, so this is the
// reference's `1 / x` (measured: the same speed as __fdiv_rn(1, x) here).
__device__ __forceinline__ float
rcp_rn(float x)
{
  return __frcp_rn(x);
}

// Packed IEEE single-precision add on a pair (elementwise, round to
// nearest): each half is exactly what __fadd_rn gives. Only the add is
// packed. The products feeding it are scalar __fmul_rn: the assembler may
// contract a packed multiply that feeds a packed add into one fused
// multiply-add (measured on sm_103a, despite .rn), which would round
// b * rcp + inv_pos once instead of twice and change grazing hits.
__device__ __forceinline__ float2
add2_rn(float2 a, float2 b)
{
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
      "mov.b64 pa, {%2, %3};\n\t"
      "mov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pd, pa, pb;\n\t"
      "mov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// Three-input max / min of finite values.
__device__ __forceinline__ float
max3f(float a, float b, float c)
{
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float
min3f(float a, float b, float c)
{
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ RayCtx
make_ray(const float4 a, const float4 b)
{
  RayCtx r;
  r.px = a.x;
  r.py = a.y;
  r.pz = a.z;
  r.dx = a.w;
  r.dy = b.x;
  r.dz = b.y;
  r.tmin = b.z;
  r.tmax = b.w;
  // make_accel_ray, lbvh.h:991-1010
  const float rx = rcp_rn(r.dx), ry = rcp_rn(r.dy), rz = rcp_rn(r.dz);
  const float ix = fmul(-r.px, rx), iy = fmul(-r.py, ry), iz = fmul(-r.pz, rz);
  r.rxy = make_float2(rx, ry);
  r.ixy = make_float2(ix, iy);
  r.rzz = make_float2(rz, rz);
  r.izz = make_float2(iz, iz);
  r.sx = r.dx > 0.0f;
  r.sy = r.dy > 0.0f;
  r.sz = r.dz > 0.0f;
  // |dir| >= 2^-60 and |pos| <= 2^60 (false for NaN), with every box
  // coordinate within 2^60 (checked by k_repack), bound |b * rcp| and
  // |pos * rcp| by 2^120: every slab value is finite.
  const float lo = 0x1p-60f, hi = 0x1p60f;
  r.fast = fabsf(r.dx) >= lo && fabsf(r.dy) >= lo && fabsf(r.dz) >= lo && fabsf(r.px) <= hi &&
           fabsf(r.py) <= hi && fabsf(r.pz) <= hi;
  return r;
}

// detail::intersect (octant form) + box_intersection::operator bool,
// lbvh.h:1026-1029, 1071-1091, with the reference's NaN-propagating
// min / max ternaries.
__device__ __forceinline__ bool
box_test(const RayCtx& r, float lox, float loy, float loz, float hix, float hiy, float hiz, float& tmin_out)
{
  const float tn0 = fadd(fmul(r.sx ? lox : hix, r.rxy.x), r.ixy.x);
  const float tn1 = fadd(fmul(r.sy ? loy : hiy, r.rxy.y), r.ixy.y);
  const float tn2 = fadd(fmul(r.sz ? loz : hiz, r.rzz.x), r.izz.x);
  const float tf0 = fadd(fmul(r.sx ? hix : lox, r.rxy.x), r.ixy.x);
  const float tf1 = fadd(fmul(r.sy ? hiy : loy, r.rxy.y), r.ixy.y);
  const float tf2 = fadd(fmul(r.sz ? hiz : loz, r.rzz.x), r.izz.x);
  const float tmin = mmax(mmax(tn0, tn1), tn2);
  const float tmax = mmin(mmin(tf0, tf1), tf2);
  tmin_out = tmin;
  return tmax >= mmax(0.0f, tmin);
}

// The same test for both children of a traversal node at once, for a ray
// and scene whose slab values are all finite (RayCtx::fast): left box
// lo = (A.x, A.y, A.z), hi = (A.w, B.x, B.y); right box lo = (B.z, B.w, C.x),
// hi = (C.y, C.z, C.w). Each slab value is b * rcp + inv_pos rounded twice,
// as in the reference, the adds two at a time: the x and y planes of one
// box as a pair, the z planes of the two boxes as a pair. On finite operands the
// three-input max / min pick the value the reference's ternaries pick, up to
// the sign of a zero, and every later use of tmin / tmax is a comparison,
// which ignores that sign.
__device__ __forceinline__ float2
mul_pair(float a, float b, float2 m)
{
  return make_float2(fmul(a, m.x), fmul(b, m.y));
}

__device__ __forceinline__ void
box_pair_fast(const RayCtx& r, const float4& A, const float4& B, const float4& C, bool& lhit, bool& rhit, float& lt,
              float& rt)
{
  const float2 ln = add2_rn(mul_pair(r.sx ? A.x : A.w, r.sy ? A.y : B.x, r.rxy), r.ixy);
  const float2 lf = add2_rn(mul_pair(r.sx ? A.w : A.x, r.sy ? B.x : A.y, r.rxy), r.ixy);
  const float2 rn = add2_rn(mul_pair(r.sx ? B.z : C.y, r.sy ? B.w : C.z, r.rxy), r.ixy);
  const float2 rf = add2_rn(mul_pair(r.sx ? C.y : B.z, r.sy ? C.z : B.w, r.rxy), r.ixy);
  const float2 zn = add2_rn(mul_pair(r.sz ? A.z : B.y, r.sz ? C.x : C.w, r.rzz), r.izz);
  const float2 zf = add2_rn(mul_pair(r.sz ? B.y : A.z, r.sz ? C.w : C.x, r.rzz), r.izz);
  lt = max3f(ln.x, ln.y, zn.x);
  rt = max3f(rn.x, rn.y, zn.y);
  lhit = min3f(lf.x, lf.y, zf.x) >= fmaxf(0.0f, lt);
  rhit = min3f(rf.x, rf.y, zf.y) >= fmaxf(0.0f, rt);
}

// triangle_intersector::operator(), lbvh.h:2055-2075.
__device__ __forceinline__ bool
tri_test(const RayCtx& r, const Tri* __restrict__ tris, uint32_t p, float& t, float& u, float& v)
{
  const float4* q = reinterpret_cast<const float4*>(tris + p);
  const float4 A = __ldg(q + 0), B = __ldg(q + 1), C = __ldg(q + 2);
  const float p0x = A.x, p0y = A.y, p0z = A.z;
  const float e0x = A.w, e0y = B.x, e0z = B.y;
  const float e1x = B.z, e1y = B.w, e1z = C.x;
  const float nx = C.y, ny = C.z, nz = C.w;
  const float cx = fsub(p0x, r.px), cy = fsub(p0y, r.py), cz = fsub(p0z, r.pz);
  const float qx = fsub(fmul(r.dy, cz), fmul(r.dz, cy));
  const float qy = fsub(fmul(r.dz, cx), fmul(r.dx, cz));
  const float qz = fsub(fmul(r.dx, cy), fmul(r.dy, cx));
  const float inv_det = rcp_rn(dot3(nx, ny, nz, r.dx, r.dy, r.dz));
  u = fmul(dot3(qx, qy, qz, e1x, e1y, e1z), inv_det);
  v = fmul(dot3(qx, qy, qz, e0x, e0y, e0z), inv_det);
  const float w = fsub(fsub(1.0f, u), v);
  if ((u >= 0.0f) && (v >= 0.0f) && (w >= 0.0f)) {
    t = fmul(dot3(nx, ny, nz, cx, cy, cz), inv_det);
    return (t >= r.tmin) && (t <= r.tmax);
  }
  return false;
}

// One traversal node in two 256-bit loads (sm_100 and later; each half is
// 32-byte aligned: the node arrays come from cudaMallocAsync and hold
// 64-byte records). Read-only for the kernel's lifetime, hence .nc.
__device__ __forceinline__ void
load_wide(const WideNode* p, float4& A, float4& B, float4& C, float4& D)
{
  const float4* q = reinterpret_cast<const float4*>(p);
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(A.x), "=f"(A.y), "=f"(A.z), "=f"(A.w), "=f"(B.x), "=f"(B.y), "=f"(B.z), "=f"(B.w)
      : "l"(q));
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(C.x), "=f"(C.y), "=f"(C.z), "=f"(C.w), "=f"(D.x), "=f"(D.y), "=f"(D.z), "=f"(D.w)
      : "l"(q + 2));
}

// ---------------------------------------------------------------------------
// Traversal layout: node i = {left box, right box, left, right} in 64 bytes.
// A leaf child's box slot is unused (the reference tests leaf triangles
// directly).

__device__ __forceinline__ bool
bounded(float4 v)
{
  const float hi = 0x1p60f; // false for NaN
  return fabsf(v.x) <= hi && fabsf(v.y) <= hi && fabsf(v.z) <= hi && fabsf(v.w) <= hi;
}

__global__ void
k_repack(const Node* __restrict__ nodes, uint32_t n_nodes, WideNode* __restrict__ out, uint32_t* __restrict__ wide)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes)
    return;
  const float4* nv = reinterpret_cast<const float4*>(nodes);
  const float4 self = __ldg(nv + 2 * size_t(i) + 1);
  const uint32_t l = __float_as_uint(self.z), r = __float_as_uint(self.w);
  float4 la = make_float4(0, 0, 0, 0), lb = la, ra = la, rb = la;
  if (!(l & kLeafBit) && l < n_nodes) {
    la = __ldg(nv + 2 * size_t(l));
    lb = __ldg(nv + 2 * size_t(l) + 1);
  }
  if (!(r & kLeafBit) && r < n_nodes) {
    ra = __ldg(nv + 2 * size_t(r));
    rb = __ldg(nv + 2 * size_t(r) + 1);
  }
  if (!bounded(la) || !bounded(make_float4(lb.x, lb.y, ra.x, ra.y)) || !bounded(make_float4(ra.z, ra.w, rb.x, rb.y)))
    atomicOr(wide, 1u); // a coordinate beyond 2^60: no fast slab path
  WideNode w;
  w.a = make_float4(la.x, la.y, la.z, la.w); // left lo.xyz, hi.x
  w.b = make_float4(lb.x, lb.y, ra.x, ra.y); // left hi.yz, right lo.xy
  w.c = make_float4(ra.z, ra.w, rb.x, rb.y); // right lo.z, hi.xyz
  w.d = make_float4(__uint_as_float(l), __uint_as_float(r), 0.0f, 0.0f);
  out[i] = w;
}

// ---------------------------------------------------------------------------

// kBatch: rays [roff[k], roff[k + 1]) belong to mesh k, whose nodes start at
// moff[k] - k and whose triangles start at moff[k] (local indices inside).
//
// kHostHits: `hits` is page-locked host memory reached over the CPU-GPU
// link, where 16-byte stores scattered in time travel one by one. Each warp
// then keeps the hits of its last kHitRing ray batches (32 consecutive rays
// each) in shared memory and writes a batch out with one 512-byte store of
// the warp once its last ray has finished; a batch that finds its ring entry
// still taken by an unfinished older batch writes its hits directly.
constexpr uint32_t kHitRing = 4;
constexpr uint32_t kHitDirect = kHitRing; // a ray whose hit is written directly

#ifndef LBVH_TRACE_MIN_BLOCKS
#define LBVH_TRACE_MIN_BLOCKS 8 // resident CTAs per SM the register budget is set for
#endif
#ifndef LBVH_TRACE_MIN_BLOCKS_LEAF
#define LBVH_TRACE_MIN_BLOCKS_LEAF 9 // the same for the leaf-batching variant (56 registers)
#endif

// kLeafBatch: the leaf triangles of a visit are tested when leaf_batch of
// the warp's lanes have some pending (see below); otherwise right after the
// visit, by the lane alone.
template<bool kCounts, bool kBatch, bool kHostHits = false, bool kLeafBatch = false>
__global__ __launch_bounds__(kTraceThreads, kLeafBatch ? LBVH_TRACE_MIN_BLOCKS_LEAF : LBVH_TRACE_MIN_BLOCKS) void
k_trace(const WideNode* __restrict__ wnodes,
        const Tri* __restrict__ tris,
        const uint32_t* __restrict__ leaf_prim,
        const float4* __restrict__ rays,
        uint32_t m,
        Hit* __restrict__ hits,
        uint32_t* __restrict__ n_box,
        uint32_t* __restrict__ n_tri,
        uint32_t* __restrict__ ray_counter,
        const uint32_t* __restrict__ wide,
        uint32_t refill,
        uint32_t leaf_batch,
        const uint32_t* __restrict__ order,
        const uint32_t* __restrict__ moff,
        const uint32_t* __restrict__ roff,
        uint32_t n_meshes)
{
  const bool scene_fast = __ldg(wide) == 0;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const float inf = __int_as_float(0x7f800000);

  // The traversal stack: entries [0, sp) in local memory plus, when has_cur,
  // one more entry on top held in registers (the entry popped next). The
  // 128-entry capacity applies to the whole, so pushes drop exactly when the
  // reference's would.
  uint2 stack[kStackSize];
  uint32_t sp = 0;
  uint2 cur = make_uint2(0u, 0u);
  bool has_cur = false;
  bool pend = false;                   // the leaf children of the last visit are not yet tested
  uint32_t leaf_l = kMiss, leaf_r = kMiss; // those leaf children (kMiss: an internal child)
  uint32_t ray = kMiss; // ray index of this lane, kMiss = none
  RayCtx r{};
  uint32_t best_p = kMiss;
  float best_t = inf, best_u = 0.0f, best_v = 0.0f;
  uint32_t cb = 0, ct = 0;
  uint32_t nb = 0, tb = 0; // batched: the ray's mesh node and triangle bases

  // the warp's current batch of 32 ray ids (warp-uniform state)
  uint32_t batch = 0, batch_left = 0;
  bool no_more = false; // the last batch fetched reached the end of the rays

  // kHostHits: per warp, kHitRing staged batches {hits, first ray, rays left}
  constexpr int kWarps = kTraceThreads / 32;
  __shared__ Hit s_hits[kHostHits ? kWarps : 1][kHostHits ? kHitRing : 1][32];
  __shared__ uint32_t s_first[kHostHits ? kWarps : 1][kHostHits ? kHitRing : 1];
  __shared__ uint32_t s_left[kHostHits ? kWarps : 1][kHostHits ? kHitRing : 1];
  const uint32_t wid = threadIdx.x >> 5;
  uint32_t seq = 0;             // batches this warp has fetched
  uint32_t batch_buf = kHitDirect; // ring entry of the current batch
  uint32_t buf = kHitDirect;    // ring entry of this lane's ray
  bool flush = false;           // this lane finished the last ray of its batch
  if (kHostHits) {
    if (lane < kHitRing)
      s_left[wid][lane] = 0;
    __syncwarp();
  }

  for (;;) {
    if (kHostHits) {
      // ---- write out the batches whose last ray finished (whole warp) ----
      uint32_t fl = __ballot_sync(0xffffffffu, flush);
      if (fl) {
        __syncwarp(); // the staged hits of every lane are visible
        while (fl) {
          const uint32_t src = __ffs(fl) - 1;
          fl &= fl - 1;
          const uint32_t b = __shfl_sync(0xffffffffu, buf, src);
          const uint32_t first = s_first[wid][b];
          if (first + lane < m)
            hits[first + lane] = s_hits[wid][b][lane];
        }
        __syncwarp(); // every read of the ring entries before they are reused
        if (flush) {
          buf = kHitDirect;
          flush = false;
        }
      }
    }
    // ---- refill idle lanes from the warp's batch (ballot + shuffle) ----
    const uint32_t idle = __ballot_sync(0xffffffffu, ray == kMiss);
    if (__popc(idle) >= refill) { // warp-uniform; refill <= 32
      const uint32_t next_id = batch + 32 - batch_left;
      const bool more = (batch_left > 0 && next_id < m) || !no_more;
      if (!more) {
        if (idle == 0xffffffffu)
          break; // every ray handed to this warp has finished
      } else {
        const uint32_t want = __popc(idle);
        const uint32_t got = min(want, batch_left);
        batch_left -= got;
        uint32_t extra_base = 0;
        bool fetched = false;
        const uint32_t old_buf = batch_buf;
        if (got < want && !no_more) {
          uint32_t nb = 0;
          if (lane == 0)
            nb = atomicAdd(ray_counter, 32u);
          nb = __shfl_sync(0xffffffffu, nb, 0);
          no_more = nb + 32 >= m;
          extra_base = nb;
          batch = nb;
          batch_left = 32 - (want - got);
          fetched = true;
          if (kHostHits && nb < m) {
            // the ring entry of this batch, unless an older batch still holds it
            const uint32_t k = seq % kHitRing;
            seq++;
            batch_buf = kHitDirect;
            if (s_left[wid][k] == 0) {
              batch_buf = k;
              __syncwarp();
              if (lane == 0) {
                s_first[wid][k] = nb;
                s_left[wid][k] = min(32u, m - nb);
              }
              __syncwarp();
            }
          }
        }
        if (ray == kMiss) {
          const uint32_t k = __popc(idle & lt_mask);
          uint32_t id = kMiss;
          uint32_t id_buf = old_buf;
          if (k < got) {
            id = next_id + k;
          } else if (fetched) {
            id = extra_base + (k - got);
            id_buf = batch_buf;
          }
          if (id < m) {
            if (order) // rays taken in a sorted order; each hit still goes to its ray's slot
              id = min(__ldg(order + id), m - 1); // < m unless the ray sort gave up (error reported)
            ray = id;
            if (kHostHits)
              buf = id_buf;
            r = make_ray(__ldg(rays + 2 * size_t(id)), __ldg(rays + 2 * size_t(id) + 1));
            r.fast = r.fast && scene_fast;
          if (kBatch) { // the mesh k with roff[k] <= id < roff[k + 1]
            uint32_t lo = 0, hi = n_meshes; // invariant: roff[lo] <= id < roff[hi]
            while (hi - lo > 1) {
              const uint32_t mid = (lo + hi) >> 1;
              if (__ldg(roff + mid) <= id)
                lo = mid;
              else
                hi = mid;
            }
            tb = __ldg(moff + lo);
            nb = tb - lo;
          }
            sp = 0;
            cur = make_uint2(0u, __float_as_uint(inf)); // root, pushed with +inf
            has_cur = true;
            best_p = kMiss;
            best_t = inf;
            best_u = best_v = 0.0f;
            cb = ct = 0;
          }
        }
      }
    }
    const bool busy = ray != kMiss;

    // ---- one node visit (lbvh.h:1902-1938) for the lanes whose previous
    // visit is complete; cur passed the cull test ----
    if (busy && !pend) {
      float4 A, B, C, D;
      load_wide(wnodes + nb + cur.x, A, B, C, D);
      const uint32_t left = __float_as_uint(D.x), right = __float_as_uint(D.y);
      bool lhit = false, rhit = false;
      float lt = inf, rt = inf;
      if (kCounts)
        cb += uint32_t(!(left & kLeafBit)) + uint32_t(!(right & kLeafBit));
      if (r.fast) {
        // both boxes at once; a leaf child's box slot holds zeros, its
        // result is discarded
        box_pair_fast(r, A, B, C, lhit, rhit, lt, rt);
        lhit = lhit && !(left & kLeafBit);
        rhit = rhit && !(right & kLeafBit);
      } else {
        if (!(left & kLeafBit))
          lhit = box_test(r, A.x, A.y, A.z, A.w, B.x, B.y, lt);
        if (!(right & kLeafBit))
          rhit = box_test(r, B.z, B.w, C.x, C.y, C.z, C.w, rt);
      }
      // leaf children: tested left before right, before this lane's next
      // pop (so its cull test sees their hits, as in the reference) -- here,
      // or with the warp's other pending lanes below
      leaf_l = (left & kLeafBit) ? (left & ~kLeafBit) : kMiss;
      leaf_r = (right & kLeafBit) ? (right & ~kLeafBit) : kMiss;
      if (kLeafBatch) {
        pend = ((left | right) & kLeafBit) != 0;
      } else if ((left | right) & kLeafBit) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
          const uint32_t p = k == 0 ? leaf_l : leaf_r;
          if (p != kMiss) {
            float t, u, v;
            if (kCounts)
              ct++;
            if (tri_test(r, tris + tb, p, t, u, v) && t < best_t) {
              best_p = p;
              best_t = t;
              best_u = u;
              best_v = v;
            }
          }
        }
      }
      // pushes; the last one pushed stays in registers as the next pop
      has_cur = false;
      if (lhit && rhit) {
        const bool lfirst = lt < rt; // left nearer: push right, then left
        const uint2 far = lfirst ? make_uint2(right, __float_as_uint(rt)) : make_uint2(left, __float_as_uint(lt));
        const uint2 near = lfirst ? make_uint2(left, __float_as_uint(lt)) : make_uint2(right, __float_as_uint(rt));
        if (sp < kStackSize)
          stack[sp++] = far;
        if (sp < kStackSize) {
          cur = near;
          has_cur = true;
        }
      } else if (lhit || rhit) {
        if (sp < kStackSize) {
          cur = lhit ? make_uint2(left, __float_as_uint(lt)) : make_uint2(right, __float_as_uint(rt));
          has_cur = true;
        }
      }
    }

    // ---- leaf triangles of the pending lanes (equal t: the first tested
    // wins). The block costs the warp the same whether one lane or many run
    // it, so a lane with pending triangles sits out node visits until
    // leaf_batch lanes are pending, or until no lane is left to visit; each
    // ray still visits, tests and pops in the reference's order. ----
    const uint32_t pmask = kLeafBatch ? __ballot_sync(0xffffffffu, pend) : 0u;
    if (pmask && (uint32_t(__popc(pmask)) >= leaf_batch || __ballot_sync(0xffffffffu, busy && !pend) == 0)) {
      if (pend) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
          const uint32_t p = k == 0 ? leaf_l : leaf_r;
          if (p != kMiss) {
            float t, u, v;
            if (kCounts)
              ct++;
            if (tri_test(r, tris + tb, p, t, u, v) && t < best_t) {
              best_p = p;
              best_t = t;
              best_u = u;
              best_v = v;
            }
          }
        }
        pend = false;
      }
    }
    if (!busy || pend)
      continue;

    // ---- next entry: pop until one passes the cull test (lbvh.h:1893-1900) ----
    for (;;) {
      if (!has_cur) {
        if (sp == 0)
          break;
        cur = stack[--sp];
      }
      has_cur = !(best_t < __uint_as_float(cur.y));
      if (has_cur)
        break;
    }
    if (!has_cur) {
      Hit h;
      h.prim = (best_p != kMiss && leaf_prim) ? __ldg(leaf_prim + tb + best_p) : best_p;
      h.t = best_t;
      h.u = best_p != kMiss ? best_u : 0.0f;
      h.v = best_p != kMiss ? best_v : 0.0f;
      if (kHostHits && buf != kHitDirect) {
        s_hits[wid][buf][ray - s_first[wid][buf]] = h;
        flush = atomicSub(&s_left[wid][buf], 1u) == 1u; // the batch's last ray
      } else {
        hits[ray] = h;
      }
      if (kCounts) {
        n_box[ray] = cb;
        n_tri[ray] = ct;
      }
      ray = kMiss;
    }
  }
}

// Ray sort keys (launch_ray_keys): a heuristic trace order, so any key is
// correct; the traversal of each ray and its hit do not depend on it.
__device__ __forceinline__ uint32_t
cell4(float v, float lo, float inv)
{
  const float q = (v - lo) * inv; // NaN and out-of-range values clamp
  return q >= 15.0f ? 15u : (q > 0.0f ? uint32_t(q) : 0u);
}

__device__ __forceinline__ uint32_t
spread4(uint32_t x) // 4 bits to every third bit
{
  return (x & 1u) | ((x & 2u) << 2) | ((x & 4u) << 4) | ((x & 8u) << 6);
}

__global__ __launch_bounds__(256) void
k_ray_keys(const float4* __restrict__ rays, uint32_t m, const Node* __restrict__ nodes, uint32_t* __restrict__ keys,
           BuildState* __restrict__ st)
{
  __shared__ uint32_t s_hist[3 * 256];
  for (uint32_t k = threadIdx.x; k < 3 * 256; k += blockDim.x)
    s_hist[k] = 0;
  __syncthreads();
  const Node root = nodes[0];
  float ilo[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float ext = root.hi[k] - root.lo[k];
    ilo[k] = ext > 0.0f ? 16.0f / ext : 0.0f;
  }
  const uint32_t lane = threadIdx.x & 31;
  // whole warps iterate together, so the digit counts can be added once per
  // warp and value (a digit that most rays share -- the origin cell of
  // camera rays -- would otherwise serialize its shared-memory atomics)
  for (uint32_t base = blockIdx.x * blockDim.x; base < m; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const bool valid = i < m;
    const float4 a = valid ? __ldg(rays + 2 * size_t(i)) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 b = valid ? __ldg(rays + 2 * size_t(i) + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float dx = a.w, dy = b.x, dz = b.y;
    const float big = fmaxf(fmaxf(fabsf(dx), fabsf(dy)), fabsf(dz));
    const float id = big > 0.0f ? 8.0f / big : 0.0f; // components to [-8, 8], then cells of 1
    const uint32_t o = (spread4(cell4(a.x, root.lo[0], ilo[0])) << 2) | (spread4(cell4(a.y, root.lo[1], ilo[1])) << 1) |
                       spread4(cell4(a.z, root.lo[2], ilo[2]));
    const uint32_t d = (spread4(cell4(dx * id, -8.0f, 1.0f)) << 2) | (spread4(cell4(dy * id, -8.0f, 1.0f)) << 1) |
                       spread4(cell4(dz * id, -8.0f, 1.0f));
    const uint32_t key = (o << 12) | d;
    if (valid)
      keys[i] = key;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const uint32_t dg = valid ? (key >> (8 * k)) & 255u : 256u + lane; // invalid lanes match nobody
      const uint32_t peers = __match_any_sync(0xffffffffu, dg);
      if (valid && (__ffs(peers) - 1) == int(lane))
        atomicAdd(&s_hist[256 * k + dg], uint32_t(__popc(peers)));
    }
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < 3 * 256; k += blockDim.x)
    if (s_hist[k])
      atomicAdd(&(&st->hist[0][0])[k], s_hist[k]);
  if (blockIdx.x == 0 && threadIdx.x == 0) // the fourth digit is zero for every key
    atomicAdd(&st->hist[3][0], m);
}

cudaError_t
launch_ray_keys(const float* rays, uint32_t m, const Node* nodes, uint32_t* keys, BuildState* st, cudaStream_t s)
{
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint32_t want = ceil_div_u32(m, 256), cap = uint32_t(sms) * 8;
  k_ray_keys<<<want < cap ? want : cap, 256, 0, s>>>(reinterpret_cast<const float4*>(rays), m, nodes, keys, st);
  return cudaGetLastError();
}

cudaError_t
launch_repack(const Node* nodes, uint32_t n_nodes, WideNode* out, cudaStream_t s)
{
  // the scene-bound flag lives in the word after the last node
  uint32_t* wide = reinterpret_cast<uint32_t*>(out + n_nodes);
  cudaError_t e = cudaMemsetAsync(wide, 0, 4, s);
  if (e != cudaSuccess)
    return e;
  k_repack<<<ceil_div_u32(n_nodes, 256), 256, 0, s>>>(nodes, n_nodes, out, wide);
  return cudaGetLastError();
}

cudaError_t
launch_trace_tris(const WideNode* wnodes,
                  uint32_t n_nodes,
                  const Tri* tris,
                  const uint32_t* leaf_prim,
                  const float* rays,
                  uint32_t m,
                  Hit* hits,
                  uint32_t* n_box,
                  uint32_t* n_tri,
                  uint32_t* ray_counter,
                  int num_sms,
                  const TraceParams& p,
                  cudaStream_t s,
                  bool host_hits,
                  const uint32_t* order)
{
  if (m == 0)
    return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(ray_counter, 0, 4, s);
  if (e != cudaSuccess)
    return e;
  // persistent grid: enough resident warps per SM, never more than the rays
  const uint32_t want = ceil_div_u32(m, kTraceThreads);
  const uint32_t cap = uint32_t(num_sms) * p.blocks_per_sm;
  const uint32_t blocks = want < cap ? want : cap;
  const float4* r4 = reinterpret_cast<const float4*>(rays);
  const uint32_t* wide = reinterpret_cast<const uint32_t*>(wnodes + n_nodes);
  // leaf batching pays for long rays in loose trees (the tuner decides)
  auto go = [&](auto kernel, uint32_t* nb, uint32_t* nt) {
    kernel<<<blocks, kTraceThreads, 0, s>>>(wnodes, tris, leaf_prim, r4, m, hits, nb, nt, ray_counter, wide, p.refill,
                                           p.leaf_batch, host_hits ? nullptr : order, nullptr, nullptr, 0);
  };
  const bool counts = n_box && n_tri;
  if (p.leaf_batch > 1) {
    if (counts)
      go(k_trace<true, false, false, true>, n_box, n_tri);
    else if (host_hits)
      go(k_trace<false, false, true, true>, nullptr, nullptr);
    else
      go(k_trace<false, false, false, true>, nullptr, nullptr);
  } else {
    if (counts)
      go(k_trace<true, false>, n_box, n_tri);
    else if (host_hits)
      go(k_trace<false, false, true>, nullptr, nullptr);
    else
      go(k_trace<false, false>, nullptr, nullptr);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// User-primitive traversal: spheres with the intersector of the reference's
// example program (examples/minimal.cpp:92-135), over a tree built from the
// spheres' boxes. The traversal is traverser::operator() (lbvh.h:1874-1942)
// with the intersector swapped: one thread per ray, the same visiting order,
// stack semantics and closest-hit rule (a result replaces the closest only
// when its t is smaller; leaf children are tested left first).

struct SphereInfo
{
  float t, u, v, nx, ny, nz;
};

// The example's sphere intersection, with its operation order: the nearer
// root unless it is negative (then the other root, negative or not), the
// normal normalized as lbvh::math::normalize does (lbvh.h:724-734), and uv
// from atan2 / acos. A ray that misses returns t = +inf. The ray's tmin and
// tmax are not consulted, as in the example.
__device__ __forceinline__ SphereInfo
sphere_test(const RayCtx& r, float4 s)
{
  const float inf = __int_as_float(0x7f800000);
  const float rad = s.x, cx = s.y, cy = s.z, cz = s.w;
  const float ox = fsub(r.px, cx), oy = fsub(r.py, cy), oz = fsub(r.pz, cz); // ray.pos - s_pos
  const float a = dot3(r.dx, r.dy, r.dz, r.dx, r.dy, r.dz);
  const float b = fmul(2.0f, dot3(r.dx, r.dy, r.dz, ox, oy, oz));
  const float c = fsub(dot3(ox, oy, oz, ox, oy, oz), fmul(rad, rad));
  const float disc = fsub(fmul(b, b), fmul(fmul(4.0f, a), c));
  if (disc < 0.0f)
    return SphereInfo{ inf, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f };
  const float sq = __fsqrt_rn(disc);
  const float den = fmul(2.0f, a);
  const float t0 = fdiv(fadd(-b, sq), den);
  const float t1 = fdiv(fsub(-b, sq), den);
  const float t = (t0 < 0.0f) ? t1 : t0;
  const float vx = fsub(fadd(r.px, fmul(r.dx, t)), cx); // hit_pos - s_pos
  const float vy = fsub(fadd(r.py, fmul(r.dy, t)), cy);
  const float vz = fsub(fadd(r.pz, fmul(r.dz, t)), cz);
  const float l_inv = fdiv(1.0f, __fsqrt_rn(dot3(vx, vy, vz, vx, vy, vz)));
  const float nx = fmul(vx, l_inv), ny = fmul(vy, l_inv), nz = fmul(vz, l_inv);
  const float pi = 3.14159274101257324f; // float(M_PI)
  return SphereInfo{ t, fmul(fadd(1.0f, fdiv(atan2f(nz, nx), pi)), 0.5f), fdiv(acosf(ny), pi), nx, ny, nz };
}

__global__ __launch_bounds__(kTraceThreads) void
k_trace_spheres(const WideNode* __restrict__ wnodes,
                const float4* __restrict__ spheres,
                const float4* __restrict__ rays,
                uint32_t m,
                SphereHit* __restrict__ hits)
{
  const float inf = __int_as_float(0x7f800000);
  uint2 stack[kStackSize];
  for (uint32_t ray = blockIdx.x * blockDim.x + threadIdx.x; ray < m; ray += gridDim.x * blockDim.x) {
    RayCtx r = make_ray(__ldg(rays + 2 * size_t(ray)), __ldg(rays + 2 * size_t(ray) + 1));
    r.fast = false; // the reference's own min/max ternaries throughout
    uint32_t best_p = kMiss;
    SphereInfo best{ inf, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f };
    uint32_t sp = 0;
    stack[sp++] = make_uint2(0u, __float_as_uint(inf)); // root, pushed with +inf
    while (sp) {
      const uint2 e = stack[--sp];
      if (best.t < __uint_as_float(e.y))
        continue;
      float4 A, B, C, D;
      load_wide(wnodes + e.x, A, B, C, D);
      const uint32_t left = __float_as_uint(D.x), right = __float_as_uint(D.y);
      bool lhit = false, rhit = false;
      float lt = inf, rt = inf;
      if (left & kLeafBit) {
        const uint32_t p = left & ~kLeafBit;
        const SphereInfo h = sphere_test(r, __ldg(spheres + p));
        if (h.t < best.t) {
          best = h;
          best_p = p;
        }
      } else {
        lhit = box_test(r, A.x, A.y, A.z, A.w, B.x, B.y, lt);
      }
      if (right & kLeafBit) {
        const uint32_t p = right & ~kLeafBit;
        const SphereInfo h = sphere_test(r, __ldg(spheres + p));
        if (h.t < best.t) {
          best = h;
          best_p = p;
        }
      } else {
        rhit = box_test(r, B.z, B.w, C.x, C.y, C.z, C.w, rt);
      }
      if (lhit && rhit) {
        const bool lfirst = lt < rt; // left nearer: push right, then left
        const uint2 far = lfirst ? make_uint2(right, __float_as_uint(rt)) : make_uint2(left, __float_as_uint(lt));
        const uint2 near = lfirst ? make_uint2(left, __float_as_uint(lt)) : make_uint2(right, __float_as_uint(rt));
        if (sp < kStackSize)
          stack[sp++] = far;
        if (sp < kStackSize)
          stack[sp++] = near;
      } else if (lhit || rhit) {
        if (sp < kStackSize)
          stack[sp++] = lhit ? make_uint2(left, __float_as_uint(lt)) : make_uint2(right, __float_as_uint(rt));
      }
    }
    SphereHit out;
    out.prim = best_p;
    if (best_p == kMiss)
      best = SphereInfo{ inf, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f };
    out.t = best.t;
    out.u = best.u;
    out.v = best.v;
    out.nx = best.nx;
    out.ny = best.ny;
    out.nz = best.nz;
    out.pad = 0.0f;
    hits[ray] = out;
  }
}

cudaError_t
launch_trace_spheres(const WideNode* wnodes,
                     const float4* spheres,
                     const float* rays,
                     uint32_t m,
                     SphereHit* hits,
                     int num_sms,
                     cudaStream_t s)
{
  if (m == 0)
    return cudaSuccess;
  const uint32_t want = ceil_div_u32(m, kTraceThreads);
  const uint32_t cap = uint32_t(num_sms) * 8;
  k_trace_spheres<<<want < cap ? want : cap, kTraceThreads, 0, s>>>(wnodes, spheres,
                                                                   reinterpret_cast<const float4*>(rays), m, hits);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batched meshes (launch_batch_repack / launch_batch_trace, batch.cuh)

__global__ void
k_batch_repack(const Node* __restrict__ nodes,
               uint32_t total_nodes,
               const uint32_t* __restrict__ off,
               uint32_t n_meshes,
               WideNode* __restrict__ out,
               uint32_t* __restrict__ wide)
{
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total_nodes)
    return;
  // the mesh k with off[k] - k <= g < off[k + 1] - (k + 1)
  uint32_t lo = 0, hi = n_meshes;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(off + mid) - mid <= g)
      lo = mid;
    else
      hi = mid;
  }
  const uint32_t base = __ldg(off + lo) - lo;
  const uint32_t nn = __ldg(off + lo + 1) - __ldg(off + lo) - 1; // the mesh's internal nodes
  const float4* nv = reinterpret_cast<const float4*>(nodes + base);
  const uint32_t i = g - base;
  const float4 self = __ldg(nv + 2 * size_t(i) + 1);
  const uint32_t l = __float_as_uint(self.z), r = __float_as_uint(self.w);
  float4 la = make_float4(0, 0, 0, 0), lb = la, ra = la, rb = la;
  if (!(l & kLeafBit) && l < nn) {
    la = __ldg(nv + 2 * size_t(l));
    lb = __ldg(nv + 2 * size_t(l) + 1);
  }
  if (!(r & kLeafBit) && r < nn) {
    ra = __ldg(nv + 2 * size_t(r));
    rb = __ldg(nv + 2 * size_t(r) + 1);
  }
  if (!bounded(la) || !bounded(make_float4(lb.x, lb.y, ra.x, ra.y)) || !bounded(make_float4(ra.z, ra.w, rb.x, rb.y)))
    atomicOr(wide, 1u);
  WideNode w;
  w.a = make_float4(la.x, la.y, la.z, la.w);
  w.b = make_float4(lb.x, lb.y, ra.x, ra.y);
  w.c = make_float4(ra.z, ra.w, rb.x, rb.y);
  w.d = make_float4(__uint_as_float(l), __uint_as_float(r), 0.0f, 0.0f);
  out[g] = w;
}

cudaError_t
launch_batch_repack(const Node* nodes, uint32_t total_nodes, const uint32_t* off, uint32_t n_meshes, WideNode* out,
                    cudaStream_t s)
{
  uint32_t* wide = reinterpret_cast<uint32_t*>(out + total_nodes);
  cudaError_t e = cudaMemsetAsync(wide, 0, 4, s);
  if (e != cudaSuccess)
    return e;
  if (total_nodes)
    k_batch_repack<<<ceil_div_u32(total_nodes, 256), 256, 0, s>>>(nodes, total_nodes, off, n_meshes, out, wide);
  return cudaGetLastError();
}

cudaError_t
launch_batch_trace(const WideNode* wnodes,
                   uint32_t total_nodes,
                   const Tri* tris,
                   const uint32_t* leaf_prim,
                   const uint32_t* off,
                   const uint32_t* roff,
                   uint32_t n_meshes,
                   const float* rays,
                   uint32_t m,
                   Hit* hits,
                   uint32_t* ray_counter,
                   int num_sms,
                   const TraceParams& p,
                   cudaStream_t s)
{
  if (m == 0)
    return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(ray_counter, 0, 4, s);
  if (e != cudaSuccess)
    return e;
  const uint32_t want = ceil_div_u32(m, kTraceThreads);
  const uint32_t cap = uint32_t(num_sms) * p.blocks_per_sm;
  const uint32_t blocks = want < cap ? want : cap;
  const uint32_t* wide = reinterpret_cast<const uint32_t*>(wnodes + total_nodes);
  const float4* r4 = reinterpret_cast<const float4*>(rays);
  if (p.leaf_batch > 1)
    k_trace<false, true, false, true><<<blocks, kTraceThreads, 0, s>>>(wnodes, tris, leaf_prim, r4, m, hits, nullptr,
                                                                      nullptr, ray_counter, wide, p.refill,
                                                                      p.leaf_batch, nullptr, off, roff, n_meshes);
  else
    k_trace<false, true><<<blocks, kTraceThreads, 0, s>>>(wnodes, tris, leaf_prim, r4, m, hits, nullptr, nullptr,
                                                          ray_counter, wide, p.refill, p.leaf_batch, nullptr, off,
                                                          roff, n_meshes);
  return cudaGetLastError();
}

} // namespace lbvh_gb300
