// Closest-hit ray/triangle traversal for sm_103a.
//
// Replaces traverser<float, triangle<float>, triangle_intersection<float>>::
// operator() with triangle_intersector<float> (lbvh.h:1869-1942, 2055-2075),
// one ray per thread, with the reference's exact visiting order:
//   * a 128-entry stack of {node, tmin} that drops pushes when full
//     (lbvh.h:1746-1789), seeded with {root, +inf};
//   * pop; skip if closest.t < entry.tmin;
//   * leaf children are intersected when their parent is popped, left first;
//     internal children are box-tested (octant form, lbvh.h:1071-1091);
//   * both hit: push the farther first (equal tmin: right popped first).
// All arithmetic uses explicit round-to-nearest ops, so hits (id, t, u, v)
// are bit-identical to the reference.
#include "trace.cuh"

namespace lbvh_gb300 {

struct RayCtx
{
  float px, py, pz, dx, dy, dz, tmin, tmax;
  float rx, ry, rz;   // reciprocal direction
  float ix, iy, iz;   // (-pos) * rcp
  bool sx, sy, sz;    // dir > 0: near plane is the box minimum
};

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
  r.rx = fdiv(1.0f, r.dx);
  r.ry = fdiv(1.0f, r.dy);
  r.rz = fdiv(1.0f, r.dz);
  r.ix = fmul(-r.px, r.rx);
  r.iy = fmul(-r.py, r.ry);
  r.iz = fmul(-r.pz, r.rz);
  r.sx = r.dx > 0.0f;
  r.sy = r.dy > 0.0f;
  r.sz = r.dz > 0.0f;
  return r;
}

// detail::intersect (octant form) + box_intersection::operator bool,
// lbvh.h:1026-1029, 1071-1091. Box = {lo.x, lo.y, lo.z, hi.x}, {hi.y, hi.z}.
__device__ __forceinline__ bool
box_test(const RayCtx& r, float4 a, float2 b, float& tmin_out)
{
  const float lox = a.x, loy = a.y, loz = a.z, hix = a.w, hiy = b.x, hiz = b.y;
  const float tn0 = fadd(fmul(r.sx ? lox : hix, r.rx), r.ix);
  const float tn1 = fadd(fmul(r.sy ? loy : hiy, r.ry), r.iy);
  const float tn2 = fadd(fmul(r.sz ? loz : hiz, r.rz), r.iz);
  const float tf0 = fadd(fmul(r.sx ? hix : lox, r.rx), r.ix);
  const float tf1 = fadd(fmul(r.sy ? hiy : loy, r.ry), r.iy);
  const float tf2 = fadd(fmul(r.sz ? hiz : loz, r.rz), r.iz);
  const float tmin = mmax(mmax(tn0, tn1), tn2);
  const float tmax = mmin(mmin(tf0, tf1), tf2);
  tmin_out = tmin;
  return tmax >= mmax(0.0f, tmin);
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
  const float inv_det = fdiv(1.0f, dot3(nx, ny, nz, r.dx, r.dy, r.dz));
  u = fmul(dot3(qx, qy, qz, e1x, e1y, e1z), inv_det);
  v = fmul(dot3(qx, qy, qz, e0x, e0y, e0z), inv_det);
  const float w = fsub(fsub(1.0f, u), v);
  if ((u >= 0.0f) && (v >= 0.0f) && (w >= 0.0f)) {
    t = fmul(dot3(nx, ny, nz, cx, cy, cz), inv_det);
    return (t >= r.tmin) && (t <= r.tmax);
  }
  return false;
}

template<bool kCounts>
__global__ __launch_bounds__(kTraceThreads) void
k_trace_tris(const Node* __restrict__ nodes,
             const Tri* __restrict__ tris,
             const uint32_t* __restrict__ leaf_prim,
             const float4* __restrict__ rays,
             uint32_t m,
             Hit* __restrict__ hits,
             uint32_t* __restrict__ n_box,
             uint32_t* __restrict__ n_tri)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m)
    return;
  const RayCtx r = make_ray(__ldg(rays + 2 * size_t(i)), __ldg(rays + 2 * size_t(i) + 1));
  const float inf = __int_as_float(0x7f800000);

  uint2 stack[kStackSize];
  uint32_t sp = 0;
  stack[sp++] = make_uint2(0u, __float_as_uint(inf));

  uint32_t best_p = kMiss;
  float best_t = inf, best_u = 0.0f, best_v = 0.0f;
  uint32_t cb = 0, ct = 0;

  const float4* nv = reinterpret_cast<const float4*>(nodes);
  while (sp) {
    const uint2 e = stack[--sp];
    if (best_t < __uint_as_float(e.y))
      continue;
    const float4 nb = __ldg(nv + 2 * size_t(e.x) + 1);
    const uint32_t left = __float_as_uint(nb.z), right = __float_as_uint(nb.w);
    bool lhit = false, rhit = false;
    float lt = inf, rt = inf;
    if (left & kLeafBit) {
      const uint32_t p = left & ~kLeafBit;
      float t, u, v;
      if (kCounts)
        ct++;
      if (tri_test(r, tris, p, t, u, v) && t < best_t) {
        best_p = p;
        best_t = t;
        best_u = u;
        best_v = v;
      }
    } else {
      if (kCounts)
        cb++;
      const float4 a = __ldg(nv + 2 * size_t(left));
      const float2 b = __ldg(reinterpret_cast<const float2*>(nv + 2 * size_t(left) + 1));
      lhit = box_test(r, a, b, lt);
    }
    if (right & kLeafBit) {
      const uint32_t p = right & ~kLeafBit;
      float t, u, v;
      if (kCounts)
        ct++;
      if (tri_test(r, tris, p, t, u, v) && t < best_t) {
        best_p = p;
        best_t = t;
        best_u = u;
        best_v = v;
      }
    } else {
      if (kCounts)
        cb++;
      const float4 a = __ldg(nv + 2 * size_t(right));
      const float2 b = __ldg(reinterpret_cast<const float2*>(nv + 2 * size_t(right) + 1));
      rhit = box_test(r, a, b, rt);
    }
    if (lhit && rhit) {
      const bool lfirst = lt < rt; // left nearer: push right, then left
      const uint2 fst = lfirst ? make_uint2(right, __float_as_uint(rt)) : make_uint2(left, __float_as_uint(lt));
      const uint2 snd = lfirst ? make_uint2(left, __float_as_uint(lt)) : make_uint2(right, __float_as_uint(rt));
      if (sp < kStackSize)
        stack[sp++] = fst;
      if (sp < kStackSize)
        stack[sp++] = snd;
    } else if (lhit) {
      if (sp < kStackSize)
        stack[sp++] = make_uint2(left, __float_as_uint(lt));
    } else if (rhit) {
      if (sp < kStackSize)
        stack[sp++] = make_uint2(right, __float_as_uint(rt));
    }
  }
  Hit h;
  h.prim = (best_p != kMiss && leaf_prim) ? __ldg(leaf_prim + best_p) : best_p;
  h.t = best_t;
  h.u = best_p != kMiss ? best_u : 0.0f;
  h.v = best_p != kMiss ? best_v : 0.0f;
  hits[i] = h;
  if (kCounts) {
    n_box[i] = cb;
    n_tri[i] = ct;
  }
}

cudaError_t
launch_trace_tris(const Node* nodes,
                  const Tri* tris,
                  const uint32_t* leaf_prim,
                  const float* rays,
                  uint32_t m,
                  Hit* hits,
                  uint32_t* n_box,
                  uint32_t* n_tri,
                  cudaStream_t s)
{
  if (m == 0)
    return cudaSuccess;
  const uint32_t blocks = ceil_div_u32(m, kTraceThreads);
  const float4* r4 = reinterpret_cast<const float4*>(rays);
  if (n_box && n_tri)
    k_trace_tris<true><<<blocks, kTraceThreads, 0, s>>>(nodes, tris, leaf_prim, r4, m, hits, n_box, n_tri);
  else
    k_trace_tris<false><<<blocks, kTraceThreads, 0, s>>>(nodes, tris, leaf_prim, r4, m, hits, nullptr, nullptr);
  return cudaGetLastError();
}

} // namespace lbvh_gb300
