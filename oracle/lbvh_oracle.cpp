// ORACLE -- test infrastructure, not product code.
//
// A CPU restatement, in plain C++17, of the reference LBVH (tay10r/lbvh,
// header `lbvh.h`) for the build + closest-hit trace path. Tests, the smoke
// check and bench.py's CPU-baseline leg load it (as oracle/liboracle.so) to
// check the CUDA library and to time the reference algorithm on host cores.
// The product library never links or calls it.
//
// Parity is pinned: tests/golden/ holds outputs of the unmodified reference
// (compiled here from its own header by oracle/Makefile -> oracle/_ref/), and
// tests/test_oracle.py checks this file against them bit for bit.
//
// Compile with -ffp-contract=off and without -ffast-math: the reference's
// triangle normal (lbvh.h:1967-1972) and intersector (lbvh.h:2055-2075) are
// sensitive to FMA contraction.
//
// Threading mirrors the reference so the CPU timing is representative:
// per-stage std::thread spawn/join over contiguous chunks (lbvh.h:123-146,
// 961-986), a serial std::sort (lbvh.h:1126-1134; no TBB backend), and a serial
// box fit (lbvh.h:1826-1867).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

struct v3
{
  float x, y, z;
};

struct box3
{
  v3 lo, hi;
};

struct node32
{
  box3 box;
  uint32_t left, right;
};

static_assert(sizeof(node32) == 32, "node layout is 32 bytes");

struct tri48
{
  v3 p0, e0, e1, n;
};

static_assert(sizeof(tri48) == 48, "triangle layout is 48 bytes");

constexpr uint32_t kLeafBit = 0x80000000u; // highest_bit<u32>, lbvh.h:170-175
constexpr float kInf = std::numeric_limits<float>::infinity();

// std::min / std::max as the vector min/max use them (lbvh.h:638-660):
// std::min(a,b) = (b < a) ? b : a ; std::max(a,b) = (a < b) ? b : a.
inline float
smin(float a, float b)
{
  return (b < a) ? b : a;
}
inline float
smax(float a, float b)
{
  return (a < b) ? b : a;
}
// math::min / math::max ternaries (lbvh.h:567-580).
inline float
mmin(float a, float b)
{
  return (a < b) ? a : b;
}
inline float
mmax(float a, float b)
{
  return (a > b) ? a : b;
}

inline v3
vsub(v3 a, v3 b)
{
  return v3{ a.x - b.x, a.y - b.y, a.z - b.z };
}
inline v3
vadd(v3 a, v3 b)
{
  return v3{ a.x + b.x, a.y + b.y, a.z + b.z };
}
inline v3
vmin(v3 a, v3 b)
{
  return v3{ smin(a.x, b.x), smin(a.y, b.y), smin(a.z, b.z) };
}
inline v3
vmax(v3 a, v3 b)
{
  return v3{ smax(a.x, b.x), smax(a.y, b.y), smax(a.z, b.z) };
}
// cross, lbvh.h:609-616
inline v3
cross(v3 a, v3 b)
{
  return v3{ (a.y * b.z) - (a.z * b.y),
             (a.z * b.x) - (a.x * b.z),
             (a.x * b.y) - (a.y * b.x) };
}
// dot accumulates from 0 in x, y, z order, lbvh.h:621-630
inline float
dot(v3 a, v3 b)
{
  float out = 0;
  out += a.x * b.x;
  out += a.y * b.y;
  out += a.z * b.z;
  return out;
}

inline box3
empty_box()
{
  return box3{ { kInf, kInf, kInf }, { -kInf, -kInf, -kInf } };
}
// union_of(box, box), lbvh.h:1208-1211
inline box3
join(const box3& a, const box3& b)
{
  return box3{ vmin(a.lo, b.lo), vmax(a.hi, b.hi) };
}
// union_of(box, point), lbvh.h:1218-1223
inline box3
join(const box3& a, v3 p)
{
  return box3{ vmin(a.lo, p), vmax(a.hi, p) };
}
// center_of, lbvh.h:1160-1167
inline v3
center(const box3& b)
{
  v3 s = vadd(b.lo, b.hi);
  return v3{ s.x * 0.5f, s.y * 0.5f, s.z * 0.5f };
}

// triangle_aabb_converter, lbvh.h:2001-2012
inline box3
tri_box(const tri48& t)
{
  const v3 p1 = vsub(t.p0, t.e0);
  const v3 p2 = vadd(t.p0, t.e1);
  const v3 mn = vmin(t.p0, p1);
  const v3 mx = vmax(t.p0, p1);
  return box3{ vmin(mn, p2), vmax(mx, p2) };
}

// loop_range, lbvh.h:961-986
inline void
chunk(size_t idx, size_t count, size_t n, size_t& b, size_t& e)
{
  size_t c = n / count;
  b = c * idx;
  e = (idx + 1 == count) ? n : b + c;
}

// naive_thread_scheduler::operator(), lbvh.h:123-146
template<typename F>
void
run_threads(size_t threads, F&& f)
{
  if (threads == 0)
    threads = 1;
  std::vector<std::thread> th;
  for (size_t i = 0; i + 1 < threads; i++)
    th.emplace_back(f, i, threads);
  f(threads - 1, threads);
  for (auto& t : th)
    t.join();
}

// morton_encoder<4>::expand, lbvh.h:1351-1359
inline uint32_t
expand10(uint32_t n)
{
  n = (n | (n << 16)) & 0x030000ffu;
  n = (n | (n << 8)) & 0x0300f00fu;
  n = (n | (n << 4)) & 0x030c30c3u;
  n = (n | (n << 2)) & 0x09249249u;
  return n;
}

template<typename Conv>
box3
centroid_bounds(size_t n, size_t threads, Conv conv)
{
  // centroid_bounds_kernel per thread chunk, then a serial union in thread
  // order (lbvh.h:1282-1293, 1532-1543).
  if (threads == 0)
    threads = 1;
  std::vector<box3> tb(threads);
  run_threads(threads, [&](size_t idx, size_t cnt) {
    size_t b, e;
    chunk(idx, cnt, n, b, e);
    box3 acc = empty_box();
    for (size_t i = b; i < e; i++)
      acc = join(acc, center(conv(i)));
    tb[idx] = acc;
  });
  box3 cb = empty_box();
  for (const auto& b : tb)
    cb = join(cb, b);
  return cb;
}

template<typename Conv>
void
morton_codes(size_t n, size_t threads, const box3& cb, Conv conv, uint32_t* codes)
{
  // morton_curve_kernel, lbvh.h:1422-1475: scale = 1024 / (size + 1),
  // q = u32((c - min) * scale), code = x<<2 | y<<1 | z.
  const v3 size = vsub(cb.hi, cb.lo);
  const float dom = float(uint32_t(1024));
  const v3 scale{ dom / (size.x + 1.0f), dom / (size.y + 1.0f), dom / (size.z + 1.0f) };
  run_threads(threads, [&](size_t idx, size_t cnt) {
    size_t b, e;
    chunk(idx, cnt, n, b, e);
    for (size_t i = b; i < e; i++) {
      const v3 c = center(conv(i));
      const float fx = (c.x - cb.lo.x) * scale.x;
      const float fy = (c.y - cb.lo.y) * scale.y;
      const float fz = (c.z - cb.lo.z) * scale.z;
      const uint32_t x = uint32_t(fx), y = uint32_t(fy), z = uint32_t(fz);
      codes[i] = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
    }
  });
}

// divide_node's delta operator, lbvh.h:1602-1621: -1 out of range; equal codes
// fall back to clz(j ^ k) + 32.
inline int
delta(const uint32_t* codes, int64_t n, int64_t j, int64_t k)
{
  if (k < 0 || k >= n)
    return -1;
  const uint32_t a = codes[j], b = codes[k];
  if (a == b)
    return __builtin_clz(uint32_t(j ^ k)) + 32;
  return __builtin_clz(a ^ b);
}

// divide_node + builder_kernel body for one internal node, lbvh.h:1588-1731.
inline void
split_node(const uint32_t* codes, int64_t n, int64_t i, uint32_t& left, uint32_t& right)
{
  const int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) < 0 ? -1 : 1;
  const int dmin = delta(codes, n, i, i - d);
  int64_t lmax = 128;
  for (;;) {
    const int64_t k = i + lmax * d;
    if (k >= n)
      break;
    if (!(delta(codes, n, i, k) > dmin))
      break;
    lmax *= 4;
  }
  int64_t l = 0;
  for (int64_t div = 2;; div *= 2) {
    const int64_t t = lmax / div;
    if (delta(codes, n, i, i + (l + t) * d) > dmin)
      l += t;
    if (t == 1)
      break;
  }
  const int64_t j = i + l * d;
  const int dnode = delta(codes, n, i, j);
  int64_t s = 0;
  for (int64_t div = 2;; div *= 2) {
    const int64_t t = (l + (div - 1)) / div;
    if (delta(codes, n, i, i + (s + t) * d) > dnode)
      s += t;
    if (div >= l)
      break;
  }
  const int64_t gamma = i + s * d + (d < 0 ? d : 0);
  const int64_t lo = i < j ? i : j;
  const int64_t hi = j > i ? j : i;
  left = uint32_t(gamma) | (lo == gamma ? kLeafBit : 0u);
  right = uint32_t(gamma + 1) | (hi == gamma + 1 ? kLeafBit : 0u);
}

// builder::fit_boxes, lbvh.h:1826-1867: BFS list from the root, then a
// reverse sweep; box = left (leaf converter or child box), then union with
// the right.
template<typename Conv>
void
fit_boxes(node32* nodes, size_t nn, Conv conv)
{
  std::vector<uint32_t> order;
  order.reserve(nn);
  order.push_back(0);
  for (size_t i = 0; i < order.size(); i++) {
    const node32& nd = nodes[order[i]];
    if (!(nd.left & kLeafBit))
      order.push_back(nd.left);
    if (!(nd.right & kLeafBit))
      order.push_back(nd.right);
  }
  for (size_t i = order.size(); i > 0; i--) {
    node32& nd = nodes[order[i - 1]];
    box3 b = (nd.left & kLeafBit) ? conv(nd.left & ~kLeafBit) : nodes[nd.left].box;
    b = join(b, (nd.right & kLeafBit) ? conv(nd.right & ~kLeafBit) : nodes[nd.right].box);
    nd.box = b;
  }
}

template<typename Conv>
void
build(size_t n, size_t threads, Conv conv, node32* out_nodes)
{
  // builder::operator(), lbvh.h:1793-1822.
  const box3 cb = centroid_bounds(n, threads, conv);
  std::vector<uint32_t> codes(n);
  morton_codes(n, threads, cb, conv, codes.data());
  // Only the sorted code sequence reaches the output (leaf slot p holds
  // primitive p), so sorting the codes alone matches the reference.
  std::sort(codes.begin(), codes.end());
  const int64_t nn = int64_t(n) - 1;
  run_threads(threads, [&](size_t idx, size_t cnt) {
    size_t b, e;
    chunk(idx, cnt, size_t(nn), b, e);
    for (size_t i = b; i < e; i++) {
      uint32_t l, r;
      split_node(codes.data(), int64_t(n), int64_t(i), l, r);
      out_nodes[i].left = l;
      out_nodes[i].right = r;
      out_nodes[i].box = box3{ { 0, 0, 0 }, { 0, 0, 0 } };
    }
  });
  fit_boxes(out_nodes, size_t(nn), conv);
}

// ---- traversal -----------------------------------------------------------

struct hit16
{
  uint32_t prim;
  float t, u, v;
};

struct accel
{
  v3 pos, dir, rcp, inv_pos;
  int oct[3], ioct[3];
};

// make_accel_ray, lbvh.h:991-1010
inline accel
make_accel(v3 pos, v3 dir)
{
  accel a;
  a.pos = pos;
  a.dir = dir;
  a.rcp = v3{ 1 / dir.x, 1 / dir.y, 1 / dir.z };
  a.inv_pos = v3{ (-pos.x) * a.rcp.x, (-pos.y) * a.rcp.y, (-pos.z) * a.rcp.z };
  a.oct[0] = dir.x > 0 ? 0 : 3;
  a.oct[1] = dir.y > 0 ? 1 : 4;
  a.oct[2] = dir.z > 0 ? 2 : 5;
  a.ioct[0] = 3 - a.oct[0];
  a.ioct[1] = 5 - a.oct[1];
  a.ioct[2] = 7 - a.oct[2];
  return a;
}

// detail::intersect, octant form (lbvh.h:1071-1091); the hit test is
// box_intersection::operator bool (lbvh.h:1026-1029).
inline bool
box_hit(const box3& b, const accel& a, float& tmin_out)
{
  const float bd[6] = { b.lo.x, b.lo.y, b.lo.z, b.hi.x, b.hi.y, b.hi.z };
  const float tn0 = (bd[a.oct[0]] * a.rcp.x) + a.inv_pos.x;
  const float tn1 = (bd[a.oct[1]] * a.rcp.y) + a.inv_pos.y;
  const float tn2 = (bd[a.oct[2]] * a.rcp.z) + a.inv_pos.z;
  const float tf0 = (bd[a.ioct[0]] * a.rcp.x) + a.inv_pos.x;
  const float tf1 = (bd[a.ioct[1]] * a.rcp.y) + a.inv_pos.y;
  const float tf2 = (bd[a.ioct[2]] * a.rcp.z) + a.inv_pos.z;
  const float tmin = mmax(mmax(tn0, tn1), tn2);
  const float tmax = mmin(mmin(tf0, tf1), tf2);
  tmin_out = tmin;
  return tmax >= mmax(0.0f, tmin);
}

// triangle_intersector::operator(), lbvh.h:2055-2075
inline bool
tri_hit(const tri48& tri, v3 pos, v3 dir, float rtmin, float rtmax, float& t, float& u, float& v)
{
  const v3 c = vsub(tri.p0, pos);
  const v3 r = cross(dir, c);
  const float inv_det = 1 / dot(tri.n, dir);
  u = dot(r, tri.e1) * inv_det;
  v = dot(r, tri.e0) * inv_det;
  const float w = 1.0f - u - v;
  if ((u >= 0) && (v >= 0) && (w >= 0)) {
    t = dot(tri.n, c) * inv_det;
    if ((t >= rtmin) && (t <= rtmax))
      return true;
  }
  return false;
}

// traverser::operator(), lbvh.h:1874-1942, with a 128-entry stack that drops
// pushes when full (lbvh.h:1746-1789).
inline hit16
trace_one(const node32* nodes,
          const tri48* tris,
          const float* ray,
          uint32_t* n_box,
          uint32_t* n_tri)
{
  struct ent
  {
    uint32_t node;
    float tmin;
  };
  ent stack[128];
  size_t sp = 0;
  stack[sp++] = ent{ 0, kInf };
  const v3 pos{ ray[0], ray[1], ray[2] };
  const v3 dir{ ray[3], ray[4], ray[5] };
  const float rtmin = ray[6], rtmax = ray[7];
  const accel a = make_accel(pos, dir);
  hit16 best{ 0xffffffffu, kInf, 0.0f, 0.0f };
  uint32_t cb = 0, ct = 0;
  while (sp) {
    const ent e = stack[--sp];
    if (best.t < e.tmin)
      continue;
    const node32& nd = nodes[e.node];
    bool lhit = false, rhit = false;
    float lt = kInf, rt = kInf;
    if (nd.left & kLeafBit) {
      const uint32_t p = nd.left & ~kLeafBit;
      float t, u, v;
      ct++;
      if (tri_hit(tris[p], pos, dir, rtmin, rtmax, t, u, v) && t < best.t)
        best = hit16{ p, t, u, v };
    } else {
      cb++;
      lhit = box_hit(nodes[nd.left].box, a, lt);
    }
    if (nd.right & kLeafBit) {
      const uint32_t p = nd.right & ~kLeafBit;
      float t, u, v;
      ct++;
      if (tri_hit(tris[p], pos, dir, rtmin, rtmax, t, u, v) && t < best.t)
        best = hit16{ p, t, u, v };
    } else {
      cb++;
      rhit = box_hit(nodes[nd.right].box, a, rt);
    }
    if (lhit && rhit) {
      if (lt < rt) {
        if (sp < 128)
          stack[sp++] = ent{ nd.right, rt };
        if (sp < 128)
          stack[sp++] = ent{ nd.left, lt };
      } else {
        if (sp < 128)
          stack[sp++] = ent{ nd.left, lt };
        if (sp < 128)
          stack[sp++] = ent{ nd.right, rt };
      }
    } else if (lhit) {
      if (sp < 128)
        stack[sp++] = ent{ nd.left, lt };
    } else if (rhit) {
      if (sp < 128)
        stack[sp++] = ent{ nd.right, rt };
    }
  }
  if (n_box)
    *n_box = cb;
  if (n_tri)
    *n_tri = ct;
  return best;
}

} // namespace

// ---------------------------------------------------------------------------
// User primitive: the sphere of the reference's example program
// (examples/minimal.cpp:16-42, {radius, pos}) with its intersector
// (examples/minimal.cpp:92-135), traced by traverser::operator()
// (lbvh.h:1874-1942) with that intersector swapped in.

struct sphere16
{
  float radius;
  float pos[3];
};
static_assert(sizeof(sphere16) == 16, "sphere layout is 16 bytes");

struct sphere_hit32
{
  uint32_t prim;
  float t, u, v;
  float n[3];
  float pad;
};
static_assert(sizeof(sphere_hit32) == 32, "sphere hit layout is 32 bytes");

// normalize, lbvh.h:724-734: v * (1 / sqrt(dot(v, v)))
inline v3
normalize(v3 v)
{
  const float l_inv = 1.0f / std::sqrt(dot(v, v));
  return v3{ v.x * l_inv, v.y * l_inv, v.z * l_inv };
}

// The example's intersector: t = +inf when the ray's line misses; otherwise
// the root (-b + sqrt(disc)) / 2a unless it is negative, then the other one.
inline sphere_hit32
sphere_hit(const sphere16& s, v3 pos, v3 dir)
{
  sphere_hit32 h{ 0xffffffffu, kInf, 0.0f, 0.0f, { 0.0f, 0.0f, 0.0f }, 0.0f };
  const v3 sp{ s.pos[0], s.pos[1], s.pos[2] };
  const v3 dist = vsub(pos, sp);
  const float a = dot(dir, dir);
  const float b = 2 * dot(dir, dist);
  const float c = dot(dist, dist) - (s.radius * s.radius);
  const float disc = (b * b) - (4 * a * c);
  if (disc < 0)
    return h;
  const float t0 = (-b + std::sqrt(disc)) / (2 * a);
  const float t1 = (-b - std::sqrt(disc)) / (2 * a);
  float t = t0;
  if (t < 0)
    t = t1;
  const v3 hit{ pos.x + (dir.x * t), pos.y + (dir.y * t), pos.z + (dir.z * t) };
  const v3 n = normalize(vsub(hit, sp));
  const float pi = float(M_PI);
  h.t = t;
  h.u = (1.0f + std::atan2(n.z, n.x) / pi) * 0.5f;
  h.v = std::acos(n.y) / pi;
  h.n[0] = n.x;
  h.n[1] = n.y;
  h.n[2] = n.z;
  return h;
}

inline sphere_hit32
trace_sphere_one(const node32* nodes, const sphere16* spheres, const float* ray)
{
  struct ent
  {
    uint32_t node;
    float tmin;
  };
  ent stack[128];
  size_t sp = 0;
  stack[sp++] = ent{ 0, kInf };
  const v3 pos{ ray[0], ray[1], ray[2] };
  const v3 dir{ ray[3], ray[4], ray[5] };
  const accel a = make_accel(pos, dir);
  sphere_hit32 best{ 0xffffffffu, kInf, 0.0f, 0.0f, { 0.0f, 0.0f, 0.0f }, 0.0f };
  while (sp) {
    const ent e = stack[--sp];
    if (best.t < e.tmin)
      continue;
    const node32& nd = nodes[e.node];
    bool lhit = false, rhit = false;
    float lt = kInf, rt = kInf;
    if (nd.left & kLeafBit) {
      const uint32_t p = nd.left & ~kLeafBit;
      sphere_hit32 h = sphere_hit(spheres[p], pos, dir);
      if (h.t < best.t) {
        h.prim = p;
        best = h;
      }
    } else {
      lhit = box_hit(nodes[nd.left].box, a, lt);
    }
    if (nd.right & kLeafBit) {
      const uint32_t p = nd.right & ~kLeafBit;
      sphere_hit32 h = sphere_hit(spheres[p], pos, dir);
      if (h.t < best.t) {
        h.prim = p;
        best = h;
      }
    } else {
      rhit = box_hit(nodes[nd.right].box, a, rt);
    }
    if (lhit && rhit) {
      if (lt < rt) {
        if (sp < 128)
          stack[sp++] = ent{ nd.right, rt };
        if (sp < 128)
          stack[sp++] = ent{ nd.left, lt };
      } else {
        if (sp < 128)
          stack[sp++] = ent{ nd.left, lt };
        if (sp < 128)
          stack[sp++] = ent{ nd.right, rt };
      }
    } else if (lhit) {
      if (sp < 128)
        stack[sp++] = ent{ nd.left, lt };
    } else if (rhit) {
      if (sp < 128)
        stack[sp++] = ent{ nd.right, rt };
    }
  }
  return best;
}

extern "C" {

// triangle<float>(a, b, c), lbvh.h:1967-1972: e0 = a - b, e1 = c - a,
// normal = cross(e0, e1). verts: n x 9 floats; out: n x 12 floats.
void
orc_make_triangles(const float* verts, size_t n, float* out_tris)
{
  for (size_t i = 0; i < n; i++) {
    const float* p = verts + i * 9;
    const v3 a{ p[0], p[1], p[2] }, b{ p[3], p[4], p[5] }, c{ p[6], p[7], p[8] };
    tri48 t;
    t.p0 = a;
    t.e0 = vsub(a, b);
    t.e1 = vsub(c, a);
    t.n = cross(t.e0, t.e1);
    std::memcpy(out_tris + i * 12, &t, sizeof(t));
  }
}

void
orc_tri_boxes(const float* tris, size_t n, float* out_boxes)
{
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  for (size_t i = 0; i < n; i++) {
    box3 b = tri_box(t[i]);
    std::memcpy(out_boxes + i * 6, &b, sizeof(b));
  }
}

void
orc_centroid_bounds(const float* tris, size_t n, size_t threads, float* out6)
{
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  box3 cb = centroid_bounds(n, threads, [t](size_t i) { return tri_box(t[i]); });
  std::memcpy(out6, &cb, sizeof(cb));
}

// Morton codes in input order, the sorted code sequence, and the stable
// (ascending original index on ties) sort permutation.
void
orc_curve(const float* tris,
          size_t n,
          size_t threads,
          uint32_t* out_codes,
          uint32_t* out_sorted_codes,
          uint32_t* out_stable_perm)
{
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  auto conv = [t](size_t i) { return tri_box(t[i]); };
  const box3 cb = centroid_bounds(n, threads, conv);
  std::vector<uint32_t> codes(n);
  morton_codes(n, threads, cb, conv, codes.data());
  if (out_codes)
    std::memcpy(out_codes, codes.data(), n * 4);
  std::vector<uint32_t> perm(n);
  for (size_t i = 0; i < n; i++)
    perm[i] = uint32_t(i);
  std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
    return codes[a] < codes[b];
  });
  for (size_t i = 0; i < n; i++) {
    if (out_sorted_codes)
      out_sorted_codes[i] = codes[perm[i]];
    if (out_stable_perm)
      out_stable_perm[i] = perm[i];
  }
}

int
orc_build(const float* tris, size_t n, size_t threads, void* out_nodes)
{
  if (n < 2)
    return 1;
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  build(n, threads, [t](size_t i) { return tri_box(t[i]); }, static_cast<node32*>(out_nodes));
  return 0;
}

// Build over caller boxes (6 floats each) with an identity converter, the
// user-converter form of builder::operator().
int
orc_build_boxes(const float* boxes, size_t n, size_t threads, void* out_nodes)
{
  if (n < 2)
    return 1;
  const box3* b = reinterpret_cast<const box3*>(boxes);
  build(n, threads, [b](size_t i) { return b[i]; }, static_cast<node32*>(out_nodes));
  return 0;
}

// Splits only (node left/right from a given sorted code sequence).
void
orc_split(const uint32_t* sorted_codes, size_t n, uint32_t* out_lr)
{
  for (size_t i = 0; i + 1 < n; i++)
    split_node(sorted_codes, int64_t(n), int64_t(i), out_lr[2 * i], out_lr[2 * i + 1]);
}

// Refit: recompute every node box over the existing topology with the
// fit_boxes order (lbvh.h:1826-1867); left/right are kept.
int
orc_refit(void* nodes, size_t n_nodes, const float* tris)
{
  if (n_nodes < 1)
    return 1;
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  fit_boxes(static_cast<node32*>(nodes), n_nodes, [t](size_t i) { return tri_box(t[i]); });
  return 0;
}

// Closest-hit trace of m rays (8 floats: pos, dir, tmin, tmax); hits are 16
// bytes {prim, t, u, v}; misses are {UINT32_MAX, +inf, 0, 0}. Rays are
// interleaved across threads as lbvh_test.cpp:154-175 does. n_box / n_tri
// (optional) receive per-ray box-test and triangle-test counts.
void
orc_trace(const void* nodes,
          const float* tris,
          const float* rays,
          size_t m,
          size_t threads,
          void* out_hits,
          uint32_t* n_box,
          uint32_t* n_tri)
{
  const node32* nd = static_cast<const node32*>(nodes);
  const tri48* t = reinterpret_cast<const tri48*>(tris);
  hit16* h = static_cast<hit16*>(out_hits);
  run_threads(threads, [&](size_t idx, size_t cnt) {
    for (size_t i = idx; i < m; i += cnt)
      h[i] = trace_one(nd, t, rays + 8 * i, n_box ? n_box + i : nullptr, n_tri ? n_tri + i : nullptr);
  });
}

// Closest sphere hit of m rays (8 floats) over a tree built from the
// spheres' boxes; hits are 32 bytes {prim, t, u, v, normal, pad}, misses
// {UINT32_MAX, +inf, 0, 0, 0, 0, 0}.
void
orc_trace_spheres(const void* nodes, const float* spheres, const float* rays, size_t m, size_t threads, void* out_hits)
{
  const node32* nd = static_cast<const node32*>(nodes);
  const sphere16* sph = reinterpret_cast<const sphere16*>(spheres);
  sphere_hit32* h = static_cast<sphere_hit32*>(out_hits);
  run_threads(threads, [&](size_t idx, size_t cnt) {
    for (size_t i = idx; i < m; i += cnt)
      h[i] = trace_sphere_one(nd, sph, rays + 8 * i);
  });
}

// check_bvh (lbvh_test.cpp:369-446): root unreferenced, every other internal
// node referenced once, every leaf in [0, n_nodes] referenced once. Then
// check_volumes (lbvh_test.cpp:458-518): no child volume above its parent's.
// Returns the number of violations found (0 = valid).
long
orc_check_bvh(const void* nodes, size_t n_nodes)
{
  const node32* nd = static_cast<const node32*>(nodes);
  long errors = 0;
  std::vector<uint32_t> nc(n_nodes, 0), lc(n_nodes + 1, 0);
  for (size_t i = 0; i < n_nodes; i++) {
    const uint32_t c[2] = { nd[i].left, nd[i].right };
    for (uint32_t x : c) {
      if (x & kLeafBit) {
        uint32_t p = x & ~kLeafBit;
        if (p > n_nodes)
          errors++;
        else
          lc[p]++;
      } else {
        if (x >= n_nodes)
          errors++;
        else
          nc[x]++;
      }
    }
  }
  if (n_nodes && nc[0] != 0)
    errors++;
  for (size_t i = 1; i < n_nodes; i++)
    errors += nc[i] != 1;
  for (size_t i = 0; i <= n_nodes; i++)
    errors += lc[i] != 1;
  if (errors)
    return errors;
  auto vol = [](const box3& b) {
    v3 s = vsub(b.hi, b.lo);
    return s.x * s.y * s.z;
  };
  std::vector<uint32_t> st{ 0 };
  while (!st.empty()) {
    uint32_t i = st.back();
    st.pop_back();
    const float pv = vol(nd[i].box);
    const uint32_t c[2] = { nd[i].left, nd[i].right };
    for (uint32_t x : c) {
      if (!(x & kLeafBit)) {
        if (pv < vol(nd[x].box))
          errors++;
        st.push_back(x);
      }
    }
  }
  return errors;
}

} // extern "C"
