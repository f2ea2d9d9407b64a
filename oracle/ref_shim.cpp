// Test infrastructure only: a thin extern "C" shim over the UNMODIFIED
// reference header `lbvh.h` (tay10r/lbvh), compiled from the reference's own
// source tree by oracle/Makefile into oracle/_ref/libref.so. It exists to pin
// the CPU restatement in oracle/lbvh_oracle.cpp and to generate the golden
// fixtures under tests/golden/. Nothing in the product links or loads it.
//
// Every function forwards to the reference's own templates:
//   build   -> lbvh::builder<float>::operator()          (lbvh.h:1793-1822)
//   curve   -> detail::morton_curve_builder::operator()  (lbvh.h:1520-1553)
//   bounds  -> detail::centroid_bounds_kernel + union    (lbvh.h:1282-1293,1532-1543)
//   sort    -> detail::space_filling_curve::sort         (lbvh.h:1126-1134)
//   trace   -> lbvh::traverser<...>::operator()          (lbvh.h:1869-1942)
//   spheres -> the same traverser with the example program's sphere type
//              and intersector (examples/minimal.cpp:16-42, 92-135), restated
//   triangle/ctor, converter, intersector                (lbvh.h:1959-2076)
//   OBJ load -> tinyobj::ObjReader as lbvh_test.cpp:602-649 uses it
//
// The reference's `triangle<float>` keeps its four vec3 members private; it is
// a standard-layout class of 12 floats {p0, e0, e1, normal}, so the shim moves
// it in and out with memcpy.

#include <lbvh.h>

#include "third-party/tiny_obj_loader.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace {

using tri_t = lbvh::triangle<float>;
using node_t = lbvh::node<float>;
using conv_t = lbvh::triangle_aabb_converter<float>;
using isect_t = lbvh::triangle_intersection<float>;

static_assert(sizeof(tri_t) == 48, "triangle<float> is 12 floats");
static_assert(sizeof(node_t) == 32, "node<float> is 32 bytes");

std::vector<tri_t>
load_tris(const float* tris, size_t n)
{
  std::vector<tri_t> v(n);
  if (n)
    std::memcpy(v.data(), tris, n * sizeof(tri_t));
  return v;
}

struct hit_out
{
  uint32_t prim;
  float t;
  float u;
  float v;
};

// The sphere and sphere_hit types of the reference's example program
// (examples/minimal.cpp:16-42), restated: a sphere is {radius, pos}; a hit
// orders by tmin, against another hit and against a distance.
struct sphere_t
{
  float radius;
  float pos[3];
};

struct sphere_hit_t
{
  float tmin = std::numeric_limits<float>::infinity();
  float uv[2]{ 0, 0 };
  float normal[3]{ 0, 0, 0 };
  bool operator<(const sphere_hit_t& other) const noexcept { return tmin < other.tmin; }
  bool operator<(float distance) const noexcept { return tmin < distance; }
};

struct sphere_hit_out
{
  uint32_t prim;
  float t, u, v;
  float n[3];
  float pad;
};

// The example's intersector (examples/minimal.cpp:92-135), restated in plain
// float operations in the example's order (the same order the port and the
// GPU kernel use): the quadratic's roots, the nearer unless negative, the
// normal as lbvh::math::normalize forms it, uv from atan2 and acos.
sphere_hit_t
intersect_sphere(const sphere_t& s, const lbvh::ray<float>& ray)
{
  const float ox = ray.pos.x - s.pos[0], oy = ray.pos.y - s.pos[1], oz = ray.pos.z - s.pos[2];
  const float dx = ray.dir.x, dy = ray.dir.y, dz = ray.dir.z;
  float dd = 0, dof = 0, oo = 0; // dot products accumulate from 0 in x, y, z order
  dd += dx * dx;
  dd += dy * dy;
  dd += dz * dz;
  dof += dx * ox;
  dof += dy * oy;
  dof += dz * oz;
  oo += ox * ox;
  oo += oy * oy;
  oo += oz * oz;
  const float qb = 2.0f * dof;
  const float qc = oo - s.radius * s.radius;
  const float disc = qb * qb - (4.0f * dd) * qc;
  sphere_hit_t h;
  if (disc < 0)
    return h;
  const float root = std::sqrt(disc);
  const float near = (-qb + root) / (2.0f * dd);
  const float other = (-qb - root) / (2.0f * dd);
  const float t = near < 0 ? other : near;
  const float vx = (ray.pos.x + dx * t) - s.pos[0];
  const float vy = (ray.pos.y + dy * t) - s.pos[1];
  const float vz = (ray.pos.z + dz * t) - s.pos[2];
  float vv = 0;
  vv += vx * vx;
  vv += vy * vy;
  vv += vz * vz;
  const float inv_len = 1.0f / std::sqrt(vv);
  const float nx = vx * inv_len, ny = vy * inv_len, nz = vz * inv_len;
  const float pi = float(M_PI);
  h.tmin = t;
  h.uv[0] = (1.0f + std::atan2(nz, nx) / pi) * 0.5f;
  h.uv[1] = std::acos(ny) / pi;
  h.normal[0] = nx;
  h.normal[1] = ny;
  h.normal[2] = nz;
  return h;
}

} // namespace

extern "C" {

// lbvh::triangle<float>(a, b, c) for n vertex triples (9 floats each).
void
ref_make_triangles(const float* verts, size_t n, float* out_tris)
{
  for (size_t i = 0; i < n; i++) {
    const float* p = verts + i * 9;
    lbvh::vec3<float> a{ p[0], p[1], p[2] };
    lbvh::vec3<float> b{ p[3], p[4], p[5] };
    lbvh::vec3<float> c{ p[6], p[7], p[8] };
    tri_t t(a, b, c);
    std::memcpy(out_tris + i * 12, &t, sizeof(tri_t));
  }
}

// lbvh::triangle_aabb_converter<float> for n triangles -> n boxes (6 floats).
void
ref_tri_boxes(const float* tris, size_t n, float* out_boxes)
{
  auto v = load_tris(tris, n);
  conv_t conv;
  for (size_t i = 0; i < n; i++) {
    auto b = conv(v[i]);
    std::memcpy(out_boxes + i * 6, &b, sizeof(b));
  }
}

// Full reference build: n triangles -> n-1 nodes (32 bytes each).
int
ref_build(const float* tris, size_t n, size_t threads, void* out_nodes)
{
  if (n < 2)
    return 1;
  auto v = load_tris(tris, n);
  lbvh::builder<float> builder{ lbvh::naive_thread_scheduler(threads) };
  auto bvh = builder(v.data(), n, conv_t());
  std::memcpy(out_nodes, &bvh[0], bvh.size() * sizeof(node_t));
  return 0;
}

// Same as ref_build, but the primitives are user boxes (6 floats each) and the
// converter is the identity, as examples/minimal.cpp's sphere_to_box lambda is.
int
ref_build_boxes(const float* boxes, size_t n, size_t threads, void* out_nodes)
{
  if (n < 2)
    return 1;
  std::vector<lbvh::aabb<float>> v(n);
  std::memcpy(v.data(), boxes, n * sizeof(lbvh::aabb<float>));
  lbvh::builder<float> builder{ lbvh::naive_thread_scheduler(threads) };
  auto bvh = builder(
    v.data(), n, [](const lbvh::aabb<float>& b) { return b; });
  std::memcpy(out_nodes, &bvh[0], bvh.size() * sizeof(node_t));
  return 0;
}

// Centroid bounds exactly as morton_curve_builder computes them.
void
ref_centroid_bounds(const float* tris, size_t n, size_t threads, float* out6)
{
  auto v = load_tris(tris, n);
  lbvh::naive_thread_scheduler sched(threads);
  conv_t conv;
  std::vector<lbvh::aabb<float>> thread_boxes(sched.max_threads());
  lbvh::detail::centroid_bounds_kernel<float, tri_t, conv_t> kern(
    v.data(), n, conv, thread_boxes.data());
  sched(kern);
  auto cb = lbvh::detail::get_empty_aabb<float>();
  for (const auto& b : thread_boxes)
    cb = lbvh::detail::union_of(cb, b);
  std::memcpy(out6, &cb, sizeof(cb));
}

// Morton curve: per-primitive codes in input order (entry.primitive == i),
// then the reference's own (unstable) sort, then std::stable_sort of the same
// entries for the stable permutation.
void
ref_curve(const float* tris,
          size_t n,
          size_t threads,
          uint32_t* out_codes,
          uint32_t* out_sorted_codes,
          uint32_t* out_stable_perm)
{
  auto v = load_tris(tris, n);
  lbvh::naive_thread_scheduler sched(threads);
  lbvh::detail::morton_curve_builder<float, lbvh::naive_thread_scheduler> cb(
    sched);
  auto curve = cb(v.data(), n, conv_t());
  using entry = decltype(curve)::entry;
  std::vector<entry> entries(n);
  for (size_t i = 0; i < n; i++) {
    entries[i] = curve[i];
    if (out_codes)
      out_codes[i] = curve[i].code;
  }
  curve.sort();
  if (out_sorted_codes)
    for (size_t i = 0; i < n; i++)
      out_sorted_codes[i] = curve[i].code;
  std::stable_sort(entries.begin(),
                   entries.end(),
                   [](const entry& a, const entry& b) { return a.code < b.code; });
  if (out_stable_perm)
    for (size_t i = 0; i < n; i++)
      out_stable_perm[i] = entries[i].primitive;
}

// Closest-hit traversal of m rays (8 floats each: pos, dir, tmin, tmax) with
// the reference traverser and triangle_intersector. Rays are split across
// `threads` threads with rows interleaved, as lbvh_test.cpp:154-175 does.
// Misses report prim = UINT32_MAX, t = +inf, u = v = 0.
void
ref_trace(const void* nodes,
          size_t n_nodes,
          const float* tris,
          size_t n_tris,
          const float* rays,
          size_t m,
          size_t threads,
          void* out_hits)
{
  std::vector<node_t> nv(n_nodes);
  std::memcpy(nv.data(), nodes, n_nodes * sizeof(node_t));
  lbvh::bvh<float> bvh(std::move(nv));
  auto v = load_tris(tris, n_tris);
  lbvh::traverser<float, tri_t, isect_t> trav(bvh, v.data());
  lbvh::triangle_intersector<float> isector;
  auto* hits = static_cast<hit_out*>(out_hits);
  auto work = [&](lbvh::work_division div) {
    for (size_t i = div.idx; i < m; i += div.max) {
      const float* r = rays + i * 8;
      lbvh::ray<float> ray{ { r[0], r[1], r[2] }, { r[3], r[4], r[5] }, r[6], r[7] };
      auto isect = trav(ray, isector);
      if (isect)
        hits[i] = hit_out{ isect.primitive,
                           isect.info.distance,
                           isect.info.uv.x,
                           isect.info.uv.y };
      else
        hits[i] = hit_out{ 0xffffffffu,
                           std::numeric_limits<float>::infinity(),
                           0.0f,
                           0.0f };
    }
  };
  lbvh::naive_thread_scheduler sched(threads);
  sched(work);
}

// traverser<float, sphere, sphere_hit>::operator() with the example's
// intersector over a node array built from the spheres' boxes.
void
ref_trace_spheres(const void* nodes,
                  size_t n_nodes,
                  const float* spheres,
                  size_t n_spheres,
                  const float* rays,
                  size_t m,
                  size_t threads,
                  void* out_hits)
{
  std::vector<node_t> nv(n_nodes);
  std::memcpy(nv.data(), nodes, n_nodes * sizeof(node_t));
  lbvh::bvh<float> bvh(std::move(nv));
  std::vector<sphere_t> sv(n_spheres);
  std::memcpy(sv.data(), spheres, n_spheres * sizeof(sphere_t));
  lbvh::traverser<float, sphere_t, sphere_hit_t> trav(bvh, sv.data());
  auto* hits = static_cast<sphere_hit_out*>(out_hits);
  auto work = [&](lbvh::work_division div) {
    for (size_t i = div.idx; i < m; i += div.max) {
      const float* r = rays + i * 8;
      lbvh::ray<float> ray{ { r[0], r[1], r[2] }, { r[3], r[4], r[5] }, r[6], r[7] };
      auto isect = trav(ray, intersect_sphere);
      sphere_hit_out o{ 0xffffffffu, std::numeric_limits<float>::infinity(), 0.0f, 0.0f, { 0, 0, 0 }, 0.0f };
      if (isect)
        o = sphere_hit_out{ isect.primitive,
                            isect.info.tmin,
                            isect.info.uv[0],
                            isect.info.uv[1],
                            { isect.info.normal[0], isect.info.normal[1], isect.info.normal[2] },
                            0.0f };
      hits[i] = o;
    }
  };
  lbvh::naive_thread_scheduler sched(threads);
  sched(work);
}

// Loads an OBJ with the reference's vendored tinyobj exactly as
// lbvh_test.cpp:602-649 does and returns up to `cap` reference triangles.
// Returns the triangle count, or -1 if the file cannot be parsed.
long
ref_load_obj(const char* path, float* out_tris, size_t cap)
{
  tinyobj::ObjReader reader;
  if (!reader.ParseFromFile(path))
    return -1;
  size_t count = 0;
  for (const auto& shape : reader.GetShapes())
    count += shape.mesh.indices.size() / 3;
  if (!out_tris)
    return long(count);
  const auto& attrib = reader.GetAttrib();
  size_t k = 0;
  for (const auto& shape : reader.GetShapes()) {
    for (size_t i = 0; i + 2 < shape.mesh.indices.size() && k < cap; i += 3) {
      const float* a = &attrib.vertices[shape.mesh.indices[i + 0].vertex_index * 3];
      const float* b = &attrib.vertices[shape.mesh.indices[i + 1].vertex_index * 3];
      const float* c = &attrib.vertices[shape.mesh.indices[i + 2].vertex_index * 3];
      tri_t t(lbvh::vec3<float>{ a[0], a[1], a[2] },
              lbvh::vec3<float>{ b[0], b[1], b[2] },
              lbvh::vec3<float>{ c[0], c[1], c[2] });
      std::memcpy(out_tris + k * 12, &t, sizeof(tri_t));
      k++;
    }
  }
  return long(k);
}

} // extern "C"
