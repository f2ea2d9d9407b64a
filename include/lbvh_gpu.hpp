// lbvh_gpu.hpp -- GB300 drop-ins for tay10r/lbvh's builder and traverser.
//
// Include after the reference header `lbvh.h` (it must be on the include
// path) and link liblbvh_gb300.so. Code written against the reference keeps
// its types -- lbvh::triangle<float>, lbvh::aabb<float>, lbvh::bvh<float>,
// lbvh::ray<float>, lbvh::triangle_intersection<float> -- and swaps two names:
//
//   lbvh::builder<float>                 -> lbvh::gpu::builder<float>
//   lbvh::traverser<float, triangle<float>, triangle_intersection<float>>
//                                        -> lbvh::gpu::traverser<...same...>
//
// The node array a gpu::builder returns is bit-identical to the reference
// builder's for the same input (lbvh.h:1793-1822), and gpu::traverser returns
// the same closest hits as the reference traverser (lbvh.h:1869-1942). Errors
// are reported as lbvh::gpu::error exceptions (the reference has no error
// path: everything there is noexcept and n < 2 is undefined behaviour).
#pragma once

#include "lbvh_gb300.h"

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace lbvh {
namespace gpu {

//! A failed call into the GPU library.
class error : public std::runtime_error
{
public:
  error(int status, const std::string& what)
    : std::runtime_error(what)
    , status_(status)
  {}
  int status() const noexcept { return status_; }

private:
  int status_;
};

//! A device, a CUDA stream and the build workspace (lbvh_ctx). One per host
//! thread; the reference's builder owns a CPU scheduler in its place
//! (lbvh.h:312-327).
class context final
{
public:
  explicit context(int device = 0, void* cuda_stream = nullptr)
  {
    const int st = lbvh_ctx_create(device, cuda_stream, &ctx_);
    if (st != LBVH_OK)
      throw error(st, std::string("lbvh_ctx_create: ") + lbvh_status_string(st));
  }
  ~context() { lbvh_ctx_destroy(ctx_); }
  context(const context&) = delete;
  context& operator=(const context&) = delete;

  lbvh_ctx* get() const noexcept { return ctx_; }

  //! Throws for a non-OK status, with the context's last message.
  void check(int status, const char* what) const
  {
    if (status != LBVH_OK)
      throw error(status, std::string(what) + ": " + lbvh_status_string(status) + " (" +
                            lbvh_ctx_last_error(ctx_) + ")");
  }

  void synchronize() const { check(lbvh_ctx_synchronize(ctx_), "lbvh_ctx_synchronize"); }

private:
  lbvh_ctx* ctx_ = nullptr;
};

//! The calling thread's context on device 0 and the default stream.
inline context&
default_context()
{
  thread_local context ctx(0, nullptr);
  return ctx;
}

namespace detail {

//! An owned lbvh_bvh handle.
class device_bvh final
{
public:
  explicit device_bvh(context& ctx)
    : ctx_(&ctx)
  {
    ctx.check(lbvh_bvh_create(ctx.get(), &h_), "lbvh_bvh_create");
  }
  ~device_bvh() { lbvh_bvh_destroy(ctx_->get(), h_); }
  device_bvh(const device_bvh&) = delete;
  device_bvh& operator=(const device_bvh&) = delete;
  lbvh_bvh* get() const noexcept { return h_; }

private:
  context* ctx_;
  lbvh_bvh* h_ = nullptr;
};

static_assert(sizeof(triangle<float>) == 48, "triangle<float> is {p0, e0, e1, normal}");
static_assert(sizeof(aabb<float>) == 24, "aabb<float> is {min, max}");
static_assert(sizeof(node<float>) == 32, "node<float> is 32 bytes");
static_assert(sizeof(ray<float>) == 32, "ray<float> is {pos, dir, tmin, tmax}");
static_assert(sizeof(lbvh_node) == sizeof(node<float>), "node layout");

//! Copies the device node array into a reference bvh<float>.
inline bvh<float>
download(context& ctx, const device_bvh& d, size_t count)
{
  std::vector<node<float>> nodes(count - 1);
  ctx.check(lbvh_bvh_nodes(ctx.get(), d.get(), nodes.data()), "lbvh_bvh_nodes");
  return bvh<float>(std::move(nodes));
}

} // namespace detail

//! lbvh::builder on the GPU. builder<float>()(prims, count, converter)
//! returns the same bvh<float> as lbvh::builder<float> (lbvh.h:329-345).
//! With triangle<float> + triangle_aabb_converter<float> the whole build runs
//! on the GPU; any other primitive/converter pair converts on the host (the
//! converter is arbitrary C++) and builds the boxes on the GPU.
template<typename scalar_type>
class builder;

template<>
class builder<float> final
{
public:
  using bvh_type = bvh<float>;

  //! flags: 0 (reference parity) or LBVH_BUILD_SORTED_LEAVES.
  explicit builder(context& ctx = default_context(), uint32_t flags = 0)
    : ctx_(&ctx)
    , flags_(flags)
  {}

  template<typename primitive, typename aabb_converter>
  bvh_type operator()(const primitive* primitives, size_type count, const aabb_converter& converter)
  {
    if (count < 2)
      throw error(LBVH_ERR_INVALID_ARG, "lbvh::gpu::builder needs at least 2 primitives");
    detail::device_bvh d(*ctx_);
    if constexpr (std::is_same<primitive, triangle<float>>::value &&
                  std::is_same<aabb_converter, triangle_aabb_converter<float>>::value) {
      ctx_->check(lbvh_build_triangles(ctx_->get(), reinterpret_cast<const float*>(primitives), count, flags_,
                                       d.get()),
                  "lbvh_build_triangles");
    } else {
      std::vector<aabb<float>> boxes(count);
      for (size_type i = 0; i < count; i++)
        boxes[i] = converter(primitives[i]);
      ctx_->check(lbvh_build_boxes(ctx_->get(), reinterpret_cast<const float*>(boxes.data()), count, flags_,
                                   d.get()),
                  "lbvh_build_boxes");
    }
    return detail::download(*ctx_, d, count);
  }

private:
  context* ctx_;
  uint32_t flags_;
};

//! lbvh::traverser on the GPU for triangles with triangle_intersector<float>.
//! Construction uploads the tree and the triangles once (checking the tree);
//! operator() traces one ray like the reference (one GPU round trip), trace()
//! traces a batch.
template<typename scalar_type, typename primitive_type, typename intersection_info>
class traverser;

template<>
class traverser<float, triangle<float>, triangle_intersection<float>> final
{
public:
  using intersection = intersection_container<float, triangle_intersection<float>>;
  using ray_type = ray<float>;

  traverser(const bvh<float>& b, const triangle<float>* p, context& ctx = default_context())
    : ctx_(&ctx)
    , d_(new detail::device_bvh(ctx))
  {
    if (b.size() < 1)
      throw error(LBVH_ERR_INVALID_ARG, "lbvh::gpu::traverser needs a built BVH");
    ctx.check(lbvh_bvh_import_triangles(ctx.get(), &b[0], b.size(), reinterpret_cast<const float*>(p), d_->get()),
              "lbvh_bvh_import_triangles");
  }

  //! traverser::operator()(ray, triangle_intersector<float>), lbvh.h:1869-1942.
  template<typename intersector_type>
  intersection operator()(const ray_type& r, const intersector_type&) const
  {
    static_assert(std::is_same<intersector_type, triangle_intersector<float>>::value,
                  "the GPU traverser implements triangle_intersector<float>");
    intersection out;
    trace(&r, 1, &out);
    return out;
  }

  //! m rays -> m closest hits (misses: primitive = UINT32_MAX).
  void trace(const ray_type* rays, size_type m, intersection* out) const
  {
    std::vector<lbvh_hit> hits(m);
    ctx_->check(lbvh_trace_triangles(ctx_->get(), d_->get(), reinterpret_cast<const float*>(rays), m, hits.data()),
                "lbvh_trace_triangles");
    for (size_type i = 0; i < m; i++) {
      out[i] = intersection();
      if (hits[i].prim != LBVH_MISS) {
        out[i].primitive = hits[i].prim;
        out[i].info.distance = hits[i].t;
        out[i].info.uv.x = hits[i].u;
        out[i].info.uv.y = hits[i].v;
      }
    }
  }

private:
  context* ctx_;
  std::shared_ptr<detail::device_bvh> d_;
};

} // namespace gpu
} // namespace lbvh
