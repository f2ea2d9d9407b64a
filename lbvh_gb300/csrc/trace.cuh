// Traversal launch parameters and launchers.
#pragma once

#include "common.cuh"

namespace lbvh_gb300 {

constexpr int kTraceThreads = 128;
constexpr uint32_t kStackSize = 128; // traversal_stack<scalar, 128>, lbvh.h:1874

// Launch shape of the persistent traversal kernel (set per context).
struct TraceParams
{
  uint32_t blocks_per_sm = 8; // resident 128-thread blocks per SM
  uint32_t refill = 12;       // idle lanes at which a warp takes new rays
  uint32_t leaf_batch = 1;    // lanes with pending triangle tests before a warp runs them (1: at once)
};

// Traversal copy of an internal node: both children's boxes plus the child
// references, 64 bytes.
//   a = {left lo.xyz, left hi.x}, b = {left hi.yz, right lo.xy},
//   c = {right lo.z, right hi.xyz}, d = {left, right, 0, 0}
struct __align__(16) WideNode
{
  float4 a, b, c, d;
};
static_assert(sizeof(WideNode) == 64, "wide node layout");

cudaError_t launch_repack(const Node* nodes, uint32_t n_nodes, WideNode* out, cudaStream_t s);

// wnodes holds n_nodes nodes followed by the scene-bound flag word.
cudaError_t launch_trace_tris(const WideNode* wnodes,
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
                              bool host_hits = false,         // hits: page-locked host memory
                              const uint32_t* order = nullptr); // device hits only: trace ray order[q] q-th

// Sort keys of m rays for a coherent trace order: the origin's cell (4 bits
// per axis of the root box, z-order) above the direction's cell (4 bits per
// axis of the direction scaled by its largest component), 24 bits; the key
// histograms of the sort's four 8-bit digits go to st->hist, which must be
// zero.
cudaError_t launch_ray_keys(const float* rays, uint32_t m, const Node* nodes, uint32_t* keys, BuildState* st,
                            cudaStream_t s);

// Hit record of the sphere intersector: {prim, t, uv, normal, pad}, 32 bytes.
struct __align__(16) SphereHit
{
  uint32_t prim;
  float t, u, v;
  float nx, ny, nz, pad;
};

// spheres: n x {radius, x, y, z}; leaf slot p is sphere p (parity leaf order).
cudaError_t launch_trace_spheres(const WideNode* wnodes,
                                 const float4* spheres,
                                 const float* rays,
                                 uint32_t m,
                                 SphereHit* hits,
                                 int num_sms,
                                 cudaStream_t s);

} // namespace lbvh_gb300
