// Batched build + trace of many independent meshes.
#pragma once

#include "build.cuh"
#include "trace.cuh"

namespace lbvh_gb300 {

constexpr int kBatchMaxThreads = 1024; // largest CTA of the batched build

// Device views for one batched build of n_meshes meshes, total triangles.
// Mesh m owns triangles [off[m], off[m + 1]) and nodes
// [off[m] - m, off[m + 1] - m - 1): its node block is exactly the node array
// the reference builds for that mesh alone (local child indices).
struct BatchBuffers
{
  const uint32_t* off;        // n_meshes + 1 triangle offsets
  uint32_t n_meshes;
  uint32_t total;             // off[n_meshes]: all triangles
  uint32_t* queue;            // mesh dispenser (zeroed before the launch)
  uint32_t* keys_a;           // total
  uint32_t* keys_b;           // total
  Box* boxes;                 // total leaf boxes
  uint32_t* slots;            // total arrival slots (cleared per mesh)
  uint32_t* error;            // sticky kErr* bits
  // sorted-leaf mode only (nullptr otherwise):
  uint32_t* vals_a;           // total: the stable sort permutation, per mesh (mesh-local ids)
  uint32_t* vals_b;           // total
  Tri* sorted_tris;           // total: each mesh's triangles in leaf (Morton) order
};

// With b.sorted_tris set, leaf slot p of mesh k holds the p-th triangle of
// the mesh in stable Morton order (the plain build's sorted-leaf mode, mesh by
// mesh): the permutation ends in b.vals_a, the reordered triangles in
// b.sorted_tris.
// threads: CTA size (256..1024, a multiple of 32); radix_bits: digit width
// of the CTA-local sort (4, 6 or 8 bits: 8, 5 or 4 passes over the 30-bit
// codes); items: keys per thread in each ranked chunk (4 or 8).
cudaError_t launch_batch_build(const Tri* tris, const BatchBuffers& b, Node* nodes, uint32_t threads,
                               uint32_t radix_bits, uint32_t items, int num_sms, cudaStream_t s);

// Traversal copy of every mesh's nodes (local child references), plus the
// scene-bound flag word after the last node.
cudaError_t launch_batch_repack(const Node* nodes, uint32_t total_nodes, const uint32_t* off, uint32_t n_meshes,
                                WideNode* out, cudaStream_t s);

// Rays [roff[m], roff[m + 1]) are traced against mesh m.
// leaf_prim (sorted-leaf batches): mesh-local triangle id of each leaf slot,
// indexed like the triangles; nullptr for reference leaf order.
cudaError_t launch_batch_trace(const WideNode* wnodes,
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
                               cudaStream_t s);

} // namespace lbvh_gb300
