// Traversal launch parameters and launchers.
#pragma once

#include "common.cuh"

namespace lbvh_gb300 {

constexpr int kTraceThreads = 128;
constexpr uint32_t kStackSize = 128; // traversal_stack<scalar, 128>, lbvh.h:1874

cudaError_t launch_trace_tris(const Node* nodes,
                              const Tri* tris,
                              const uint32_t* leaf_prim,
                              const float* rays,
                              uint32_t m,
                              Hit* hits,
                              uint32_t* n_box,
                              uint32_t* n_tri,
                              cudaStream_t s);

} // namespace lbvh_gb300
