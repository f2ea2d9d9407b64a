/*
 * lbvh_gb300 -- C ABI of the GB300 LBVH build + closest-hit trace library.
 *
 * This is the drop-in boundary for tay10r/lbvh's build and traversal path
 * (header `lbvh.h`). The reference is a header-only C++ template library
 * whose interface is lbvh::builder<float> (lbvh.h:312-353), lbvh::bvh<float>
 * (lbvh.h:259-299) and lbvh::traverser (lbvh.h:502-534); every entry point
 * below names the reference function it replaces. The C++ header
 * lbvh_gpu.hpp wraps these functions behind the reference's own types.
 *
 * Data layouts are the reference's:
 *   triangle   12 float32 {p0, e0 = a - b, e1 = c - a, normal}  (lbvh.h:1959-1983)
 *   box        6 float32 {min.xyz, max.xyz}                      (lbvh.h:208-215)
 *   node       lbvh_node, 32 bytes                               (lbvh.h:220-255)
 *   ray        8 float32 {pos, dir, tmin, tmax}                  (lbvh.h:388-401)
 *   hit        lbvh_hit, 16 bytes {prim, t, u, v}                (lbvh.h:359-382, 2015-2035)
 *
 * Pointers: every array argument may be device memory (cudaMalloc, managed)
 * or host memory (pageable or pinned); the library inspects it. Device
 * arguments are used in place and the call is asynchronous on the context's
 * stream. Host inputs are copied in before the call returns; a call that
 * writes host memory synchronizes the stream before it returns.
 *
 * Errors: every function returns an lbvh_status. Device-side failures of an
 * asynchronous call (a bounded wait that gave up, a malformed tree) are
 * reported by the next synchronizing call on the same context.
 *
 * Threading: a context serializes its work on one CUDA stream; use one
 * context per host thread. Work on one context must not be issued from two
 * threads at once.
 */
#ifndef LBVH_GB300_H
#define LBVH_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LBVH_API __attribute__((visibility("default")))
#else
#define LBVH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lbvh_status
{
  LBVH_OK = 0,
  LBVH_ERR_INVALID_ARG = 1, /* null pointer, n < 2, n too large, bad flags */
  LBVH_ERR_OOM = 2,         /* device allocation failed */
  LBVH_ERR_TIMEOUT = 3,     /* a bounded device-side wait expired */
  LBVH_ERR_DEVICE = 4,      /* CUDA runtime error; see lbvh_ctx_last_error */
  LBVH_ERR_BAD_TOPOLOGY = 5, /* a node array that is not a binary tree */
  LBVH_ERR_NOT_RESIDENT = 6, /* server: a trace or refit of a scene it does not hold */
  LBVH_ERR_BUDGET = 7,       /* server: a build larger than the whole HBM budget */
  LBVH_ERR_CANCELLED = 8,    /* server: cancelled (lbvh_server_cancel) before it started */
  LBVH_ERR_EXPIRED = 9       /* server: still queued after the server's max_queue_s */
} lbvh_status;

typedef struct lbvh_ctx lbvh_ctx; /* device, stream, workspace */
typedef struct lbvh_bvh lbvh_bvh; /* one device-resident BVH */

/* lbvh::node<float> (lbvh.h:220-255). left/right with LBVH_LEAF_BIT set are
 * leaf slots; otherwise they index internal nodes. nodes[0] is the root. */
typedef struct lbvh_node
{
  float lo[3];
  float hi[3];
  uint32_t left;
  uint32_t right;
} lbvh_node;

/* intersection_container<float, triangle_intersection<float>>
 * (lbvh.h:359-382, 2015-2035). A miss is {LBVH_MISS, +inf, 0, 0}. */
typedef struct lbvh_hit
{
  uint32_t prim;
  float t;
  float u;
  float v;
} lbvh_hit;

#define LBVH_LEAF_BIT 0x80000000u
#define LBVH_MISS 0xffffffffu
#define LBVH_MAX_PRIMS ((1u << 30) - 1)

/* Build flags. The default (0) is reference parity: leaf slot p holds
 * primitive p in input order, exactly as the reference's builder does
 * (lbvh.h:1728-1729, 1855-1862), so the node array is bit-identical to the
 * reference's. */

/* Leaf slot p holds the p-th primitive in (stable) Morton order: the intended
 * LBVH. Node array = the reference builder's output for the input permuted
 * by that order; trace reports original primitive ids. */
#define LBVH_BUILD_SORTED_LEAVES 0x1u
/* Keep the per-primitive Morton codes, the sorted codes, the stable sort
 * permutation and the centroid bounds for lbvh_bvh_curve. */
#define LBVH_BUILD_KEEP_CURVE 0x2u

/* Library version as major * 10000 + minor * 100 + patch. */
LBVH_API int lbvh_version(void);

/* Human-readable name of a status code. */
LBVH_API const char* lbvh_status_string(int status);

/* Creates a context on `device` that issues all its work on `stream` (a
 * cudaStream_t; NULL is the default stream). No reference counterpart: the
 * reference's builder owns a CPU task scheduler instead (lbvh.h:312-327). */
LBVH_API int lbvh_ctx_create(int device, void* stream, lbvh_ctx** out);
LBVH_API int lbvh_ctx_destroy(lbvh_ctx* ctx);
/* Waits for the context's stream and reports deferred device errors. */
LBVH_API int lbvh_ctx_synchronize(lbvh_ctx* ctx);
/* Message describing the last failure on this context ("" if none). */
LBVH_API const char* lbvh_ctx_last_error(const lbvh_ctx* ctx);
/* Grows the context workspace for builds of up to n_prims primitives and
 * traces of up to n_rays host-side rays, so later calls allocate nothing. */
LBVH_API int lbvh_ctx_reserve(lbvh_ctx* ctx, size_t n_prims, size_t n_rays);

/* Launch-shape parameters (lbvh_ctx_set_param). No reference counterpart:
 * they tune the GPU kernels, not the results. */
#define LBVH_PARAM_TRACE_BLOCKS_PER_SM 1 /* persistent traversal grid, 1..32 */
#define LBVH_PARAM_TRACE_REFILL 2        /* idle lanes before a warp refills, 1..32 */
#define LBVH_PARAM_BATCH_THREADS 3       /* CTA size of the batched build, 256..1024 */
#define LBVH_PARAM_TRACE_CHUNK 4         /* rays per chunk of a trace with host rays or hits, whose copies
                                            then overlap the traversal of other chunks (0: no chunks) */
#define LBVH_PARAM_TRACE_IN_PLACE 5      /* host rays / hits in page-locked (pinned) memory: 0 copies them,
                                            1 reads the rays in place, 2 (default) also writes the hits in
                                            place, each warp's batch of 32 as one 512-byte store (the
                                            traversal then reaches host memory over the CPU-GPU link);
                                            pageable host memory is always copied */
#define LBVH_PARAM_TRACE_LEAF_BATCH 8    /* lanes of a traversal warp with pending leaf-triangle tests
                                            before the warp runs them together, 1..32 (1, the default: each
                                            lane tests its triangles right after its visit); results do not
                                            change; long rays through loose trees gain from 4-8 */
#define LBVH_PARAM_BATCH_RADIX_BITS 9     /* digit width of the batched build's CTA-local radix sort: 4, 6
                                            or 8 bits (8, 5 or 4 passes over the 30-bit codes) */
#define LBVH_PARAM_BATCH_KEYS_PER_THREAD 10 /* keys per thread in each chunk that sort ranks: 4 or 8 */
#define LBVH_PARAM_SORT_TILE_KEYS 11     /* keys per tile of a keys-only onesweep sort: 0 (default: 1,024 up
                                            to 65,536 codes, else 4,096), 1024 or 4096 */
#define LBVH_PARAM_BUCKET_SORT_MIN 12    /* keys-only builds of at least this many primitives sort by
                                            buckets of the top 12 code bits (>= 65,536; default 1,500,000) */
#define LBVH_PARAM_BOUNDS_BLOCKS_PER_SM 13 /* CTAs per SM of the bounds pass, 1..16 (default 4) */
#define LBVH_PARAM_TREE_WALK_FUSED 14    /* trees of more than 49,152 primitives: 0 (default) merges the
                                            subtrees the local tree phase leaves at its CTA edges in
                                            shared memory, window by window; 1 walks them up through
                                            device-scope slots from each CTA's tail of the local phase */
#define LBVH_PARAM_SMALL_BUILD_MAX 16   /* builds of up to this many primitives (0..16384, default 16384)
                                            without LBVH_BUILD_SORTED_LEAVES or LBVH_BUILD_KEEP_CURVE run
                                            as one launch: a cluster of up to 16 CTAs that keeps the
                                            boxes, codes, sort and tree in shared memory; 0 always takes
                                            the multi-kernel build (the same nodes either way) */
#define LBVH_PARAM_TRACE_RAY_ORDER 17  /* 1: a trace of at least 4,096 rays whose hits go to device memory
                                            (or are staged there) first sorts the rays by origin cell, then
                                            direction cell (4 bits per axis each), and traverses them in that
                                            order; every hit still goes to its ray's slot, so the results
                                            are the same; 0 (default): the caller's order */
#define LBVH_PARAM_LOOKBACK_SPIN_LIMIT 6 /* polls of a radix-sort look-back wait before the build gives up
                                            and reports LBVH_ERR_TIMEOUT, 1..2^24 (default 2^22, a few
                                            seconds); no tree is built after a wait gave up */
#define LBVH_PARAM_TEST_LOOKBACK_STALL 7 /* test only: 1 makes every look-back wait for a word no tile
                                            ever writes, so each wait runs out after the spin limit and
                                            the build reports LBVH_ERR_TIMEOUT; 0 (default) for real use */
#define LBVH_PARAM_TEST_TREE_MERGE_CAP 15 /* test only: subtrees one tree-merge CTA holds in shared memory,
                                            1..3200; fewer than a window has make the build take the
                                            merge's fallback walk; 0 (default) for real use */
LBVH_API int lbvh_ctx_set_param(lbvh_ctx* ctx, int param, int value);

/* Replaces the reference triangle constructor triangle<float>(a, b, c)
 * (lbvh.h:1967-1972) for n triangles: verts is n x 9 float32 (a, b, c),
 * tris_out is n x 12 float32. Bit-identical to the reference compiled
 * without FP contraction. */
LBVH_API int lbvh_make_triangles(lbvh_ctx* ctx, const float* verts, size_t n, float* tris_out);

/* An empty BVH handle; builds reuse its storage. */
LBVH_API int lbvh_bvh_create(lbvh_ctx* ctx, lbvh_bvh** out);
LBVH_API int lbvh_bvh_destroy(lbvh_ctx* ctx, lbvh_bvh* bvh);

/* Replaces lbvh::builder<float>::operator()(const triangle<float>*, size_t,
 * const triangle_aabb_converter<float>&) (lbvh.h:329-345, 1793-1822):
 * builds `bvh` over n >= 2 triangles. Device `tris` are borrowed by the BVH
 * (as the reference traverser borrows its primitives, lbvh.h:507-524) and
 * must outlive it; host `tris` are copied into BVH-owned device memory. */
LBVH_API int lbvh_build_triangles(lbvh_ctx* ctx, const float* tris, size_t n, uint32_t flags, lbvh_bvh* bvh);

/* Replaces lbvh::builder<float>::operator() with a caller aabb_converter
 * (lbvh.h:342-345): the caller passes the converted boxes, n x 6 float32.
 * Same borrowing rule as lbvh_build_triangles. */
LBVH_API int lbvh_build_boxes(lbvh_ctx* ctx, const float* boxes, size_t n, uint32_t flags, lbvh_bvh* bvh);

/* Refit: recomputes every node box of an existing BVH over new primitive
 * positions, keeping the topology. No reference entry point (the
 * reference's fit, builder::fit_boxes lbvh.h:1826-1867, is protected); the
 * result equals that fit run over the existing nodes. `tris` (`boxes`) must
 * hold the same number of primitives in the same order as the build input;
 * it replaces the BVH's primitives. */
LBVH_API int lbvh_refit_triangles(lbvh_ctx* ctx, lbvh_bvh* bvh, const float* tris);
LBVH_API int lbvh_refit_boxes(lbvh_ctx* ctx, lbvh_bvh* bvh, const float* boxes);

/* Makes `bvh` from an existing node array (n_nodes x 32 bytes, host or
 * device, e.g. a reference lbvh::bvh<float>, lbvh.h:259-299) and its
 * n_nodes + 1 triangles, for lbvh_trace_triangles -- the reference traverser's
 * constructor traverser(const bvh<float>&, const triangle<float>*)
 * (lbvh.h:520-524). The nodes are copied; the check_bvh invariants
 * (lbvh_test.cpp:369-446) are verified on the device and a violation returns
 * LBVH_ERR_BAD_TOPOLOGY. Synchronizes. Same borrowing rule for device
 * triangles as lbvh_build_triangles. */
LBVH_API int lbvh_bvh_import_triangles(lbvh_ctx* ctx, const void* nodes, size_t n_nodes, const float* tris,
                                       lbvh_bvh* bvh);

/* Replaces bvh<float>::size() (lbvh.h:274): n_prims, n_nodes = n_prims - 1. */
LBVH_API int lbvh_bvh_info(const lbvh_bvh* bvh, size_t* n_prims, size_t* n_nodes, uint32_t* flags);
/* Replaces bvh<float>::begin()/operator[] (lbvh.h:270-292): copies the
 * (n_prims - 1) x 32-byte node array to dst (host or device). */
LBVH_API int lbvh_bvh_nodes(lbvh_ctx* ctx, const lbvh_bvh* bvh, void* dst);
/* Copies the primitives the BVH reads, in input order (n triangles of 48
 * bytes, or n boxes of 24 bytes). With lbvh_bvh_nodes this is the raw dump of
 * a BVH; lbvh_bvh_import_triangles loads such a dump back (a build in
 * reference leaf order). No reference counterpart: the reference's bvh<float>
 * holds only nodes and its caller keeps the primitives (lbvh.h:259-299). */
LBVH_API int lbvh_bvh_primitives(lbvh_ctx* ctx, const lbvh_bvh* bvh, void* dst);
/* Device address of the node array (valid until the next build/destroy). */
LBVH_API const void* lbvh_bvh_device_nodes(const lbvh_bvh* bvh);
/* Intermediate build arrays of a LBVH_BUILD_KEEP_CURVE build: Morton codes
 * in input order (morton_curve_kernel, lbvh.h:1422-1475), sorted codes
 * (space_filling_curve::sort, lbvh.h:1126-1134), the stable sort permutation,
 * and the centroid bounds (6 floats). Any output may be NULL. */
LBVH_API int lbvh_bvh_curve(lbvh_ctx* ctx, const lbvh_bvh* bvh, uint32_t* codes, uint32_t* sorted_codes,
                   uint32_t* perm, float* bounds6);

/* Replaces traverser<float, triangle<float>, triangle_intersection<float>>::
 * operator()(ray, triangle_intersector<float>) (lbvh.h:1869-1942,
 * 2055-2075) for m rays: rays is m x 8 float32, hits receives m lbvh_hit.
 * Requires a BVH built from triangles. */
LBVH_API int lbvh_trace_triangles(lbvh_ctx* ctx, const lbvh_bvh* bvh, const float* rays, size_t m, void* hits);
/* The sphere primitive and hit of the reference's example program
 * (examples/minimal.cpp:16-42): a sphere is {radius, x, y, z}; a hit is
 * sphere_hit {tmin, uv, normal} with the hit sphere's index. A miss is
 * {LBVH_MISS, +inf, 0, 0, {0, 0, 0}}. */
typedef struct lbvh_sphere_hit
{
  uint32_t prim;
  float t;
  float u;
  float v;
  float normal[3];
  float pad;
} lbvh_sphere_hit;

/* Replaces traverser<float, sphere, sphere_hit>::operator()(ray,
 * intersect_sphere) (lbvh.h:1869-1942 with the intersector of
 * examples/minimal.cpp:92-135) for m rays: the user-primitive path, the
 * intersector running on the device. `bvh` must have been built, without
 * LBVH_BUILD_SORTED_LEAVES, from these n spheres' boxes (the example's
 * sphere_to_box: {pos - radius, pos + radius}, e.g. with lbvh_build_boxes).
 * spheres is n x 4 float32, rays m x 8 float32, hits m lbvh_sphere_hit. The
 * hit index, t and normal are bit-identical to the reference; u and v come
 * from atan2 and acos and agree to within a few units in the last place. */
LBVH_API int lbvh_trace_spheres(lbvh_ctx* ctx, const lbvh_bvh* bvh, const float* spheres, const float* rays, size_t m,
                                void* hits);
/* Makes the BVH's traversal copy now, on the context's stream (traces make
 * it on first use otherwise). Callers that trace one BVH from several streams
 * call this once after each build / refit / import, before those traces. */
LBVH_API int lbvh_bvh_prepare_trace(lbvh_ctx* ctx, lbvh_bvh* bvh);
/* Same, also writing per-ray counts of box tests and triangle tests. */
LBVH_API int lbvh_trace_triangles_counts(lbvh_ctx* ctx, const lbvh_bvh* bvh, const float* rays, size_t m,
                                void* hits, uint32_t* n_box, uint32_t* n_tri);

/* ---- batched meshes --------------------------------------------------
 * Many independent meshes built and traced together. No single reference
 * counterpart: the batch equals running lbvh::builder<float> (lbvh.h:1793-1822)
 * and lbvh::traverser (lbvh.h:1869-1942) once per mesh. Mesh k's triangles are
 * [offsets[k], offsets[k + 1]) of one concatenated array (each mesh >= 2);
 * its node block starts at node offsets[k] - k, holds offsets[k + 1] -
 * offsets[k] - 1 nodes with mesh-local indices, and is bit-identical to the
 * reference's node array for that mesh alone. */
typedef struct lbvh_batch lbvh_batch;
LBVH_API int lbvh_batch_create(lbvh_ctx* ctx, lbvh_batch** out);
LBVH_API int lbvh_batch_destroy(lbvh_ctx* ctx, lbvh_batch* batch);
/* Builds every mesh in one persistent launch (one CTA per mesh at a time).
 * offsets: n_meshes + 1 uint32 (host or device); a bad device-side offsets
 * array is reported as LBVH_ERR_BAD_TOPOLOGY by the next synchronizing call. */
LBVH_API int lbvh_batch_build_triangles(lbvh_ctx* ctx, const float* tris, size_t total, const uint32_t* offsets,
                                        size_t n_meshes, lbvh_batch* batch);
/* lbvh_batch_build_triangles with build flags: 0 (reference leaf order, as
 * above) or LBVH_BUILD_SORTED_LEAVES, in which each mesh's node block equals
 * lbvh_build_triangles(..., LBVH_BUILD_SORTED_LEAVES) of that mesh alone and
 * lbvh_batch_trace_triangles reports mesh-local ids in input order. */
LBVH_API int lbvh_batch_build(lbvh_ctx* ctx, const float* tris, size_t total, const uint32_t* offsets, size_t n_meshes,
                              uint32_t flags, lbvh_batch* batch);
LBVH_API int lbvh_batch_info(const lbvh_batch* batch, size_t* n_meshes, size_t* total_prims, size_t* total_nodes);
/* As lbvh_bvh_prepare_trace, for a batch. */
LBVH_API int lbvh_batch_prepare_trace(lbvh_ctx* ctx, lbvh_batch* batch);
/* Copies all node blocks (total_prims - n_meshes nodes of 32 bytes). */
LBVH_API int lbvh_batch_nodes(lbvh_ctx* ctx, const lbvh_batch* batch, void* dst);
/* Copies mesh k's node block (its triangle count - 1 nodes), which is the node
 * array the reference's builder makes for that mesh alone. */
LBVH_API int lbvh_batch_mesh_nodes(lbvh_ctx* ctx, const lbvh_batch* batch, size_t k, void* dst);
/* Traces rays [ray_offsets[k], ray_offsets[k + 1]) against mesh k (m rays in
 * all, n_meshes + 1 offsets); hit primitive ids are mesh-local. Host ray
 * offsets are staged in the context, so once lbvh_batch_prepare_trace has
 * run, contexts on different streams may trace one batch at the same time. */
LBVH_API int lbvh_batch_trace_triangles(lbvh_ctx* ctx, const lbvh_batch* batch, const float* rays,
                                        const uint32_t* ray_offsets, size_t m, void* hits);

/* Largest primitive count lbvh_build_triangles_noalloc accepts. */
#define LBVH_NOALLOC_MAX_PRIMS 65536u

/* Allocation-free triangle build. No counterpart in the reference (whose
 * builder always allocates its own node vector, lbvh.h:1812).
 *
 * For callers that must not allocate device memory where they build: a
 * real-time loop that sizes all its buffers up front and forbids cudaMalloc
 * on its frame path, a plugin whose host application owns the GPU memory
 * budget, or a process whose device memory is held by another allocator.
 * The caller passes device triangles (n x 12 float32, 16-byte aligned) and a
 * device node array of (n - 1) x 32 bytes (32-byte aligned); the result is
 * bit-identical to lbvh_build_triangles with flags 0. All other memory is a
 * fixed scratch array inside the library, sized for LBVH_NOALLOC_MAX_PRIMS
 * primitives (about 1.5 MB, held by every GPU that loads the library until
 * the process exits); larger n is rejected with LBVH_ERR_INVALID_ARG, as are
 * host pointers. The call allocates nothing and does not synchronize: work
 * is queued on `stream` (a cudaStream_t, NULL = default stream) on the
 * current device. If d_status is not NULL it receives, in stream order, the
 * build's device error bits (0 = success).
 *
 * The first call on each device looks up the scratch array's device address
 * and keeps it for the life of the process; make it before capturing any
 * stream, and do not call again on a device after a cudaDeviceReset of it.
 * Every call clears the scratch it uses before building, so no state
 * carries over between calls. Every call on a device shares the one scratch
 * array: calls whose GPU work overlaps (other streams, other threads) race
 * and corrupt each other, so serialize them per device. */
LBVH_API int lbvh_build_triangles_noalloc(const float* d_tris, size_t n, void* d_nodes, uint32_t* d_status,
                                          void* stream);

/* ---- Request server -------------------------------------------------------
 * No reference counterpart (the reference builds and traces one scene per
 * call). A server keeps BVHs resident on one GPU and runs build / refit /
 * trace requests as they arrive: one dispatch thread and `slots` worker
 * threads, each worker with its own stream and context, so requests admitted
 * while others run overlap on the device. Admission is against an HBM budget
 * with least-recently-used eviction of scenes no waiting or running request
 * needs; builds of at most batch_max_tris triangles that wait together are
 * coalesced into one batched build, small traces (at most
 * trace_batch_max_rays rays) of one tree into one launch and of one batch
 * into one batched trace. A scene's requests start in submission order.
 * An evicted scene is dumped to host memory (its nodes and triangles, as
 * lbvh_bvh_nodes / lbvh_bvh_primitives give them) while host_budget allows,
 * and the next trace or refit of it loads it back (lbvh_bvh_import_triangles,
 * tree checked on the device) instead of failing with LBVH_ERR_NOT_RESIDENT;
 * the least recently used dumps are dropped to stay within host_budget.
 * Every result equals the same request run alone through lbvh_build_triangles
 * / lbvh_refit_triangles / lbvh_trace_triangles. */
typedef struct lbvh_server lbvh_server;

#define LBVH_REQ_BUILD 0 /* data: rows triangles (n x 12 float32); (re)builds the scene */
#define LBVH_REQ_REFIT 1 /* data: the scene's triangles moved (same count and order) */
#define LBVH_REQ_TRACE 2 /* data: rows rays (n x 8 float32); hits: rows lbvh_hit */

typedef struct lbvh_server_config
{
  int device;
  int slots;                   /* worker streams (1..64) */
  size_t hbm_budget;           /* bytes of resident scenes: 144 per triangle + 64 KiB each */
  size_t batch_max_tris;       /* largest build that is coalesced (0: never) */
  size_t batch_max_requests;   /* most requests in one coalesced launch */
  size_t trace_batch_max_rays; /* largest trace that is coalesced */
  size_t host_budget;          /* bytes of host memory for evicted scenes (0: evicted scenes are dropped) */
  double max_queue_s;          /* a request not started this many seconds after its arrival fails with
                                  LBVH_ERR_EXPIRED (0: requests wait as long as they must) */
} lbvh_server_config;

typedef struct lbvh_request_done
{
  uint64_t ticket;
  int status;                  /* lbvh_status of the request */
  int kind;                    /* LBVH_REQ_* */
  int64_t scene;
  double arrival;              /* seconds since the server started: submitted */
  double start;                /* dispatched to a worker */
  double done;                 /* its GPU work and result copy finished */
  char message[160];           /* why it failed ("" on success) */
} lbvh_request_done;

typedef struct lbvh_server_stats
{
  uint64_t submitted, completed, coalesced_requests, evictions;
  uint64_t resident_scenes, resident_bytes;
  uint64_t spills, reloads;        /* evictions kept on the host; scenes loaded back */
  uint64_t spilled_scenes, spilled_bytes;
  uint64_t cancelled, expired;     /* requests that never ran: lbvh_server_cancel, max_queue_s */
} lbvh_server_stats;

LBVH_API int lbvh_server_create(const lbvh_server_config* config, lbvh_server** out);
/* Queues a request. `data` (host or device) must stay valid and unchanged,
 * and `hits` (trace only: rows lbvh_hit, host or device) writable, until the
 * request is reported done. Returns its ticket. */
LBVH_API int lbvh_server_submit(lbvh_server* server, int kind, int64_t scene, const float* data, size_t rows,
                                void* hits, uint64_t* ticket);
/* Waits up to timeout_s seconds for finished requests and moves up to `max`
 * of them into out (each request is reported once); *n_out = how many. */
LBVH_API int lbvh_server_wait_any(lbvh_server* server, lbvh_request_done* out, size_t max, double timeout_s,
                                  size_t* n_out);
/* The server's clock: seconds since it was created (the clock of
 * lbvh_request_done's times). */
LBVH_API double lbvh_server_clock(const lbvh_server* server);
/* Cancels a request that has not started: it is reported done with
 * LBVH_ERR_CANCELLED and never runs (later requests of its scene run as if it
 * had not been submitted). A request that has started or finished is not
 * affected. Returns LBVH_OK either way; the outcome is the request's report. */
LBVH_API int lbvh_server_cancel(lbvh_server* server, uint64_t ticket);
/* Test hook (failure injection on the host): the next `count` device
 * allocations the server's workers make for request data (triangles, node
 * and ray/hit staging buffers) fail as on an exhausted device. Each affected
 * request reports LBVH_ERR_OOM, the HBM budget it held is returned, a scene
 * whose rebuild failed keeps its previous tree, and the server goes on. */
LBVH_API int lbvh_server_inject_alloc_failures(lbvh_server* server, uint32_t count);
/* Blocks until every request submitted so far has finished. */
LBVH_API int lbvh_server_drain(lbvh_server* server);
LBVH_API int lbvh_server_stats_get(lbvh_server* server, lbvh_server_stats* out);
/* The scenes resident after the dispatcher's last step (up to cap ids). */
LBVH_API int lbvh_server_resident(lbvh_server* server, int64_t* scenes, size_t cap, size_t* n_out);
/* Finishes all queued work, stops the threads and frees every resident
 * scene. Finished requests not yet taken by lbvh_server_wait_any are lost. */
LBVH_API int lbvh_server_destroy(lbvh_server* server);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LBVH_GB300_H */
