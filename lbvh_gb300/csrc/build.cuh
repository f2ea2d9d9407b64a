// Build-side launch parameters, workspace views and launchers.
#pragma once

#include "common.cuh"

#include <utility>

namespace lbvh_gb300 {

constexpr int kBoundsThreads = 256;
constexpr int kMortonThreads = 256;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems; // 4096 keys per tile
// keys-only sorts of at most kSmallTileMaxPrims codes: tiles of kSmallTile
constexpr int kSmallTileItems = 4;
constexpr int kSmallTile = kSortThreads * kSmallTileItems; // 1024 keys per tile
constexpr uint32_t kSmallTileMaxPrims = 65536;
// look-back words a sort of n codes needs (tiles x 256)
constexpr size_t sort_tiles(size_t n)
{
  return n <= kSmallTileMaxPrims ? (n + kSmallTile - 1) / kSmallTile : (n + kSortTile - 1) / kSortTile;
}
// look-back words for any tile choice (the smaller tiles need the most)
constexpr size_t sort_tiles_any(size_t n)
{
  return (n + kSmallTile - 1) / kSmallTile;
}
constexpr uint32_t kMaxBoundsBlocksPerSm = 16; // bounds-pass CTAs per SM a context may ask for
// Keys-only sort of large builds: partition by the top 12 code bits, then
// sort each bucket by its low 18 bits in shared memory (used when every
// bucket fits).
constexpr uint32_t kMsdMinPrims = 1500000; // smaller builds use the onesweep passes only (faster below ~1.5M)
constexpr int kTopBits = 12, kTopBuckets = 1 << kTopBits;
// the bucket sort's two passes over the low 18 bits: an unstable one by bits
// 0-12, a stable one by bits 13-17
constexpr int kFirstBits = 13, kFirstDigits = 1 << kFirstBits;
constexpr int kSecondBits = 5, kSecondDigits = 1 << kSecondBits;
constexpr int kPartThreads = 1024, kPartItems = 16;
constexpr int kPartTile = kPartThreads * kPartItems; // 16384 keys per partition tile (one CTA per SM)
constexpr size_t kPartSmem = (size_t(2) * kTopBuckets + 2 * size_t(kPartTile)) * 4;
constexpr int kBucketThreads = 1024, kBucketItems = 8;
constexpr int kBucketChunk = kBucketThreads * kBucketItems; // 8192 keys ranked per step
constexpr uint32_t kBucketMax = 20480;          // largest bucket sorted in shared memory
constexpr size_t kBucketSmem = size_t(2) * kBucketMax * 4 + size_t(kBucketThreads / 32) * kSecondDigits * 2 +
                               size_t(kFirstDigits + kSecondDigits) * 4;
constexpr int kFitThreads = 256;
constexpr uint32_t kTreeBlock = 1024; // leaf slots per CTA of the tree build
// Pending-list capacity per CTA: the canonical pieces of a slot range number
// at most two per tree level, and the tree has at most 63 levels.
constexpr uint32_t kTreePendingPerBlock = 128;
constexpr uint32_t kTreeThreads = 256; // threads per CTA of the tree build (4 slots each)
// dynamic shared memory of the tree build: deltas, slots, node records (each
// array starts on a 32-byte boundary)
constexpr size_t kTreeSmem = (kTreeBlock + 8) * 4 + kTreeBlock * 4 + kTreeBlock * 32;
// Trees beyond this many primitives may walk their CTA-edge nodes from the
// local phase's tail (LBVH_PARAM_TREE_WALK_FUSED).
constexpr uint32_t kTreeGlobalCtaMaxPrims = 49152;
static_assert(((kTreeBlock + 8) * 4) % 32 == 0 && (kTreeBlock * 4) % 32 == 0, "smem alignment");
constexpr uint32_t kSpinLimit = 1u << 22;   // look-back polls before giving up
constexpr int kLookbackWindow = 8;          // look-back words read per poll
constexpr uint32_t kMaxTreeDepth = 64;      // 30-bit codes + 32-bit index tie-break
constexpr uint32_t kMaxPrims = (1u << 30) - 1; // look-back counts are 30-bit

// Merge phase of the tree build (k_tree_merge). The local phase leaves, per
// CTA, the maximal subtrees it completed -- its "pieces", which partition the
// CTA's leaf range -- ordered by first leaf, after a header. One merge CTA
// takes a window of consecutive groups (CTAs of the local phase, or windows
// of the level below), builds the nodes above their pieces with every
// arrival slot and child box in shared memory, and leaves the pieces of its
// window the same way; the last level is one CTA that reaches the root.
struct PieceRec
{
  uint32_t R;  // last leaf of the piece (its first is the previous piece's R + 1)
  int32_t dR;  // boundary delta after the piece: delta(R)
  Box box;
};
static_assert(sizeof(PieceRec) == 32, "piece record layout");
struct PieceHdr
{
  uint32_t count; // pieces of the group
  uint32_t L0;    // first leaf of the group
  int32_t dL;     // boundary delta before the group: delta(L0 - 1)
  uint32_t pad;
};
static_assert(sizeof(PieceHdr) == 16, "piece header layout");
constexpr int kMergeThreads = 1024;
constexpr uint32_t kMergeCap = 3200;        // pieces a merge CTA holds in shared memory
constexpr uint32_t kMergeGroups = 128;      // local-phase groups per window below the last level
constexpr uint32_t kMergeGroupsLater = 16;  // window groups per window below the last level
constexpr uint32_t kMergeFinalFirst = 160;  // local-phase groups the last level takes at once
constexpr uint32_t kMergeFinalLater = 16;   // window groups the last level takes at once
constexpr uint32_t kMergeMaxGroups = 160;   // largest window
constexpr uint32_t kMergeMaxLevels = 6;     // 2^30 leaves: 2^20 CTAs -> 8192 -> 512 -> 32 -> 2 -> 1
constexpr uint32_t kMergeOut = kTreePendingPerBlock; // pieces a window leaves (two per tree level)
// shared memory of k_tree_merge: group prefix, piece ends, deltas, slots,
// two child boxes per slot, the window's own pieces
constexpr size_t kMergeSmem = size_t(kMergeMaxGroups + 1) * 4 + size_t(kMergeCap) * (4 + 4 + 1) +
                              size_t(kMergeCap) * 2 * sizeof(Box) + size_t(kMergeOut) * 48 + 64;

constexpr size_t
align256(size_t x)
{
  return (x + 255) / 256 * 256;
}

// Where each level's pieces and headers live in the build's pending area:
// level 0 is written by the local phase (one group per CTA), level k >= 1 by
// the k-th merge launch (one group per window); the last launch writes none.
struct TreeScratch
{
  uint32_t merges;                          // merge launches (0: the local phase built the whole tree)
  uint32_t groups[kMergeMaxLevels + 1];     // groups of each level
  uint32_t window[kMergeMaxLevels];         // groups per window of each merge launch
  size_t pieces[kMergeMaxLevels + 1];       // byte offsets
  size_t hdrs[kMergeMaxLevels + 1];
  size_t bytes;
};

constexpr TreeScratch
tree_scratch(size_t n)
{
  TreeScratch t{};
  uint32_t g = uint32_t((n + kTreeBlock - 1) / kTreeBlock);
  size_t off = 0;
  for (uint32_t lv = 0;; lv++) {
    t.groups[lv] = g;
    t.pieces[lv] = off;
    off = align256(off + size_t(g) * kMergeOut * sizeof(PieceRec));
    t.hdrs[lv] = off;
    off = align256(off + size_t(g) * sizeof(PieceHdr));
    if (g <= 1 || lv == kMergeMaxLevels)
      break;
    const uint32_t final_max = lv == 0 ? kMergeFinalFirst : kMergeFinalLater;
    const uint32_t w = g <= final_max ? g : (lv == 0 ? kMergeGroups : kMergeGroupsLater);
    t.window[lv] = w;
    t.merges = lv + 1;
    g = (g + w - 1) / w;
  }
  t.bytes = off;
  return t;
}
// the largest build still ends in one window
static_assert(tree_scratch(kMaxPrims).groups[tree_scratch(kMaxPrims).merges] == 1,
              "merge levels");

// Keys-only builds of up to kSmallMaxPrims primitives run as one launch of
// k_small_build: a thread-block cluster of ceil(n / kSmallSlots) CTAs, each
// holding kSmallSlots primitives' boxes and codes in shared memory, which
// computes the bounds, the codes, the sort (over distributed shared memory),
// the local tree phase and (CTA 0) the merge without touching global memory
// in between.
constexpr uint32_t kSmallSlots = 1024;
constexpr int kSmallThreads = 1024;
constexpr uint32_t kSmallMaxCtas = 16; // a non-portable cluster size, checked per device
constexpr uint32_t kSmallMaxPrims = kSmallSlots * kSmallMaxCtas;
constexpr uint32_t kSmallMergeCap = kSmallMaxCtas * kMergeOut; // every piece of every CTA
// shared memory of k_small_build, byte offsets (each part on 32 bytes)
constexpr size_t kSmBox = 0;                                   // Box[kSmallSlots]: leaf boxes
constexpr size_t kSmKey = kSmBox + kSmallSlots * 24;           // uint32[2][kSmallSlots]: codes
constexpr size_t kSmPiece = kSmKey + 2 * kSmallSlots * 4;      // PieceRec[kMergeOut]: the CTA's pieces
constexpr size_t kSmUnion = kSmPiece + kMergeOut * 32;         // sort, tree or merge scratch:
// tree: int[kSmallSlots + 8] deltas, uint32[kSmallSlots] slots, Node[kSmallSlots], PendingNode[kMergeOut]
constexpr size_t kSmTreeSlot = (kSmallSlots + 8) * 4 + 32;
constexpr size_t kSmTreeRec = kSmTreeSlot + kSmallSlots * 4 + 32;
constexpr size_t kSmTreePend = kSmTreeRec + kSmallSlots * 32;
constexpr size_t kSmTree = kSmTreePend + kMergeOut * 32;
// merge: Box[2 x kSmallMergeCap] child boxes (piece i's own box at 2i first), uint32 ends, uint32 slots,
// int8 deltas, MergeOut[kMergeOut]
constexpr size_t kSmMergeR = size_t(kSmallMergeCap) * 2 * 24;
constexpr size_t kSmMergeSlot = kSmMergeR + kSmallMergeCap * 4;
constexpr size_t kSmMergeD = kSmMergeSlot + kSmallMergeCap * 4;
constexpr size_t kSmMergeOut = kSmMergeD + kSmallMergeCap;
constexpr size_t kSmMerge = kSmMergeOut + kMergeOut * 48;
constexpr size_t kSmSort = 2 * kSmallSlots * 4; // uint32[2][kSmallSlots]: bitonic exchange buffers
constexpr size_t kSmallSmem =
  kSmUnion + (kSmMerge > kSmTree ? (kSmMerge > kSmSort ? kSmMerge : kSmSort) : (kSmTree > kSmSort ? kSmTree : kSmSort));
static_assert(kSmUnion % 32 == 0 && kSmPiece % 32 == 0 && kSmTreeRec % 32 == 0, "small build smem alignment");

// Per-leaf box sources for the templated build kernels.
struct TriLeaf
{
  const Tri* tris;
  __device__ __forceinline__ Box operator()(uint32_t i) const { return load_tri_box(tris, i); }
  // Starts moving triangles [b0, b0 + cnt) into L2 (by the CTA's threads).
  __device__ __forceinline__ void prefetch(uint32_t b0, uint32_t cnt) const
  {
    const char* p = reinterpret_cast<const char*>(tris + b0);
    const uint32_t lines = (cnt * 48 + 127) / 128;
    for (uint32_t k = threadIdx.x; k < lines; k += blockDim.x)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(p + 128 * size_t(k)));
  }
};

struct BoxLeaf
{
  const Box* boxes;
  __device__ __forceinline__ Box operator()(uint32_t i) const
  {
    const float2* p = reinterpret_cast<const float2*>(boxes + i);
    const float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    return Box{ { a.x, a.y, b.x }, { b.y, c.x, c.y } };
  }
  // Starts moving the boxes of leaves [b0, b0 + cnt) into L2 (by the CTA's threads).
  __device__ __forceinline__ void prefetch(uint32_t b0, uint32_t cnt) const
  {
    const char* p = reinterpret_cast<const char*>(boxes + b0);
    const uint32_t lines = (cnt * 24 + 127) / 128;
    for (uint32_t k = threadIdx.x; k < lines; k += blockDim.x)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(p + 128 * size_t(k)));
  }
};

// Views into the context workspace for one build of n primitives.
struct BuildBuffers
{
  BuildState* state;
  void* partials;                 // bounds_blocks ArgBox records
  uint32_t* keys_a;               // codes (input order), then sorted codes
  uint32_t* keys_b;
  uint32_t* vals_a;               // sort permutation (pairs mode)
  uint32_t* vals_b;
  unsigned long long* lookback;   // tiles x 256 look-back words
  uint2* child;                   // refit: n-1 {left, right}
  uint32_t* leaf_parent;          // refit: n
  uint32_t* node_parent;          // refit: n-1
  unsigned long long* slots;      // n-1 epoch-tagged arrival slots (persistent)
  void* pending;                  // tree build: pieces and headers of every level (tree_scratch)
  Box* boxes;                     // optional: leaf boxes staged by the bounds pass (n)
  uint32_t bounds_blocks;
  uint32_t morton_blocks;
  bool msd;                       // keys-only build large enough for the bucket sort (kMsdMinPrims)
  uint32_t msd_range;             // bucket sort: codes per range (a multiple of 256)
  uint32_t msd_ranges;            // bucket sort: ranges = CTAs of the Morton pass
  uint32_t msd_group;             // bucket sort: ranges per CTA of the partition
  uint32_t sort_ctas;             // bucket sort: persistent CTAs (one per SM)
  uint32_t* top_rows;             // bucket sort: msd_ranges x kTopBuckets counts (in vals_a)
  uint32_t tile_keys;             // keys-only onesweep tile: 0 automatic (kSmallTile up to
                                  // kSmallTileMaxPrims codes, else kSortTile), or kSmallTile / kSortTile
  uint32_t walk_fused;            // trees beyond kTreeGlobalCtaMaxPrims: 0 merge the local phase's
                                  // pieces in shared memory, 1 walk them from the local phase's tail
  uint32_t merge_cap;             // test only: pieces a merge CTA holds (0: kMergeCap); fewer make
                                  // the merge fall back to its walk over global slots
  uint32_t spin_limit;            // look-back polls before a wait gives up (0: kSpinLimit)
  uint32_t wait_xor;              // test only: nonzero makes every look-back wait for a tag no
                                  // tile publishes, so each wait runs out (0 in normal use)
};

cudaError_t launch_make_triangles(const float* verts, uint32_t n, Tri* out, cudaStream_t s);
// Largest keys-only build k_small_build runs on the current device (0 when
// its cluster cannot be scheduled there); checked once per device.
uint32_t small_build_limit();
// The whole keys-only build of n <= small_build_limit() primitives in one
// launch: sorted codes to codes_out, nodes to `nodes`, errors to st->error.
cudaError_t launch_small_build_tris(const Tri* tris, uint32_t n, uint32_t* codes_out, Node* nodes, BuildState* st,
                                    cudaStream_t s);
cudaError_t launch_small_build_boxes(const Box* boxes, uint32_t n, uint32_t* codes_out, Node* nodes, BuildState* st,
                                     cudaStream_t s);
// Bounds + Morton codes; with b.boxes set, also stages the leaf boxes there
// (input order) so the Morton pass and launch_fit_staged read 24 bytes per
// leaf instead of the 48-byte triangle.
cudaError_t launch_curve_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, cudaStream_t s);
cudaError_t launch_curve_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, cudaStream_t s);
// passes < 4 (keys below 2^(8 passes)): the sorted keys / values end in
// keys_b / vals_b when passes is odd, else in keys_a / vals_a.
cudaError_t launch_sort(uint32_t n, bool pairs, uint32_t epoch_base, const BuildBuffers& b, cudaStream_t s,
                        uint32_t passes = 4);
// Tree construction + box fit from the sorted codes in keys_a; `epoch` tags
// this build's arrival slots and must differ from every earlier one on the
// same slots.
cudaError_t launch_fit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch,
                            cudaStream_t s);
cudaError_t launch_fit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch,
                             cudaStream_t s);
// Tree + fit over the leaf boxes staged by launch_curve_tris (input order).
cudaError_t launch_fit_staged(uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch, cudaStream_t s);
cudaError_t launch_gather_tris(const Tri* tris, const uint32_t* perm, uint32_t n, Tri* out, cudaStream_t s);
cudaError_t launch_gather_boxes(const Box* boxes, const uint32_t* perm, uint32_t n, Box* out, cudaStream_t s);
// Checks an outside node array (n_nodes internal nodes, n_nodes + 1 leaves)
// with leaf_parent / node_parent as counters; sets kErrBadTopology on failure.
cudaError_t launch_validate(const Node* nodes, uint32_t n_nodes, const BuildBuffers& b, cudaStream_t s);
cudaError_t launch_refit_tris(const Tri* tris, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch,
                              cudaStream_t s);
cudaError_t launch_refit_boxes(const Box* boxes, uint32_t n, const BuildBuffers& b, Node* nodes, uint32_t epoch,
                               cudaStream_t s);

} // namespace lbvh_gb300
