// Host-side declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rtbvh.h"
#include "device_common.cuh"

namespace rtbvh {

// Device memory of the library comes from one stream-ordered pool per device
// that keeps freed memory reserved (up to a cap) for the next call, so
// repeated builds neither map fresh memory nor synchronise in cudaFree.
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s);
// Stream-ordered free of a pool allocation.
void pool_free(void* p, cudaStream_t s);
// Frees long-lived pool allocations whose last use may be on any stream:
// waits for the device once, then frees them (NULL entries are skipped).
void pool_free_now(void* const* ptrs, int count);

template <class T>
cudaError_t device_alloc(T** p, size_t count, cudaStream_t s) {
  *p = nullptr;
  if (count == 0) return cudaSuccess;
  return pool_alloc(reinterpret_cast<void**>(p), count * sizeof(T), s);
}

// Stream-ordered scratch buffer from the library pool.
template <class T>
struct Scratch {
  T* ptr = nullptr;
  size_t count = 0;
  cudaStream_t stream = nullptr;
  cudaError_t alloc(size_t n, cudaStream_t s) {
    stream = s;
    count = n;
    if (n == 0) return cudaSuccess;
    return pool_alloc(reinterpret_cast<void**>(&ptr), n * sizeof(T), s);
  }
  ~Scratch() {
    if (ptr) pool_free(ptr, stream);
  }
  Scratch() = default;
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
};

// ------------------------------------------------------------------ prep
// Triangle::aabb / Triangle::center (shared/src/lib.rs:27-39) of n triangles
// (9 floats each). centers are written as float4 (w = 0).
cudaError_t launch_triangle_prep(const float* vertices, size_t n, DAabb* aabbs, float4* centers, cudaStream_t s);
// Primitive::aabb of point primitives (rtbvh_ffi/src/lib.rs:396-422): the
// empty box grown by the point. Also repacks the centres into float4.
cudaError_t launch_point_prep(const float* centers, size_t stride_floats, size_t n, DAabb* aabbs, float4* centers4,
                              cudaStream_t s);
// Repacks strided centres into float4.
cudaError_t launch_pack_centers(const float* centers, size_t stride_floats, size_t n, float4* centers4,
                                cudaStream_t s);
// Aabb::union_of_list (src/aabb.rs:124-131) into *world (one DAabb).
cudaError_t launch_world_bounds(const DAabb* aabbs, size_t n, DAabb* world, uint32_t* acc6, cudaStream_t s);
// MortonEncoder::encode of every centre against `world` (src/morton.rs:36-61);
// vals[i] = i.
cudaError_t launch_morton(const float4* centers, size_t n, const DAabb* world, uint32_t* keys, uint32_t* vals,
                          cudaStream_t s);
// Leaf-ordered triangles, kTriFloat4 float4 (64 bytes) per index slot:
// {v0, prim}, {v1 - v0, flags}, {v2 - v0, 0}, {0} for p = indices[k]. The
// flags word is 0 when gathered; an Mbvh whose traversal tree was built by
// build_mbvh (with triangles) sets kTriEscape there.
constexpr int kTriFloat4 = 4;
constexpr uint32_t kTriEscape = 1u;
cudaError_t launch_gather_triangles(const float* vertices, const uint32_t* indices, size_t n, float4* out,
                                    cudaStream_t s);

// ------------------------------------------------------------------ sort
// Stable LSD radix sort (onesweep) of (key, value) pairs on the low `bits`
// key bits. Buffers are ping-ponged; the sorted data ends in keys/vals.
// `status` receives kStatusTimeout if a look-back wait gave up.
size_t radix_sort_temp_bytes(size_t n);
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, size_t n, int bits, void* temp, size_t temp_bytes,
                             uint32_t* status, cudaStream_t s);

// ------------------------------------------------------------------ builds
struct BuildOutput {
  DAabb* nodes = nullptr;        // device, node_count entries (library pool, owned by caller)
  uint32_t* indices = nullptr;   // device, prim_count entries
  uint32_t node_count = 0;
};
// Builder::construct_locally_ordered_clustered (src/bvh.rs:113-137,
// src/builders/locb.rs). aabbs/centers are device arrays of n entries.
ResultCode build_locb(const DAabb* aabbs, const float4* centers, size_t n, cudaStream_t s, BuildOutput* out);
// Builder::construct_binned_sah (src/bvh.rs:87-111, src/builders/binned_sah.rs).
ResultCode build_binned_sah(const DAabb* aabbs, const float4* centers, size_t n, size_t prims_per_leaf,
                            cudaStream_t s, BuildOutput* out);

// SpatialSahBuilder::build (src/builders/spatial_sah.rs:926-1034): tris
// are the n triangles (9 floats each, prim-id order), centers their
// Primitive::center. *index_count gets the length of prim_indices
// (max_reference_count; entries past the leaves' ranges are 0). fixes:
// RTBVH_SPATIAL_FIX_* bits, 0 = the reference as written. Error where the
// reference panics.
uint64_t spatial_max_refs(size_t n);
ResultCode build_spatial_sah(const DAabb* aabbs, const float4* centers, const float* tris, size_t n,
                             size_t prims_per_leaf, uint32_t fixes, cudaStream_t s, BuildOutput* out,
                             uint32_t* index_count);

// Triangles for build_mbvh's escape flags (see build_mbvh): leaves index
// `indices` (index_count slots), which index `vertices` (vertex_count
// triangles, 9 floats each); `tris` are the leaf-ordered triangle records
// (kTriFloat4 float4 per index slot) whose flags word gets kTriEscape or 0;
// `tb` (node_count entries) receives the traversal boxes; with
// `tboxes_out`, build_mbvh also allocates the quad nodes' subtree boxes
// (DTBox per quad node, from `tb`) and stores them there.
struct MbvhTriangles {
  const uint32_t* indices = nullptr;
  uint32_t index_count = 0;
  const float* vertices = nullptr;
  uint32_t vertex_count = 0;
  float4* tris = nullptr;
  DAabb* tb = nullptr;
  DTBox** tboxes_out = nullptr;
};
// Mbvh::construct (src/bvh.rs:381-404). mnodes is allocated here. With
// `tri` (for BVH2s whose boxes need not contain these triangles: binned-SAH
// builds, whose left boxes can miss primitives, src/builders/
// binned_sah.rs:236-256; triangles attached after a build) the same passes
// also compute every node's box from the triangles into tri->tb (leaf:
// vertex boxes grown by 1e-4; interior: union of the children) and flag the
// escaped triangles: those whose grown vertex box does not lie inside every
// slot box the quad nodes test on the way to them. *escaped receives their
// number.
ResultCode build_mbvh(const DAabb* nodes, uint32_t node_count, cudaStream_t s, DMNode** mnodes,
                      uint32_t* mnode_count, const MbvhTriangles* tri = nullptr, uint32_t* escaped = nullptr);
// The closest-hit traversal tree: a 4-wide collapse of the BVH2 with tight
// slot boxes (largest-area child opened first), as exact nodes and compact
// copies; *wcount nodes, root 0. No tree (*wcount 0, Ok) when a node's box
// does not contain its children's (checked unless `nested` is known), or
// (indices given) when the leaves do not hold each of the index_count slots
// and each primitive exactly once -- spatial-split trees, whose leaf boxes
// bound fragments -- closest hit then reads the exact nodes in the
// reference's order.
ResultCode build_wide(const DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                      cudaStream_t s, DMNode** wnodes, DQNode** wq, uint32_t* wcount, bool nested = false);
// Traversal trees of a concatenated forest (LOCB meshes): mesh m's tree in
// nodes [off_m, off_m + n_m) of wnodes (exact) and wq (compact), root off_m;
// q0/q1 hold total_prims entries each.
cudaError_t launch_wide_segments(const DAabb* nodes, uint32_t node_count, const uint32_t* prim_off,
                                 const uint32_t* order, uint32_t mesh_count, uint32_t total_prims, DMNode* wnodes,
                                 DQNode* wq, uint2* q0, uint2* q1, uint32_t* status, unsigned blocks, cudaStream_t s);
// Compact (64-byte) copies of quad nodes for the closest-hit traversal;
// with live_count (device) only the first *live_count of `count` nodes.
cudaError_t launch_quantize_mbvh(const DMNode* mnodes, uint32_t count, DQNode* qnodes, cudaStream_t s,
                                 const uint32_t* live_count = nullptr);


// Bvh::refit (src/bvh.rs:176-205) bounds, topology kept. Leaves index
// `indices` (index_count slots), which index `aabbs` (prim_count boxes).
ResultCode refit_bvh(DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                     uint32_t prim_count, const DAabb* aabbs, cudaStream_t s);

// refit_bvh with its scratch in a static device array instead of per-call
// allocations (see rtbvh_gpu_refit_noalloc). Asynchronous on `s`; index
// errors are ORed into *status (the structure's status word).
ResultCode refit_bvh_noalloc(DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                             uint32_t prim_count, const DAabb* aabbs, uint32_t* status, cudaStream_t s);

// ------------------------------------------------------------------ traversal
struct TraceArgs {
  const DMNode* mnodes = nullptr;
  const DAabb* nodes = nullptr;
  uint32_t node_count = 0;
  const float4* tris = nullptr;  // leaf-ordered, kTriFloat4 float4 per index slot
  uint32_t prim_count = 0;       // index slots (bounds of leaf ranges)
  const float* rays = nullptr;
  const float* t_max = nullptr;
  size_t ray_count = 0;
  float4* hits = nullptr;
  uint32_t* stats = nullptr;
  uint32_t* status = nullptr;
  bool any_hit = false;
  const uint32_t* order = nullptr;  // optional: position k of the launch traces ray order[k]
  bool reorder = false;             // sort rays by (origin cell, direction) before tracing
  // Forest of many meshes: ray r belongs to the mesh m with
  // seg_ray_off[m] <= r < seg_ray_off[m + 1] and starts at quad node
  // seg_root[m]; a mesh without quad nodes (seg_root[m] == seg_root[m + 1])
  // is empty and its rays miss.
  const uint32_t* seg_ray_off = nullptr;
  const uint32_t* seg_root = nullptr;
  uint32_t seg_count = 0;
  // Launch shape of the persistent MBVH traversal (0: defaults): resident
  // blocks per SM (capped at the occupancy limit) and the number of rays a
  // warp takes from the global ray counter at a time.
  uint32_t blocks_per_sm = 0;
  uint32_t ray_batch = 0;
  // Optional closest-hit traversal tree (compact nodes `qnodes`, their
  // exact copies `qexact`, `q_count` nodes, root 0 or seg_qroot[m] per mesh):
  // closest-hit launches without statistics trace finite rays through it
  // (any hit, statistics and other rays use mnodes).
  const DQNode* qnodes = nullptr;
  const DMNode* qexact = nullptr;
  uint32_t q_count = 0;
  // the triangle records carry escape flags (build_mbvh with triangles):
  // rays that hit an escaped triangle are traced again over mnodes
  bool q_gates = false;
  const uint32_t* seg_qroot = nullptr;
  // Stack bound of the compact closest-hit walk: 32, 48 or 64 entries (0:
  // 64). A ray that needs more reports prim -2 and kStatusStackOverflow.
  uint32_t stack_limit = 0;
  // Optional subtree boxes of the quad nodes (mnodes): the exact-order pass
  // over the rays the compact walk hands on also skips slots whose subtree
  // box the ray cannot enter below its current t.
  const DTBox* tboxes = nullptr;
  // Optional per-ray counts of the compact closest-hit walk (3 per ray:
  // traversal-tree node visits, triangle tests, 1 if handed to the exact walk).
  uint32_t* walk_stats = nullptr;
  // Internal: the ray count is read from this device word (at most ray_count).
  const unsigned int* ray_count_dev = nullptr;
};
cudaError_t launch_trace_mbvh(const TraceArgs& a, cudaStream_t s);
cudaError_t launch_trace_bvh(const TraceArgs& a, cudaStream_t s);

// Candidate lists (see k_candidates in traverse.cu): ray r's first
// max_per_ray yielded primitive ids go to out[r * max_per_ray ...] (out may
// be NULL); counts[r] is the number of yields (UINT32_MAX: the walk failed).
struct CandArgs {
  const DMNode* mnodes = nullptr;
  const DAabb* nodes = nullptr;
  uint32_t node_count = 0;
  const uint32_t* indices = nullptr;
  uint32_t prim_count = 0;
  const float* rays = nullptr;
  const float* t_max = nullptr;
  size_t ray_count = 0;
  uint32_t max_per_ray = 0;
  uint32_t* out = nullptr;
  uint32_t* counts = nullptr;
  uint32_t* status = nullptr;
};
cudaError_t launch_candidates(const CandArgs& a, bool mbvh, cudaStream_t s);

// Packets of four rays (see packets.cu). origin/direction: three arrays of
// 4 * packet_count floats each (lane k of packet p at 4p + k); t: in/out.
struct PacketArgs {
  const DMNode* mnodes = nullptr;
  const DAabb* nodes = nullptr;
  uint32_t node_count = 0;
  const float4* tris = nullptr;
  uint32_t prim_count = 0;
  const float* origin[3] = {nullptr, nullptr, nullptr};
  const float* direction[3] = {nullptr, nullptr, nullptr};
  float* t = nullptr;
  size_t packet_count = 0;
  float4* hits = nullptr;     // optional, 4 * packet_count
  uint32_t* stats = nullptr;  // optional, 3 per packet
  uint32_t* status = nullptr;
};
cudaError_t launch_trace_packets(const PacketArgs& a, bool mbvh, cudaStream_t s);

// ------------------------------------------------------------------ many meshes
// Per-mesh clustering of a concatenated forest (see locb.cu).
// Meshes order[0, big_count) (the largest, more than kSegClusterMinPrims
// primitives) are clustered by `clusters` thread-block clusters of
// kSegCluster blocks (cluster_sums: kSegCluster words per cluster); the rest
// by up to `blocks` single blocks, on `side` (between the events fork and
// join) when it is given.
constexpr uint32_t kSegCluster = 8;
constexpr uint32_t kSegClusterMinPrims = 4096;  // default threshold (RTBatchTuning::cluster_min_prims)
cudaError_t launch_locb_segments(const DAabb* aabbs, const uint32_t* sorted, uint32_t* indices,
                                 const uint32_t* prim_off, const uint32_t* order, const DAabb* worlds,
                                 uint32_t mesh_count, uint32_t total_prims, DAabb* lvl0, DAabb* lvl1,
                                 DAabb* final_nodes, uint32_t* nb, uint32_t* status, unsigned blocks,
                                 uint32_t big_count, uint32_t* cluster_sums, unsigned clusters, cudaStream_t s,
                                 cudaStream_t side, cudaEvent_t fork, cudaEvent_t join);
// Per-mesh MBVH collapse of a concatenated forest (see mbvh.cu).
cudaError_t launch_collapse_segments(const DAabb* nodes, uint32_t node_count, const uint32_t* prim_off,
                                     const uint32_t* order, uint32_t mesh_count, uint32_t* parent, uint32_t* arrive,
                                     uint32_t* cnt_e, uint32_t* cnt_o, uint32_t* mbase, uint2* q0, uint2* q1,
                                     DMNode* mnodes, uint32_t m_capacity, uint32_t* status, unsigned blocks,
                                     cudaStream_t s);

// ------------------------------------------------------------------ backward
cudaError_t launch_intersect_backward(const float* vertices, size_t prim_count, const float* rays,
                                      const float4* hits, const float* grad_tuv, size_t ray_count,
                                      float* grad_vertices, float* grad_rays, cudaStream_t s);

// Number of SMs of the current device (cached).
int sm_count();

inline ResultCode cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return Ok;
  if (e == cudaErrorMemoryAllocation) return OutOfMemory;
  return DeviceError;
}

}  // namespace rtbvh
