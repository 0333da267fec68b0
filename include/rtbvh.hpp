/*
 * rtbvh.hpp -- C++ form of rtbvh.h (the same library, the same symbols).
 *
 * The reference's rtbvh_ffi crate emits two headers from one cbindgen run
 * (rtbvh_ffi/build.rs:15-45): rtbvh.h for C and rtbvh.hpp for C++, the latter
 * with everything in `namespace rtbvh`, `enum class` enumerations and the
 * functions in an `extern "C"` block, include guard RTBVH_HPP. This header is
 * that C++ form for this library: a C++ caller written against the
 * reference's rtbvh.hpp (rtbvh::create_bvh, rtbvh::RTBvh,
 * rtbvh::ResultCode::Ok, rtbvh::BvhType::BinnedSAH ...) compiles unchanged
 * and links against librtbvh_rs.so / librtbvh_gb300.so. Layouts and values
 * equal rtbvh.h's; each declaration means what its rtbvh.h counterpart
 * documents. Include one of the two headers in a translation unit, not both.
 */
#ifndef RTBVH_HPP
#define RTBVH_HPP

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <new>
#include <ostream>

namespace rtbvh {

/* rtbvh_ffi/src/lib.rs:129-133 (repr(u32)) */
enum class BvhType : uint32_t {
  LocallyOrderedClustered = 0,
  BinnedSAH = 1,
};

/* rtbvh_ffi/src/lib.rs:17-25 (repr(C)), plus this library's extensions */
enum class ResultCode {
  Ok = 0,
  Error = 1,
  NoPrimitives = 2,
  InequalAabbsAndPrimitives = 3,
  Nan = 4,
  /* extensions (no counterpart in the reference) */
  DeviceError = 5,
  Timeout = 6,
  StackOverflow = 7,
  OutOfMemory = 8,
  InvalidArgument = 9,
};

/* rtbvh_ffi/src/lib.rs:144-151 -- 32 bytes */
struct RTAabb {
  float min[3];
  int32_t count;
  float max[3];
  int32_t left_first;
};

/* rtbvh_ffi/src/lib.rs:175-179 -- 32 bytes */
struct RTBvhNode {
  RTAabb aabb;
};

/* rtbvh_ffi/src/lib.rs:197-208 -- 128 bytes */
struct RTMbvhNode {
  float min_x[4];
  float max_x[4];
  float min_y[4];
  float max_y[4];
  float min_z[4];
  float max_z[4];
  int32_t children[4];
  int32_t counts[4];
};

/* rtbvh_ffi/src/lib.rs:210-220 */
struct RTBvh {
  uint32_t id;
  uint32_t node_count;
  const RTBvhNode *nodes;
  uint32_t index_count;
  const uint32_t *indices;
};

/* rtbvh_ffi/src/lib.rs:234-244 */
struct RTMbvh {
  uint32_t id;
  uint32_t node_count;
  const RTMbvhNode *nodes;
  uint32_t index_count;
  const uint32_t *indices;
};

/* (primitive id, in/out t, user data) -> true stops the traversal */
using RTIntersectFn = bool (*)(uint32_t, float *, void *);

/* ------------------------------------------------------------------ part 2 types */
using rtbvh_stream_t = void *;

struct RTGpuView {
  const void *nodes;
  uint32_t node_count;
  const uint32_t *indices;
  uint32_t index_count;
  const float *leaf_triangles;
};

struct RTBatch {
  uint32_t id;
};

struct RTGpuBatchView {
  const RTBvhNode *nodes;
  uint32_t node_capacity;
  const uint32_t *indices;
  const RTMbvhNode *mnodes;
  const uint32_t *mnode_base;
  const uint32_t *prim_offsets;
  uint32_t mesh_count;
  const float *leaf_triangles;
};

struct RTBatchTuning {
  uint32_t trace_blocks_per_sm;
  uint32_t trace_ray_batch;
  uint32_t cluster_min_prims;
  float pipeline_ms;
  uint32_t trace_stack;
};

extern "C" {

/* ------------------------------------------------------------------ part 1: rtbvh_ffi */
ResultCode create_spatial_Bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers, uintptr_t stride,
                              const float *vertices, uintptr_t vertex_stride, uintptr_t triangle_stride,
                              uint32_t prims_per_leaf, RTBvh *result);
ResultCode create_bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers, uintptr_t center_stride,
                      uintptr_t prims_per_leaf, BvhType bvh_type, RTBvh *result);
ResultCode create_mbvh(RTBvh bvh, RTMbvh *mbvh);
ResultCode refit(const RTAabb *aabbs, RTBvh bvh);
ResultCode intersect(RTBvh bvh, const float *origin, const float *direction, float *t, void *user_data,
                     RTIntersectFn intersect);
ResultCode intersect_packet(RTBvh bvh, const float *origin_x, const float *origin_y, const float *origin_z,
                            const float *direction_x, const float *direction_y, const float *direction_z, float *t,
                            void *user_data, RTIntersectFn intersect);
ResultCode intersect_mbvh(RTMbvh bvh, const float *origin, const float *direction, float *t, void *user_data,
                          RTIntersectFn intersect);
ResultCode intersect_mbvh_packet(RTMbvh bvh, const float *origin_x, const float *origin_y, const float *origin_z,
                                 const float *direction_x, const float *direction_y, const float *direction_z,
                                 float *t, void *user_data, RTIntersectFn intersect);
void free_bvh(RTBvh bvh);
void free_mbvh(RTMbvh bvh);

/* ------------------------------------------------------------------ part 2: GPU entry points */
#define RTBVH_FLAG_NO_HOST_MIRROR 1u
#define RTBVH_TRACE_ANY_HIT 1u
#define RTBVH_TRACE_STATS 2u
#define RTBVH_TRACE_REORDER 4u
#define RTBVH_TRACE_EXACT_NODES 8u
#define RTBVH_TRACE_WALK_STATS 16u
#define RTBVH_SPATIAL_FIX_CLIP 1u
#define RTBVH_SPATIAL_FIX_EXIT_BIN 2u
#define RTBVH_SPATIAL_FIX_SWEEP_BOX 4u
#define RTBVH_SPATIAL_FIX_SPLIT_SPACE 8u
#define RTBVH_SPATIAL_FIX_FALLBACK 16u
#define RTBVH_SPATIAL_FIX_ALL 31u
#define RTBVH_REFIT_NOALLOC_MAX_NODES 1048576u

ResultCode rtbvh_gpu_create_bvh_from_triangles(const float *vertices, uintptr_t prim_count,
                                               uintptr_t prims_per_leaf, BvhType bvh_type, uint32_t flags,
                                               rtbvh_stream_t stream, RTBvh *result);
ResultCode rtbvh_gpu_create_bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers,
                                uintptr_t center_stride, uintptr_t prims_per_leaf, BvhType bvh_type, uint32_t flags,
                                rtbvh_stream_t stream, RTBvh *result);
ResultCode rtbvh_gpu_create_spatial_bvh(const float *vertices, uintptr_t prim_count, const RTAabb *aabbs,
                                        const float *centers, uintptr_t center_stride, uintptr_t prims_per_leaf,
                                        uint32_t fixes, uint32_t flags, rtbvh_stream_t stream, RTBvh *result);
ResultCode rtbvh_gpu_create_mbvh(RTBvh bvh, uint32_t flags, rtbvh_stream_t stream, RTMbvh *result);
ResultCode rtbvh_gpu_set_triangles(uint32_t structure_id, int is_mbvh, const float *vertices, uintptr_t prim_count,
                                   rtbvh_stream_t stream);
ResultCode rtbvh_gpu_intersect_mbvh(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                    float *hits, uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_intersect_bvh(RTBvh bvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                   float *hits, uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_intersect_mbvh_packets(RTMbvh mbvh, const float *origin_x, const float *origin_y,
                                            const float *origin_z, const float *direction_x, const float *direction_y,
                                            const float *direction_z, float *t, uintptr_t packet_count, float *hits,
                                            uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_intersect_bvh_packets(RTBvh bvh, const float *origin_x, const float *origin_y,
                                           const float *origin_z, const float *direction_x, const float *direction_y,
                                           const float *direction_z, float *t, uintptr_t packet_count, float *hits,
                                           uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_mbvh_candidates(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                     uint32_t max_per_ray, uint32_t *candidates, uint32_t *counts,
                                     rtbvh_stream_t stream);
ResultCode rtbvh_gpu_bvh_candidates(RTBvh bvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                    uint32_t max_per_ray, uint32_t *candidates, uint32_t *counts,
                                    rtbvh_stream_t stream);
ResultCode rtbvh_intersect_mbvh_batch(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                      float *hits, uint32_t flags);
ResultCode rtbvh_gpu_status(uint32_t structure_id, int is_mbvh);
ResultCode rtbvh_gpu_view(uint32_t structure_id, int is_mbvh, RTGpuView *view);
ResultCode rtbvh_gpu_traversal_tree(RTMbvh mbvh, const RTMbvhNode **exact, const void **compact, uint32_t *count);
ResultCode rtbvh_gpu_refit(uint32_t bvh_id, const float *vertices, const RTAabb *aabbs, uint32_t mbvh_id,
                           rtbvh_stream_t stream);
ResultCode rtbvh_gpu_refit_mbvh(uint32_t mbvh_id, const float *vertices, const RTAabb *aabbs,
                                rtbvh_stream_t stream);
ResultCode rtbvh_serialize_bvh(RTBvh bvh, uint8_t *buffer, uintptr_t capacity, uintptr_t *size);
ResultCode rtbvh_deserialize_bvh(const uint8_t *buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                 RTBvh *result);
ResultCode rtbvh_serialize_mbvh(RTMbvh mbvh, uint8_t *buffer, uintptr_t capacity, uintptr_t *size);
ResultCode rtbvh_deserialize_mbvh(const uint8_t *buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                  RTMbvh *result);
ResultCode rtbvh_gpu_refit_noalloc(uint32_t bvh_id, const RTAabb *aabbs, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_intersect_backward(const float *vertices, uintptr_t prim_count, const float *rays,
                                        const float *hits, const float *grad_tuv, uintptr_t ray_count,
                                        float *grad_vertices, float *grad_rays, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_batch_create(const float *vertices, const uint32_t *prim_offsets, uint32_t mesh_count,
                                  const float *rays, const float *t_max, const uint32_t *ray_offsets, float *hits,
                                  uint32_t flags, rtbvh_stream_t stream, RTBatch *result);
ResultCode rtbvh_gpu_batch_run(RTBatch batch, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_batch_run_uncaptured(RTBatch batch, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_batch_view(RTBatch batch, RTGpuBatchView *view);
ResultCode rtbvh_gpu_batch_status(RTBatch batch);
void rtbvh_gpu_batch_free(RTBatch batch);
ResultCode rtbvh_gpu_batch_tune(RTBatch batch, rtbvh_stream_t stream, RTBatchTuning *result);
ResultCode rtbvh_gpu_batch_get_tuning(RTBatch batch, RTBatchTuning *result);
ResultCode rtbvh_gpu_batch_set_tuning(RTBatch batch, const RTBatchTuning *tuning, rtbvh_stream_t stream);
const char *rtbvh_gpu_version();

}  // extern "C"

}  // namespace rtbvh

#endif  // RTBVH_HPP
