/*
 * rtbvh.h -- C ABI of the GB300 BVH build + ray traversal library
 * (librtbvh_gb300.so; also installed as librtbvh_rs.so).
 *
 * Part 1 is a drop-in for the C ABI of meirbon/rtbvh's `rtbvh_ffi` crate
 * (rtbvh_ffi/src/lib.rs, header generated by cbindgen in rtbvh_ffi/build.rs):
 * same symbol names, same enum values, same struct layouts, same ownership
 * (the library owns every structure; handles are by-value views that stay
 * valid until free_*). Builds run on the GPU; node arrays are mirrored to
 * host memory so that the handle pointers and the host-callback traversal
 * entry points keep working.
 *
 * Part 2 adds GPU entry points (prefix rtbvh_gpu_) that take device pointers
 * and a CUDA stream: builds from device triangles, the fused closest-hit /
 * any-hit traversal, refit and the differentiable backward pass. They return
 * ResultCode, extended by the values marked "extension" below.
 */
#ifndef RTBVH_H
#define RTBVH_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* rtbvh_ffi/src/lib.rs:17-25 */
typedef enum ResultCode {
  Ok = 0,
  Error = 1,
  NoPrimitives = 2,
  InequalAabbsAndPrimitives = 3,
  Nan = 4,
  /* extensions (no counterpart in the reference) */
  DeviceError = 5,   /* a CUDA call failed */
  Timeout = 6,       /* a bounded device-side wait gave up */
  StackOverflow = 7, /* a traversal stack bound was exceeded */
  OutOfMemory = 8,
  InvalidArgument = 9
} ResultCode;

/* rtbvh_ffi/src/lib.rs:129-133 (repr(u32)) */
#ifdef __cplusplus
enum BvhType : uint32_t {
  LocallyOrderedClustered = 0,
  BinnedSAH = 1,
};
#else
enum BvhType {
  LocallyOrderedClustered = 0,
  BinnedSAH = 1,
};
typedef uint32_t BvhType;
#endif

/* rtbvh_ffi/src/lib.rs:144-151 -- 32 bytes */
typedef struct RTAabb {
  float min[3];
  int32_t count;
  float max[3];
  int32_t left_first;
} RTAabb;

/* rtbvh_ffi/src/lib.rs:175-179 -- 32 bytes */
typedef struct RTBvhNode {
  RTAabb aabb;
} RTBvhNode;

/* rtbvh_ffi/src/lib.rs:197-208 -- 128 bytes, quad node in SoA form */
typedef struct RTMbvhNode {
  float min_x[4];
  float max_x[4];
  float min_y[4];
  float max_y[4];
  float min_z[4];
  float max_z[4];
  int32_t children[4];
  int32_t counts[4];
} RTMbvhNode;

/* rtbvh_ffi/src/lib.rs:210-220 */
typedef struct RTBvh {
  uint32_t id;
  uint32_t node_count;
  const RTBvhNode *nodes;
  uint32_t index_count;
  const uint32_t *indices;
} RTBvh;

/* rtbvh_ffi/src/lib.rs:234-244 */
typedef struct RTMbvh {
  uint32_t id;
  uint32_t node_count;
  const RTMbvhNode *nodes;
  uint32_t index_count;
  const uint32_t *indices;
} RTMbvh;

/* Candidate callback of the host traversal entry points:
 * (primitive id, in/out t, user data) -> true stops the traversal. */
typedef bool (*RTIntersectFn)(uint32_t, float *, void *);

/* ------------------------------------------------------------------ part 1 */

/* rtbvh_ffi/src/lib.rs:345-389: Builder::construct_spatial_sah
 * (src/bvh.rs:59-85, src/builders/spatial_sah.rs) over RTTriangleWrapper
 * primitives, built on the GPU from host inputs. Vertex k of triangle i is
 * read at float offset (i * triangle_stride / 4) + k * (vertex_stride / 4),
 * its centre at i * stride / 4; aabbs NULL -> Primitive::aabb of the
 * wrapper, which reads the vertices at (vertex0 offset * (vertex_stride / 4))
 * / 4 (the triangle's own vertices when vertex_stride is 16): where that
 * would read past the triangles' vertices this library returns
 * InvalidArgument. The result is the reference's as written (no
 * RTBVH_SPATIAL_FIX_* bits): its index vector has max_reference_count =
 * n + (n as f32 * 0.75) as usize entries, and on many inputs some
 * primitives are not referenced by any leaf (see rtbvh_gpu_create_spatial_bvh
 * for corrected builds). centers/vertices/result NULL or stride % 4 != 0 ->
 * Error; an input on which the reference panics -> Error. */
ResultCode create_spatial_Bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers, uintptr_t stride,
                              const float *vertices, uintptr_t vertex_stride, uintptr_t triangle_stride,
                              uint32_t prims_per_leaf, RTBvh *result);

/* rtbvh_ffi/src/lib.rs:428-493. Host inputs; the build runs on the GPU.
 * centers/result NULL -> Error; center_stride must be 12 or 16 (the reference
 * aborts on any other value, this library returns Error); aabbs NULL -> the
 * boxes are the centre points; prims_per_leaf 0 -> 1. */
ResultCode create_bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers, uintptr_t center_stride,
                      uintptr_t prims_per_leaf, BvhType bvh_type, RTBvh *result);

/* rtbvh_ffi/src/lib.rs:499-513 */
ResultCode create_mbvh(RTBvh bvh, RTMbvh *mbvh);

/* rtbvh_ffi/src/lib.rs:519-538. Recomputes the node boxes of a stored Bvh from
 * new primitive boxes, on the GPU. The boxes equal the reference's bit for
 * bit; the node topology is kept (the reference also zeroes every node's
 * count/left_first, a defect this library does not reproduce). */
ResultCode refit(const RTAabb *aabbs, RTBvh bvh);

/* rtbvh_ffi/src/lib.rs:551-581 (host traversal calling back per candidate) */
ResultCode intersect(RTBvh bvh, const float *origin, const float *direction, float *t, void *user_data,
                     RTIntersectFn intersect);

/* rtbvh_ffi/src/lib.rs:599-686 */
ResultCode intersect_packet(RTBvh bvh, const float *origin_x, const float *origin_y, const float *origin_z,
                            const float *direction_x, const float *direction_y, const float *direction_z, float *t,
                            void *user_data, RTIntersectFn intersect);

/* rtbvh_ffi/src/lib.rs:700-731 */
ResultCode intersect_mbvh(RTMbvh bvh, const float *origin, const float *direction, float *t, void *user_data,
                          RTIntersectFn intersect);

/* rtbvh_ffi/src/lib.rs:749-835 */
ResultCode intersect_mbvh_packet(RTMbvh bvh, const float *origin_x, const float *origin_y, const float *origin_z,
                                 const float *direction_x, const float *direction_y, const float *direction_z,
                                 float *t, void *user_data, RTIntersectFn intersect);

/* rtbvh_ffi/src/lib.rs:837-849 */
void free_bvh(RTBvh bvh);
void free_mbvh(RTMbvh bvh);

/* ------------------------------------------------------------------ part 2
 * GPU entry points. No counterpart in the reference (it has no GPU path);
 * each is the device-side form of the reference call named beside it.
 * `stream` is a cudaStream_t (NULL: the legacy default stream).
 * Device arrays:
 *   vertices  n x 9 float   v0, v1, v2 of triangle i
 *   aabbs     n x RTAabb
 *   rays      R x 6 float   origin, direction
 *   t_max     R float       per-ray upper bound (NULL: 1e34, Ray::new)
 *   hits      R x 4         float t, float u, float v, int32 prim (-1: miss)
 */
typedef void *rtbvh_stream_t;

/* flags for the build entry points */
#define RTBVH_FLAG_NO_HOST_MIRROR 1u /* keep nodes on the device only (handle pointers are NULL) */

/* flags for the trace entry points */
#define RTBVH_TRACE_ANY_HIT 1u /* stop at the first accepted triangle (occlusion) */
#define RTBVH_TRACE_STATS 2u   /* write per-ray node visits / triangle tests / max stack depth */
#define RTBVH_TRACE_REORDER 4u /* MBVH: trace in (origin cell, direction)-sorted order; results are unchanged */
/* MBVH closest hit without statistics reads a 64-byte compact copy of every
 * quad node (8-bit outward-rounded child bounds) by default: the nearest
 * hit (t, u, v and its triangle) is the reference's, but where two
 * triangles are hit at exactly the same t either may be reported. This flag
 * reads the exact 128-byte nodes in the reference's visit order instead. */
#define RTBVH_TRACE_EXACT_NODES 8u
/* MBVH closest hit over the compact nodes (the default walk) with per-ray
 * counts of that walk in `stats` (3 per ray): traversal-tree node visits,
 * triangle tests, and 1 if the ray was handed on to the exact-node walk
 * (its hit is that walk's; its counts cover the compact part only). These
 * are this library's own work per ray, not the reference iterator's (for
 * those use RTBVH_TRACE_STATS). Hits are those of the call without the
 * flag. InvalidArgument with RTBVH_TRACE_STATS, _ANY_HIT, _EXACT_NODES or
 * _REORDER, on a Bvh, or on an Mbvh without a traversal tree; Error if
 * stats is NULL. The host-buffer entry ignores it. */
#define RTBVH_TRACE_WALK_STATS 16u

/* Builder::construct_binned_sah / construct_locally_ordered_clustered on
 * device triangles (src/bvh.rs:87-137, with aabbs = Triangle::aabb and
 * centres = Triangle::center of shared/src/lib.rs:27-39). The triangles are
 * kept with the structure for traversal. */
ResultCode rtbvh_gpu_create_bvh_from_triangles(const float *vertices, uintptr_t prim_count,
                                               uintptr_t prims_per_leaf, BvhType bvh_type, uint32_t flags,
                                               rtbvh_stream_t stream, RTBvh *result);

/* create_bvh (rtbvh_ffi/src/lib.rs:428-493) with device inputs. centers has
 * center_stride bytes per primitive (12 or 16). aabbs must not be NULL. */
ResultCode rtbvh_gpu_create_bvh(const RTAabb *aabbs, uintptr_t prim_count, const float *centers,
                                uintptr_t center_stride, uintptr_t prims_per_leaf, BvhType bvh_type, uint32_t flags,
                                rtbvh_stream_t stream, RTBvh *result);

/* Corrections of the reference's spatial-split builder
 * (src/builders/spatial_sah.rs), for rtbvh_gpu_create_spatial_bvh. 0 builds
 * the reference as written. */
#define RTBVH_SPATIAL_FIX_CLIP 1u        /* split_edge returns a + t*(b-a), not a*t*(b-a) (:90-93) */
#define RTBVH_SPATIAL_FIX_EXIT_BIN 2u    /* a reference leaves its last bin, not its first (:545-546) */
#define RTBVH_SPATIAL_FIX_SWEEP_BOX 4u   /* the sweep's left box is the union of bins 0..i, not of
                                            their suffix unions (:549-570) */
#define RTBVH_SPATIAL_FIX_SPLIT_SPACE 8u /* allocate_children gives the freed split space to the left
                                            child and keeps the right child on its moved references
                                            (:375-424); without it references are lost */
#define RTBVH_SPATIAL_FIX_FALLBACK 16u   /* the equal-count fallback counts from the task's begin
                                            (:643-648) */
#define RTBVH_SPATIAL_FIX_ALL 31u

/* Builder::construct_spatial_sah (src/bvh.rs:59-85) on device triangles
 * (n x 9 floats, kept with the structure for traversal). aabbs NULL ->
 * Triangle::aabb, centers NULL -> Triangle::center (shared/src/lib.rs:27-39);
 * center_stride 12 or 16 bytes. fixes: RTBVH_SPATIAL_FIX_* bits. The index
 * vector has max_reference_count entries (RTBvh::index_count); a triangle
 * split by the builder has several. Error where the reference panics. */
ResultCode rtbvh_gpu_create_spatial_bvh(const float *vertices, uintptr_t prim_count, const RTAabb *aabbs,
                                        const float *centers, uintptr_t center_stride, uintptr_t prims_per_leaf,
                                        uint32_t fixes, uint32_t flags, rtbvh_stream_t stream, RTBvh *result);

/* Mbvh::construct (src/bvh.rs:381-404) on the GPU. */
ResultCode rtbvh_gpu_create_mbvh(RTBvh bvh, uint32_t flags, rtbvh_stream_t stream, RTMbvh *result);

/* Attaches device triangles (prim-id order) to a Bvh (is_mbvh = 0) or Mbvh
 * (is_mbvh = 1) for the fused traversal; they are re-laid in leaf order
 * (v0, v1-v0, v2-v0). Structures built by rtbvh_gpu_create_bvh_from_triangles
 * (and Mbvhs made from them) already carry them. An Mbvh's closest-hit
 * traversal tree is rebuilt from the new triangles (see
 * rtbvh_gpu_traversal_tree), so that its hits stay the reference's walk's
 * over the unchanged boxes. */
ResultCode rtbvh_gpu_set_triangles(uint32_t structure_id, int is_mbvh, const float *vertices, uintptr_t prim_count,
                                   rtbvh_stream_t stream);

/* MbvhIndexIterator (src/iter_indices.rs:212-313) driving the triangle test
 * of src/builders/spatial_sah.rs:132-163, for R rays, one ray per thread.
 * Asynchronous on `stream`; errors found on the device (stack overflow) are
 * reported by rtbvh_gpu_status. stats: R x 3 uint32 or NULL. */
ResultCode rtbvh_gpu_intersect_mbvh(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                    float *hits, uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);

/* BvhIndexIterator (src/iter_indices.rs:18-107) driving the triangle test. */
ResultCode rtbvh_gpu_intersect_bvh(RTBvh bvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                   float *hits, uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);

/* Packets of four rays: intersect_mbvh_packet (rtbvh_ffi/src/lib.rs:749-835)
 * over MbvhPacketIndexIterator (src/iter_indices.rs:316-414) for
 * packet_count packets at once, on the device, with the reference's packet
 * triangle test SpatialTriangle::intersect4 (src/builders/spatial_sah.rs:
 * 165-244, t_min 1e-4) as the candidate callback (examples/benchmark.rs:
 * 43-68). The six ray arrays and t are device arrays of 4 * packet_count
 * floats in the FFI's SoA form: lane k of packet p is element 4p + k. t is
 * in/out like the FFI's t (initial bound in, nearest accepted t out).
 * hits (R x 4: t, u, v, prim; NULL to skip) and stats (3 uint32 per packet:
 * node tests, triangle tests, max stack depth; with RTBVH_TRACE_STATS) are
 * optional. A node is entered when any lane of the packet hits it, so each
 * lane's nearest hit is the nearest its packet test accepts. RTBVH_TRACE_ANY_HIT
 * and RTBVH_TRACE_REORDER are not supported here (InvalidArgument); NaN
 * inputs are traced as the iterator traces them (the FFI's early Nan return
 * is the caller's check). Asynchronous on `stream`. */
ResultCode rtbvh_gpu_intersect_mbvh_packets(RTMbvh mbvh, const float *origin_x, const float *origin_y,
                                            const float *origin_z, const float *direction_x, const float *direction_y,
                                            const float *direction_z, float *t, uintptr_t packet_count, float *hits,
                                            uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);

/* intersect_packet (rtbvh_ffi/src/lib.rs:599-686) over BvhPacketIndexIterator
 * (src/iter_indices.rs:110-200), same arrays and rules as above; a packet
 * with a NaN origin or direction component walks nothing. */
ResultCode rtbvh_gpu_intersect_bvh_packets(RTBvh bvh, const float *origin_x, const float *origin_y,
                                           const float *origin_z, const float *direction_x, const float *direction_y,
                                           const float *direction_z, float *t, uintptr_t packet_count, float *hits,
                                           uint32_t flags, uint32_t *stats, rtbvh_stream_t stream);

/* Candidate lists: the device form of intersect_mbvh with a user callback
 * (rtbvh_ffi/src/lib.rs:700-731) for primitives whose intersection test the
 * library does not know (spheres, curves, instances, ...). For each ray, the
 * primitive ids that MbvhIndexIterator (src/iter_indices.rs:212-313) yields
 * when the callback leaves t unchanged, in yield order, over the exact quad
 * nodes; t is t_max[r] (NULL: 1e34). The caller then tests the listed
 * primitives in its own kernel; its nearest accepted hit is the one the
 * callback iteration would find, since a callback that shortens t only
 * removes candidates. Ray r's first max_per_ray ids go to
 * candidates[r * max_per_ray ...] (candidates may be NULL to count only);
 * counts[r] (required) is the full number of yields, so a count above
 * max_per_ray means the list was cut and can be fetched again with a larger
 * stride (UINT32_MAX: the walk hit the stack bound, see rtbvh_gpu_status).
 * Asynchronous on `stream`. */
ResultCode rtbvh_gpu_mbvh_candidates(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                     uint32_t max_per_ray, uint32_t *candidates, uint32_t *counts,
                                     rtbvh_stream_t stream);

/* The same over the Bvh with BvhIndexIterator (src/iter_indices.rs:18-107),
 * i.e. intersect (rtbvh_ffi/src/lib.rs:551-581). A ray with a NaN origin or
 * direction component yields nothing. */
ResultCode rtbvh_gpu_bvh_candidates(RTBvh bvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                    uint32_t max_per_ray, uint32_t *candidates, uint32_t *counts,
                                    rtbvh_stream_t stream);

/* Same as rtbvh_gpu_intersect_mbvh with HOST rays / t_max / hits, returning
 * when the hits are in host memory. When every buffer is page-locked and
 * mapped for the device (cudaHostAlloc / cudaMallocHost / pinned tensors)
 * the traversal reads the rays and writes the hits in host memory itself;
 * otherwise it copies in, traces and copies out in chunks on two internal
 * streams. */
ResultCode rtbvh_intersect_mbvh_batch(RTMbvh mbvh, const float *rays, const float *t_max, uintptr_t ray_count,
                                      float *hits, uint32_t flags);

/* Reads (and clears) the device status word of a structure: Ok, or the first
 * error a traversal on it raised (StackOverflow, Timeout). Synchronises. */
ResultCode rtbvh_gpu_status(uint32_t structure_id, int is_mbvh);

/* Device views of a structure's arrays (nodes, indices, leaf-ordered
 * triangles 3 x float4 per index slot). Pointers stay valid until free_*. */
typedef struct RTGpuView {
  const void *nodes;
  uint32_t node_count;
  const uint32_t *indices;
  uint32_t index_count;
  const float *leaf_triangles;
} RTGpuView;
ResultCode rtbvh_gpu_view(uint32_t structure_id, int is_mbvh, RTGpuView *view);

/* The Mbvh's closest-hit traversal tree (no counterpart in the reference):
 * a 4-wide collapse of the source Bvh, `count` nodes with root 0, as exact
 * RTMbvhNode records (`exact`) and as the 64-byte compact records the
 * kernel reads (`compact`). Built when the Mbvh has triangles. When the
 * Bvh's boxes were built from those triangles by locally-ordered
 * clustering (or refitted from them), each slot keeps its own box; else
 * (binned SAH, whose left boxes can miss primitives; triangles attached or
 * replaced later) each slot box is recomputed from the triangles and the
 * slots whose box, as the reference's Mbvh tests it, may miss them are
 * gated: the compact record's flag byte (bits 24-31 of word 3) has bit 1
 * set on a node reached through a gated slot and bits 4-7 on gated leaf
 * slots; a ray that passes a gated slot is traced again over the exact
 * Mbvh in the reference's order. count 0: no tree (closest hit uses the
 * exact Mbvh). Device pointers, valid until the Mbvh is freed, refitted or
 * given new triangles. */
ResultCode rtbvh_gpu_traversal_tree(RTMbvh mbvh, const RTMbvhNode **exact, const void **compact, uint32_t *count);

/* Bvh::refit (src/bvh.rs:176-205) on the GPU from device triangles or device
 * aabbs (exactly one non-NULL); updates the Bvh and, if mbvh_id != UINT32_MAX,
 * re-collapses that Mbvh from it and re-lays its triangles. */
ResultCode rtbvh_gpu_refit(uint32_t bvh_id, const float *vertices, const RTAabb *aabbs, uint32_t mbvh_id,
                           rtbvh_stream_t stream);

/* An Mbvh refit (the reference refits only the Bvh, src/bvh.rs:176-205): the
 * Mbvh keeps its own copy of the Bvh's nodes, as the crate's Mbvh does
 * (src/bvh.rs:318-324); this refits that copy with Bvh::refit's arithmetic
 * from device triangles or device aabbs (exactly one non-NULL), then
 * collapses the quad nodes again (Mbvh::construct, same topology) and
 * re-lays the triangles. The source Bvh is not needed and not changed. */
ResultCode rtbvh_gpu_refit_mbvh(uint32_t mbvh_id, const float *vertices, const RTAabb *aabbs,
                                rtbvh_stream_t stream);

/* On-disk form of the crate's serde derives (src/bvh.rs:141-147 Bvh,
 * :318-324 Mbvh) as bincode 1 writes them with its default options:
 * little-endian fixed-width integers, a u64 length before each Vec, nodes as
 * their 32-byte RTAabb / 128-byte RTMbvhNode records, the BuildType as a u32
 * variant index (None 0, LocallyOrderedClustered 1, BinnedSAH 2, Spatial 3):
 *   Bvh:  u64 N, N x RTBvhNode, u64 M, M x uint32 index, uint32 build type
 *   Mbvh: u64 N, N x RTBvhNode, u64 Q, Q x RTMbvhNode, u64 M, M x uint32 index
 * serialize: buffer NULL (or too small: InvalidArgument) -> *size receives the
 * byte count. deserialize: validates the layout, the leaf ranges, child
 * pairs and indices (InvalidArgument otherwise; no primitives:
 * NoPrimitives) and, for an Mbvh, that the quad nodes are the collapse of
 * the stored Bvh nodes; creates a library-owned structure (host mirror
 * unless RTBVH_FLAG_NO_HOST_MIRROR). Triangles are not part of the format:
 * attach them with rtbvh_gpu_set_triangles before a GPU trace. */
ResultCode rtbvh_serialize_bvh(RTBvh bvh, uint8_t *buffer, uintptr_t capacity, uintptr_t *size);
ResultCode rtbvh_deserialize_bvh(const uint8_t *buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                 RTBvh *result);
ResultCode rtbvh_serialize_mbvh(RTMbvh mbvh, uint8_t *buffer, uintptr_t capacity, uintptr_t *size);
ResultCode rtbvh_deserialize_mbvh(const uint8_t *buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                  RTMbvh *result);

/* Largest tree (in nodes) that rtbvh_gpu_refit_noalloc accepts: 1,048,576
 * nodes, i.e. a BVH over up to 524,288 primitives. */
#define RTBVH_REFIT_NOALLOC_MAX_NODES 1048576u

/* No counterpart in the reference. The refit of rtbvh_gpu_refit (new
 * primitive boxes, device pointer) for callers that cannot allocate device
 * memory while they run, such as a per-frame animation loop that must not
 * call cudaMalloc (it can synchronise the device or fail mid-frame). It
 * allocates nothing: its scratch is a fixed array inside the library
 * (8 MiB + 256 bytes). The array is reserved on a GPU when the library's
 * code is first used there -- with CUDA's lazy module loading at the latest
 * on the first call -- and stays reserved until the process exits.
 * - Updates the Bvh's device nodes only, asynchronously on `stream`; the
 *   host mirror behind the handle's node pointer and any Mbvh made from the
 *   Bvh are left as they were.
 * - Trees with more than RTBVH_REFIT_NOALLOC_MAX_NODES nodes are rejected
 *   with InvalidArgument before anything runs.
 * - A tree whose leaves index past the Bvh's index or primitive counts is
 *   not read out of bounds; the error is recorded in the Bvh's status word,
 *   which rtbvh_gpu_status reports (Error) once the stream has run.
 * - The first call on a device looks up the array's device address, so make
 *   that first call before any stream capture.
 * - All calls share the one array: calls that can overlap on the GPU (other
 *   streams, other host threads) race and must be serialised by the caller.
 *   The Bvh must not be freed while a call on it can still be running. */
ResultCode rtbvh_gpu_refit_noalloc(uint32_t bvh_id, const RTAabb *aabbs, rtbvh_stream_t stream);

/* Backward pass of the closest-hit triangle test for rays traced with
 * rtbvh_gpu_intersect_mbvh (hits as written there). Maps upstream
 * (dL/dt, dL/du, dL/dv) per ray (R x 3 float) to dL/dvertices (n x 9 float,
 * overwritten, summed in a fixed order per triangle so that the result is
 * deterministic) and dL/dray (R x 6 float: origin, direction; NULL to skip).
 * vertices are the triangles the hits were traced against (prim-id order). */
ResultCode rtbvh_gpu_intersect_backward(const float *vertices, uintptr_t prim_count, const float *rays,
                                        const float *hits, const float *grad_tuv, uintptr_t ray_count,
                                        float *grad_vertices, float *grad_rays, rtbvh_stream_t stream);

/* ---- many meshes in one build + trace (no counterpart in the reference)
 * The meshes are concatenated: mesh m owns triangles
 * [prim_offsets[m], prim_offsets[m + 1]) of `vertices` (every mesh needs at
 * least one triangle) and rays [ray_offsets[m], ray_offsets[m + 1]) of
 * `rays`. Each mesh gets the locally-ordered clustering build + MBVH of its
 * own triangles (Builder::construct_locally_ordered_clustered + Mbvh::from),
 * and its rays are traced against it; hit prim ids are indices into the
 * concatenated triangles. All meshes share one set of launches: a stable
 * (mesh, Morton) sort, one block per mesh for the clustering and the
 * collapse (a thread-block cluster per large mesh for the clustering), and
 * one persistent traversal launch. create() allocates every
 * buffer and captures the whole pipeline in a CUDA graph; run() replays it
 * on the same device buffers (update their contents in place between runs).
 * prim_offsets / ray_offsets are host arrays of mesh_count + 1 entries. */
typedef struct RTBatch {
  uint32_t id;
} RTBatch;

typedef struct RTGpuBatchView {
  const RTBvhNode *nodes;        /* forest: mesh m's nodes start at 2 prim_offsets[m] - m */
  uint32_t node_capacity;
  const uint32_t *indices;       /* primitive order of every mesh, global indices */
  const RTMbvhNode *mnodes;      /* mesh m's quad nodes: [mnode_base[m], mnode_base[m + 1]) */
  const uint32_t *mnode_base;    /* device, mesh_count + 1 */
  const uint32_t *prim_offsets;  /* device, mesh_count + 1 */
  uint32_t mesh_count;
  const float *leaf_triangles;
} RTGpuBatchView;

ResultCode rtbvh_gpu_batch_create(const float *vertices, const uint32_t *prim_offsets, uint32_t mesh_count,
                                  const float *rays, const float *t_max, const uint32_t *ray_offsets, float *hits,
                                  uint32_t flags, rtbvh_stream_t stream, RTBatch *result);
/* Replays the captured build + trace on `stream`. */
ResultCode rtbvh_gpu_batch_run(RTBatch batch, rtbvh_stream_t stream);
/* The same pipeline issued as individual launches (no graph). */
ResultCode rtbvh_gpu_batch_run_uncaptured(RTBatch batch, rtbvh_stream_t stream);
ResultCode rtbvh_gpu_batch_view(RTBatch batch, RTGpuBatchView *view);
/* Reads and clears the device status of the last runs (synchronises). */
ResultCode rtbvh_gpu_batch_status(RTBatch batch);
void rtbvh_gpu_batch_free(RTBatch batch);

/* Launch parameters of a batch; 0 in a field means the default. */
typedef struct RTBatchTuning {
  uint32_t trace_blocks_per_sm; /* resident traversal blocks per SM (default: occupancy limit) */
  uint32_t trace_ray_batch;     /* rays a warp takes from the global ray counter at a time (0: the library's default, 32; at most 4096) */
  uint32_t cluster_min_prims;   /* meshes with more primitives get a thread-block cluster (default 4096) */
  float pipeline_ms;            /* tune: measured build + trace time with the chosen values */
  uint32_t trace_stack;         /* stack entries per ray of the closest-hit walk: 32, 48 or 64
                                   (0 in set_tuning: 64); a ray that needs more reports prim -2
                                   and StackOverflow (the reference's stack holds 32,
                                   src/iter_indices.rs:22) */
} RTBatchTuning;
/* Times candidate values on this batch's own meshes and rays (the pipeline
 * runs several times on `stream`, overwriting the hits), keeps the fastest
 * and re-captures the graph with it; `result` (may be NULL) receives it.
 * Results do not depend on these parameters. Synchronises. */
ResultCode rtbvh_gpu_batch_tune(RTBatch batch, rtbvh_stream_t stream, RTBatchTuning *result);
/* Reads (get) or sets and re-captures (set) the parameters. */
ResultCode rtbvh_gpu_batch_get_tuning(RTBatch batch, RTBatchTuning *result);
ResultCode rtbvh_gpu_batch_set_tuning(RTBatch batch, const RTBatchTuning *tuning, rtbvh_stream_t stream);

/* Library version string. */
const char *rtbvh_gpu_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* RTBVH_H */
