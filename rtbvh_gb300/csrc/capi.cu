// C ABI of the library: the rtbvh_ffi-compatible entry points and the GPU
// entry points declared in include/rtbvh.h.
//
// Storage mirrors rtbvh_ffi's StructureManager (rtbvh_ffi/src/lib.rs:8-127):
// the library owns every structure in two id-indexed tables (Bvh, Mbvh);
// ids are never reused; free_* empties a slot. Each entry holds the device
// arrays (nodes, indices, leaf-ordered triangles) and, unless asked not to,
// a host mirror of nodes and indices that the handle pointers refer to.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "lib_internal.h"

using namespace rtbvh;

namespace {

struct Entry {
  bool alive = false;
  bool mirrored = false;
  uint32_t node_count = 0;
  uint32_t prim_count = 0;        // index slots (prim_indices entries)
  uint32_t vertex_count = 0;      // primitives: boxes and triangles (a spatial tree has more slots)
  bool vertex_lower_bound = false;  // loaded from bytes: vertex_count is the largest index + 1
  DAabb* d_nodes = nullptr;       // Bvh; Mbvh: its own copy of the source Bvh's nodes
  uint32_t bvh_node_count = 0;    // Mbvh: entries of d_nodes
  uint32_t build_type = 0;        // the crate's BuildType (1 LOCB, 2 binned SAH, 3 spatial; 0 unknown);
                                  // an Mbvh keeps its source Bvh's
  bool boxes_cover = false;       // every box contains the attached triangles (see boxes_cover())
  DMNode* d_mnodes = nullptr;     // Mbvh
  DQNode* d_qnodes = nullptr;     // Mbvh: closest-hit traversal tree, compact nodes
  DMNode* d_wnodes = nullptr;     // Mbvh: the same tree, exact nodes
  DTBox* d_tboxes = nullptr;      // Mbvh with q_gates: subtree boxes of d_mnodes (from the triangles)
  uint32_t wcount = 0;
  bool q_gates = false;           // Mbvh: escaped triangles are flagged (collapse_entry)
  uint32_t* d_indices = nullptr;
  float4* d_tris = nullptr;       // 3 per index slot
  float* d_vertices = nullptr;    // prim-id order, 9 floats each
  uint32_t* d_status = nullptr;
  uint32_t source_bvh = UINT32_MAX;
  std::vector<DAabb> h_nodes;
  std::vector<DMNode> h_mnodes;
  std::vector<uint32_t> h_indices;

  void release() {
    void* const arrays[] = {d_nodes, d_mnodes, d_qnodes, d_wnodes, d_tboxes, d_indices, d_tris, d_vertices, d_status};
    pool_free_now(arrays, 9);
    d_nodes = nullptr;
    d_mnodes = nullptr;
    d_qnodes = nullptr;
    d_wnodes = nullptr;
    d_tboxes = nullptr;
    wcount = 0;
    q_gates = false;
    d_indices = nullptr;
    d_tris = nullptr;
    d_vertices = nullptr;
    d_status = nullptr;
    std::vector<DAabb>().swap(h_nodes);
    std::vector<DMNode>().swap(h_mnodes);
    std::vector<uint32_t>().swap(h_indices);
    node_count = prim_count = vertex_count = 0;
    alive = false;
    mirrored = false;
  }
};

std::mutex g_mu;
std::vector<std::unique_ptr<Entry>> g_bvh, g_mbvh;

Entry* lookup(uint32_t id, bool mbvh) {
  auto& t = mbvh ? g_mbvh : g_bvh;
  if (id >= t.size()) return nullptr;
  Entry* e = t[id].get();
  return (e && e->alive) ? e : nullptr;
}

uint32_t store(std::unique_ptr<Entry> e, bool mbvh) {
  auto& t = mbvh ? g_mbvh : g_bvh;
  t.push_back(std::move(e));
  return (uint32_t)(t.size() - 1);
}

// Indices for build_wide's leaf check: trees of the object-split builders
// (LOCB, binned SAH) hold each primitive once by construction and skip it;
// spatial-split trees and structures of unknown origin are checked.
const uint32_t* leaf_check(uint32_t build_type, const uint32_t* indices) {
  return (build_type == 1 || build_type == 2) ? nullptr : indices;
}

// Boxes contain the triangles they were built from for LOCB builds (a leaf
// is its primitive's box grown by 1e-4, src/builders/locb.rs) and after a
// refit from triangles (each box recomputed from them, src/bvh.rs:176-205).
// A binned-SAH build as written sizes a left child's box from bins
// [0, best_splits[axis].count), which after the longest-axis fallback is
// not the split (src/builders/binned_sah.rs:236-256), so its boxes can miss
// primitives; boxes built from aabbs, and triangles attached or replaced
// later, promise nothing either.
bool boxes_cover(uint32_t build_type) { return build_type == 1; }

// The quad nodes (*mnodes, *mcount: Mbvh::construct) and the closest-hit
// traversal tree of Mbvh entry m, from its own BVH2 nodes and triangles:
// the plain traversal tree (build_wide over m's boxes) when the boxes
// contain the triangles, else the tree over boxes recomputed from the
// triangles with escape flags in m's triangle records (build_mbvh with
// MbvhTriangles; object-split leaves only, spatial-split trees get none);
// no traversal tree while m has no triangles. The caller has released m's
// previous traversal tree and (re)gathered the triangles.
ResultCode collapse_entry(Entry& m, cudaStream_t s, DMNode** mnodes, uint32_t* mcount) {
  m.d_wnodes = nullptr;
  m.d_qnodes = nullptr;
  m.d_tboxes = nullptr;
  m.wcount = 0;
  m.q_gates = false;
  if (m.bvh_node_count == 0) {  // Mbvh::default()
    *mnodes = nullptr;
    *mcount = 0;
    return Ok;
  }
  if (!m.d_nodes) return Error;
  const bool tris = m.d_vertices && m.d_tris && !m.vertex_lower_bound;
  const uint32_t* check = leaf_check(m.build_type, m.d_indices);
  ResultCode rc;
  if (!tris || m.boxes_cover || m.build_type == 3) {
    if ((rc = build_mbvh(m.d_nodes, m.bvh_node_count, s, mnodes, mcount)) != Ok || !tris) return rc;
    return build_wide(m.d_nodes, m.bvh_node_count, check, m.prim_count, s, &m.d_wnodes, &m.d_qnodes, &m.wcount);
  }
  Scratch<DAabb> tb;
  cudaError_t err;
  if ((err = tb.alloc(m.bvh_node_count, s))) return cuda_rc(err);
  MbvhTriangles t;
  t.indices = m.d_indices;
  t.index_count = m.prim_count;
  t.vertices = m.d_vertices;
  t.vertex_count = m.vertex_count;
  t.tris = m.d_tris;
  t.tb = tb.ptr;
  t.tboxes_out = &m.d_tboxes;
  uint32_t escaped = 0;
  if ((rc = build_mbvh(m.d_nodes, m.bvh_node_count, s, mnodes, mcount, &t, &escaped)) != Ok) return rc;
  // boxes recomputed from the triangles nest by construction
  rc = build_wide(tb.ptr, m.bvh_node_count, check, m.prim_count, s, &m.d_wnodes, &m.d_qnodes, &m.wcount, true);
  m.q_gates = escaped != 0 && m.wcount != 0;
  if (!m.q_gates) {  // no ray is handed on for an escape: the subtree boxes would go unused
    pool_free(m.d_tboxes, s);
    m.d_tboxes = nullptr;
  }
  return rc;
}

cudaStream_t legacy_stream() {
  static cudaStream_t s = nullptr;
  static std::once_flag once;
  std::call_once(once, []() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); });
  return s;
}

RTBvh bvh_handle(uint32_t id, const Entry& e) {
  RTBvh h;
  h.id = id;
  h.node_count = e.node_count;
  h.nodes = e.mirrored ? reinterpret_cast<const RTBvhNode*>(e.h_nodes.data()) : nullptr;
  h.index_count = e.prim_count;
  h.indices = e.mirrored ? e.h_indices.data() : nullptr;
  return h;
}

RTMbvh mbvh_handle(uint32_t id, const Entry& e) {
  RTMbvh h;
  h.id = id;
  h.node_count = e.node_count;
  h.nodes = e.mirrored ? reinterpret_cast<const RTMbvhNode*>(e.h_mnodes.data()) : nullptr;
  h.index_count = e.prim_count;
  h.indices = e.mirrored ? e.h_indices.data() : nullptr;
  return h;
}

ResultCode mirror_bvh(Entry& e, cudaStream_t s) {
  e.h_nodes.resize(e.node_count);
  e.h_indices.resize(e.prim_count);
  cudaError_t err;
  if (e.node_count &&
      (err = cudaMemcpyAsync(e.h_nodes.data(), e.d_nodes, (size_t)e.node_count * sizeof(DAabb),
                             cudaMemcpyDeviceToHost, s)))
    return cuda_rc(err);
  if (e.prim_count && (err = cudaMemcpyAsync(e.h_indices.data(), e.d_indices, (size_t)e.prim_count * 4,
                                             cudaMemcpyDeviceToHost, s)))
    return cuda_rc(err);
  if ((err = cudaStreamSynchronize(s))) return cuda_rc(err);
  e.mirrored = true;
  return Ok;
}

ResultCode mirror_mbvh(Entry& e, cudaStream_t s) {
  e.h_mnodes.resize(e.node_count);
  e.h_indices.resize(e.prim_count);
  cudaError_t err;
  if (e.node_count && (err = cudaMemcpyAsync(e.h_mnodes.data(), e.d_mnodes, (size_t)e.node_count * sizeof(DMNode),
                                             cudaMemcpyDeviceToHost, s)))
    return cuda_rc(err);
  if (e.prim_count && (err = cudaMemcpyAsync(e.h_indices.data(), e.d_indices, (size_t)e.prim_count * 4,
                                             cudaMemcpyDeviceToHost, s)))
    return cuda_rc(err);
  if ((err = cudaStreamSynchronize(s))) return cuda_rc(err);
  e.mirrored = true;
  return Ok;
}

// Stores a built Bvh (`slots` index entries over n primitives, BuildType
// `build_type`) with its status word, optional device triangles (prim-id
// order, re-laid per index slot) and host mirror.
ResultCode store_bvh(const BuildOutput& out, uint32_t slots, size_t n, uint32_t build_type, const float* d_vertices,
                     uint32_t flags, cudaStream_t s, RTBvh* result) {
  auto e = std::make_unique<Entry>();
  e->alive = true;
  e->node_count = out.node_count;
  e->prim_count = slots;
  e->vertex_count = (uint32_t)n;
  e->d_nodes = out.nodes;
  e->d_indices = out.indices;
  e->build_type = build_type;
  e->boxes_cover = boxes_cover(build_type) && d_vertices != nullptr;  // boxes from these triangles
  ResultCode rc;
  cudaError_t err;
  if ((err = device_alloc(&e->d_status, 4, s)) || (err = cudaMemsetAsync(e->d_status, 0, 16, s))) {
    e->release();
    return cuda_rc(err);
  }
  if (d_vertices) {
    if ((err = device_alloc(&e->d_vertices, 9 * n, s)) ||
        (err = cudaMemcpyAsync(e->d_vertices, d_vertices, 36 * n, cudaMemcpyDeviceToDevice, s)) ||
        (err = device_alloc(&e->d_tris, (size_t)kTriFloat4 * slots, s)) ||
        (err = launch_gather_triangles(e->d_vertices, e->d_indices, slots, e->d_tris, s))) {
      e->release();
      return cuda_rc(err);
    }
  }
  if (!(flags & RTBVH_FLAG_NO_HOST_MIRROR)) {
    if ((rc = mirror_bvh(*e, s)) != Ok) {
      e->release();
      return rc;
    }
  } else if ((err = cudaStreamSynchronize(s))) {
    e->release();
    return cuda_rc(err);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* raw = e.get();
  uint32_t id = store(std::move(e), false);
  *result = bvh_handle(id, *raw);
  return Ok;
}

// Builds a Bvh entry from device boxes + float4 centres (+ optional device
// triangles, prim-id order) and stores it.
ResultCode build_and_store(const DAabb* d_aabbs, const float4* d_centers, size_t n, size_t ppl, BvhType type,
                           const float* d_vertices, uint32_t flags, cudaStream_t s, RTBvh* result) {
  BuildOutput out;
  ResultCode rc = (type == LocallyOrderedClustered) ? build_locb(d_aabbs, d_centers, n, s, &out)
                                                     : build_binned_sah(d_aabbs, d_centers, n, ppl, s, &out);
  if (rc != Ok) return rc;
  return store_bvh(out, (uint32_t)n, n, type == LocallyOrderedClustered ? 1u : 2u, d_vertices, flags, s, result);
}

// The spatial-split build of device boxes, float4 centres and triangles
// (prim-id order), stored with the triangles (BuildType::Spatial, 3).
ResultCode spatial_and_store(const DAabb* d_aabbs, const float4* d_centers, const float* d_vertices, size_t n,
                             size_t ppl, uint32_t fixes, uint32_t flags, cudaStream_t s, RTBvh* result) {
  BuildOutput out;
  uint32_t slots = 0;
  ResultCode rc = build_spatial_sah(d_aabbs, d_centers, d_vertices, n, ppl, fixes, s, &out, &slots);
  if (rc != Ok) return rc;
  return store_bvh(out, slots, n, 3u, d_vertices, flags, s, result);
}

// ------------------------------------------------------------- host iterators
// Used by the legacy callback entry points only (a host function pointer
// cannot run on the GPU).
struct HRay {
  float o[3], d[3], inv[3];
  float t_min, t;
  int s[3];
};
HRay make_hray(const float* o, const float* d, float t) {
  HRay r;
  for (int i = 0; i < 3; ++i) {
    r.o[i] = o[i];
    r.d[i] = d[i];
    r.inv[i] = 1.0f / d[i];
    r.s[i] = d[i] < 0.0f;
  }
  r.t_min = 1e-4f;
  r.t = t;
  return r;
}

// src/aabb.rs:145-181
bool h_slab_far(const RTAabb& b, const HRay& r, float* out) {
  auto sel = [&](int s, int a) { return s == 0 ? b.min[a] : b.max[a]; };
  float ray_min = (sel(r.s[0], 0) - r.o[0]) * r.inv[0];
  float ray_max = (sel(1 - r.s[0], 0) - r.o[0]) * r.inv[0];
  float y_min = (sel(r.s[1], 1) - r.o[1]) * r.inv[1];
  float y_max = (sel(1 - r.s[1], 1) - r.o[1]) * r.inv[1];
  if ((ray_min > y_max) || (y_min > ray_max)) return false;
  if (y_min > ray_min) ray_min = y_min;
  if (y_max < ray_max) ray_max = y_max;
  float z_min = (sel(r.s[2], 2) - r.o[2]) * r.inv[2];
  float z_max = (sel(1 - r.s[2], 2) - r.o[2]) * r.inv[2];
  if ((ray_min > z_max) || (z_min > ray_max)) return false;
  if (z_max < ray_max) ray_max = z_max;
  if (ray_max > r.t_min) {
    *out = ray_max;
    return true;
  }
  return false;
}

inline float h_sse_min(float a, float b) { return a < b ? a : b; }
inline float h_sse_max(float a, float b) { return a > b ? a : b; }

// src/mbvh_node.rs:176-240
void h_quad(const RTMbvhNode& m, const HRay& r, uint8_t ids[4], bool res[4]) {
  float tmin[4];
  for (int i = 0; i < 4; ++i) {
    float tx0 = (m.min_x[i] - r.o[0]) * r.inv[0], tx1 = (m.max_x[i] - r.o[0]) * r.inv[0];
    float ty0 = (m.min_y[i] - r.o[1]) * r.inv[1], ty1 = (m.max_y[i] - r.o[1]) * r.inv[1];
    float tz0 = (m.min_z[i] - r.o[2]) * r.inv[2], tz1 = (m.max_z[i] - r.o[2]) * r.inv[2];
    float tn = h_sse_max(h_sse_min(tx0, tx1), h_sse_max(h_sse_min(ty0, ty1), h_sse_min(tz0, tz1)));
    float tx = h_sse_min(h_sse_max(tx0, tx1), h_sse_min(h_sse_max(ty0, ty1), h_sse_max(tz0, tz1)));
    tmin[i] = tn;
    res[i] = (tx >= tn) && (tn < r.t);
  }
  uint8_t id[4] = {0, 1, 2, 3};
  auto sw = [&](int a, int b, bool swap_t) {
    if (swap_t) std::swap(tmin[a], tmin[b]);
    std::swap(id[a], id[b]);
  };
  if (tmin[0] > tmin[1]) sw(0, 1, true);
  if (tmin[2] > tmin[3]) sw(2, 3, true);
  if (tmin[0] > tmin[2]) sw(0, 2, true);
  if (tmin[1] > tmin[3]) sw(1, 3, true);
  if (tmin[2] > tmin[3]) sw(2, 3, false);
  for (int i = 0; i < 4; ++i) ids[i] = id[i];
}

// Packet form (4 rays, SoA) of the quad test, src/mbvh_node.rs:242-295.
struct HPacket {
  float o[3][4], inv[3][4];
  float t[4];
};
void h_quad4(const RTMbvhNode& m, const HPacket& p, bool res[4]) {
  const float* mins[3] = {m.min_x, m.min_y, m.min_z};
  const float* maxs[3] = {m.max_x, m.max_y, m.max_z};
  for (int s = 0; s < 4; ++s) res[s] = false;
  for (int i = 0; i < 4; ++i) {  // ray i of the packet
    float tmin[4], tmax[4];
    for (int s = 0; s < 4; ++s) {
      float t1 = (mins[0][s] - p.o[0][i]) * p.inv[0][i], t2 = (maxs[0][s] - p.o[0][i]) * p.inv[0][i];
      tmin[s] = h_sse_min(t1, t2);
      tmax[s] = h_sse_max(t1, t2);
      for (int a = 1; a < 3; ++a) {
        t1 = (mins[a][s] - p.o[a][i]) * p.inv[a][i];
        t2 = (maxs[a][s] - p.o[a][i]) * p.inv[a][i];
        tmin[s] = h_sse_max(tmin[s], h_sse_min(t1, t2));
        tmax[s] = h_sse_min(tmax[s], h_sse_max(t1, t2));
      }
      if ((tmax[s] > tmin[s]) && (tmin[s] < p.t[i])) res[s] = true;
    }
  }
}

// Aabb::intersect4 (src/aabb.rs:217-244): returns the per-ray t_min.
bool h_box4(const RTAabb& b, const HPacket& p, float out[4]) {
  bool any = false;
  for (int i = 0; i < 4; ++i) {
    float t1x = (b.min[0] - p.o[0][i]) * p.inv[0][i], t2x = (b.max[0] - p.o[0][i]) * p.inv[0][i];
    float t1y = (b.min[1] - p.o[1][i]) * p.inv[1][i], t2y = (b.max[1] - p.o[1][i]) * p.inv[1][i];
    float t1z = (b.min[2] - p.o[2][i]) * p.inv[2][i], t2z = (b.max[2] - p.o[2][i]) * p.inv[2][i];
    float tmin = h_sse_max(h_sse_min(t1x, t2x), h_sse_max(h_sse_min(t1y, t2y), h_sse_min(t1z, t2z)));
    float tmax = h_sse_min(h_sse_max(t1x, t2x), h_sse_min(h_sse_max(t1y, t2y), h_sse_max(t1z, t2z)));
    out[i] = tmin;
    if (tmax > 0.0f && tmax > tmin && tmin < p.t[i]) any = true;
  }
  return any;
}

constexpr int kHostStack = 64;

bool finite3(const float* v) { return !(v[0] != v[0] || v[1] != v[1] || v[2] != v[2]); }

}  // namespace

// =================================================================== part 1
extern "C" {

// RTTriangleWrapper (rtbvh_ffi/src/lib.rs:258-336) gathered on the host,
// then the build on the GPU with no corrections.
ResultCode create_spatial_Bvh(const RTAabb* aabbs, uintptr_t prim_count, const float* centers, uintptr_t stride,
                              const float* vertices, uintptr_t vertex_stride, uintptr_t triangle_stride,
                              uint32_t prims_per_leaf, RTBvh* result) {
  if (result == nullptr || centers == nullptr || vertices == nullptr) return Error;
  if (stride % 4 != 0) return Error;  // assert_eq!(stride % 4, 0)
  if (prim_count == 0) return NoPrimitives;
  const size_t n = prim_count;
  const uint32_t vs = (uint32_t)(vertex_stride / 4), cs = (uint32_t)stride;
  std::vector<float> tris(9 * n);
  std::vector<float4> c4(n);
  size_t extent = 0;  // floats the triangles' own vertex reads cover
  for (size_t i = 0; i < n; ++i) {
    const uint32_t off = (uint32_t)(i * triangle_stride / 4);  // vertex0_offset
    for (int k = 0; k < 3; ++k) {
      const uint32_t at = off + (uint32_t)k * vs;
      for (int a = 0; a < 3; ++a) tris[9 * i + 3 * k + a] = vertices[at + a];
      extent = std::max(extent, (size_t)at + 3);
    }
    const float* c = centers + (uint32_t)((uint32_t)i * cs / 4);  // center_i * center_stride / 4 (u32)
    c4[i] = make_float4(c[0], c[1], c[2], 0.0f);
  }
  std::vector<RTAabb> boxes;
  if (aabbs == nullptr) {  // Primitive::aabb of the wrapper (:281-296)
    boxes.resize(n);
    auto mn = [](float a, float b) { return a != a ? b : (b != b ? a : (a < b ? a : (b < a ? b : (std::signbit(a) ? a : b)))); };
    auto mx = [](float a, float b) { return a != a ? b : (b != b ? a : (a > b ? a : (b > a ? b : (std::signbit(a) ? b : a)))); };
    for (size_t i = 0; i < n; ++i) {
      const uint32_t off = (uint32_t)(i * triangle_stride / 4);
      const uint32_t base = off * vs / 4;
      if ((size_t)base + 2 * (size_t)vs + 3 > extent) return InvalidArgument;
      RTAabb b;
      for (int a = 0; a < 3; ++a) {
        b.min[a] = 1e34f;
        b.max[a] = -1e34f;
      }
      b.count = 0;
      b.left_first = 0;
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) {
          const float v = vertices[base + (uint32_t)k * vs + a];
          b.min[a] = mn(b.min[a], v);
          b.max[a] = mx(b.max[a], v);
        }
      boxes[i] = b;
    }
    aabbs = boxes.data();
  }
  cudaStream_t s = legacy_stream();
  Scratch<float> d_t;
  Scratch<DAabb> d_a;
  Scratch<float4> d_c;
  cudaError_t e;
  if ((e = d_t.alloc(9 * n, s)) || (e = d_a.alloc(n, s)) || (e = d_c.alloc(n, s)) ||
      (e = cudaMemcpyAsync(d_t.ptr, tris.data(), 36 * n, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(d_a.ptr, aabbs, 32 * n, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(d_c.ptr, c4.data(), 16 * n, cudaMemcpyHostToDevice, s)))
    return cuda_rc(e);
  return spatial_and_store(d_a.ptr, d_c.ptr, d_t.ptr, n, prims_per_leaf, 0u, 0u, s, result);
}

ResultCode create_bvh(const RTAabb* aabbs, uintptr_t prim_count, const float* centers, uintptr_t center_stride,
                      uintptr_t prims_per_leaf, BvhType bvh_type, RTBvh* result) {
  if (centers == nullptr || result == nullptr) return Error;
  if (center_stride % 4 != 0 || center_stride < 12 || center_stride > 16) return Error;
  if (prim_count == 0) return NoPrimitives;
  if (bvh_type != LocallyOrderedClustered && bvh_type != BinnedSAH) bvh_type = BinnedSAH;  // BvhType::from
  cudaStream_t s = legacy_stream();
  const size_t n = prim_count, stride = center_stride / 4;
  Scratch<float> d_c;
  Scratch<DAabb> d_a;
  Scratch<float4> d_c4;
  cudaError_t e;
  if ((e = d_c.alloc(n * stride, s)) || (e = d_a.alloc(n, s)) || (e = d_c4.alloc(n, s))) return cuda_rc(e);
  if ((e = cudaMemcpyAsync(d_c.ptr, centers, n * center_stride, cudaMemcpyHostToDevice, s))) return cuda_rc(e);
  if (aabbs) {
    if ((e = cudaMemcpyAsync(d_a.ptr, aabbs, n * sizeof(RTAabb), cudaMemcpyHostToDevice, s))) return cuda_rc(e);
    if ((e = launch_pack_centers(d_c.ptr, stride, n, d_c4.ptr, s))) return cuda_rc(e);
  } else {
    if ((e = launch_point_prep(d_c.ptr, stride, n, d_a.ptr, d_c4.ptr, s))) return cuda_rc(e);
  }
  return build_and_store(d_a.ptr, d_c4.ptr, n, prims_per_leaf, bvh_type, nullptr, 0, s, result);
}

ResultCode create_mbvh(RTBvh bvh, RTMbvh* mbvh) {
  if (mbvh == nullptr || bvh.nodes == nullptr || bvh.indices == nullptr) return Error;
  return rtbvh_gpu_create_mbvh(bvh, 0, legacy_stream(), mbvh);
}

ResultCode refit(const RTAabb* aabbs, RTBvh bvh) {
  if (aabbs == nullptr || bvh.nodes == nullptr || bvh.indices == nullptr) return Error;
  cudaStream_t s = legacy_stream();
  uint32_t n;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(bvh.id, false);
    if (!e) return Error;
    n = e->vertex_count;
  }
  Scratch<DAabb> d_a;
  cudaError_t err;
  if ((err = d_a.alloc(n, s)) ||
      (err = cudaMemcpyAsync(d_a.ptr, aabbs, (size_t)n * sizeof(RTAabb), cudaMemcpyHostToDevice, s)))
    return cuda_rc(err);
  return rtbvh_gpu_refit(bvh.id, nullptr, reinterpret_cast<const RTAabb*>(d_a.ptr), UINT32_MAX, s);
}

// rtbvh_ffi/src/lib.rs:551-581 over src/iter_indices.rs:66-107.
ResultCode intersect(RTBvh bvh, const float* origin, const float* direction, float* t, void* user_data,
                     RTIntersectFn cb) {
  if (!finite3(origin) || !finite3(direction)) return Nan;
  HRay r = make_hray(origin, direction, *t);
  const RTBvhNode* nodes = bvh.nodes;
  const uint32_t* idx = bvh.indices;
  if (bvh.node_count == 0 || nodes == nullptr) {
    *t = r.t;
    return Ok;
  }
  int32_t stack[kHostStack];
  stack[0] = 0;
  int32_t sp = 0;
  while (sp >= 0) {
    const RTAabb& nd = nodes[stack[sp--]].aabb;
    if (nd.count > -1) {
      bool stop = false;
      for (int32_t i = 0; i < nd.count && !stop; ++i) stop = cb(idx[nd.left_first + i], &r.t, user_data);
      if (stop) break;
    } else if (nd.left_first > -1) {
      const int32_t lf = nd.left_first;
      float lt = 0, rt = 0;
      bool lh = h_slab_far(nodes[lf].aabb, r, &lt), rh = h_slab_far(nodes[lf + 1].aabb, r, &rt);
      if (sp + 2 >= kHostStack) return StackOverflow;
      if (lh && rh) {
        if (lt < rt) { stack[++sp] = lf; stack[++sp] = lf + 1; }
        else { stack[++sp] = lf + 1; stack[++sp] = lf; }
      } else if (lh) {
        stack[++sp] = lf;
      } else if (rh) {
        stack[++sp] = lf + 1;
      }
    }
  }
  *t = r.t;
  return Ok;
}

// rtbvh_ffi/src/lib.rs:700-731 over src/iter_indices.rs:264-313.
ResultCode intersect_mbvh(RTMbvh bvh, const float* origin, const float* direction, float* t, void* user_data,
                          RTIntersectFn cb) {
  if (!finite3(origin) || !finite3(direction)) return Nan;
  HRay r = make_hray(origin, direction, *t);
  const RTMbvhNode* nodes = bvh.nodes;
  const uint32_t* idx = bvh.indices;
  if (bvh.node_count == 0 || nodes == nullptr) {
    *t = r.t;
    return Ok;
  }
  int32_t stack[kHostStack];
  int32_t sp = -1, current = 0;
  uint8_t ids[4];
  bool res[4];
  h_quad(nodes[0], r, ids, res);
  for (;;) {
    const RTMbvhNode& node = nodes[current];
    bool stop = false;
    for (int i = 0; i < 4 && !stop; ++i) {
      int id = ids[3 - i];
      if (!res[id]) continue;
      int32_t count = node.counts[id], lf = node.children[id];
      if (count > -1) {
        for (int32_t j = 0; j < count && !stop; ++j) stop = cb(idx[lf + j], &r.t, user_data);
      } else if (lf > -1) {
        if (sp + 1 >= kHostStack) return StackOverflow;
        stack[++sp] = lf;
      }
    }
    if (stop || sp < 0) break;
    current = stack[sp--];
    h_quad(nodes[current], r, ids, res);
  }
  *t = r.t;
  return Ok;
}

static bool load_packet(const float* ox, const float* oy, const float* oz, const float* dx, const float* dy,
                        const float* dz, const float* t, HPacket& p) {
  const float* o[3] = {ox, oy, oz};
  const float* d[3] = {dx, dy, dz};
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < 4; ++i) {
      if (o[a][i] != o[a][i] || d[a][i] != d[a][i]) return false;
      p.o[a][i] = o[a][i];
      p.inv[a][i] = 1.0f / d[a][i];
    }
  for (int i = 0; i < 4; ++i) p.t[i] = t[i];
  return true;
}

// rtbvh_ffi/src/lib.rs:599-686 over src/iter_indices.rs:169-210 (packet
// traversal is not part of the GPU path; this is the host compatibility form).
ResultCode intersect_packet(RTBvh bvh, const float* origin_x, const float* origin_y, const float* origin_z,
                            const float* direction_x, const float* direction_y, const float* direction_z, float* t,
                            void* user_data, RTIntersectFn cb) {
  HPacket p;
  if (!load_packet(origin_x, origin_y, origin_z, direction_x, direction_y, direction_z, t, p)) return Nan;
  const RTBvhNode* nodes = bvh.nodes;
  const uint32_t* idx = bvh.indices;
  if (bvh.node_count > 0 && nodes) {
    int32_t stack[kHostStack];
    stack[0] = 0;
    int32_t sp = 0;
    while (sp >= 0) {
      const RTAabb& nd = nodes[stack[sp--]].aabb;
      if (nd.count > -1) {
        bool stop = false;
        for (int32_t i = 0; i < nd.count && !stop; ++i) stop = cb(idx[nd.left_first + i], p.t, user_data);
        if (stop) break;
      } else if (nd.left_first > -1) {
        const int32_t lf = nd.left_first;
        float lt[4], rt[4];
        bool lh = h_box4(nodes[lf].aabb, p, lt), rh = h_box4(nodes[lf + 1].aabb, p, rt);
        if (sp + 2 >= kHostStack) return StackOverflow;
        if (lh && rh) {
          bool any_less = false;
          for (int i = 0; i < 4; ++i) any_less = any_less || (lt[i] < rt[i]);
          if (any_less) { stack[++sp] = lf; stack[++sp] = lf + 1; }
          else { stack[++sp] = lf + 1; stack[++sp] = lf; }
        } else if (lh) {
          stack[++sp] = lf;
        } else if (rh) {
          stack[++sp] = lf + 1;
        }
      }
    }
  }
  for (int i = 0; i < 4; ++i) t[i] = p.t[i];
  return Ok;
}

// rtbvh_ffi/src/lib.rs:749-835 over src/iter_indices.rs:367-414.
ResultCode intersect_mbvh_packet(RTMbvh bvh, const float* origin_x, const float* origin_y, const float* origin_z,
                                 const float* direction_x, const float* direction_y, const float* direction_z,
                                 float* t, void* user_data, RTIntersectFn cb) {
  HPacket p;
  if (!load_packet(origin_x, origin_y, origin_z, direction_x, direction_y, direction_z, t, p)) return Nan;
  const RTMbvhNode* nodes = bvh.nodes;
  const uint32_t* idx = bvh.indices;
  if (bvh.node_count > 0 && nodes) {
    int32_t stack[kHostStack];
    int32_t sp = -1, current = 0;
    bool res[4];
    h_quad4(nodes[0], p, res);
    for (;;) {
      const RTMbvhNode& node = nodes[current];
      bool stop = false;
      for (int i = 0; i < 4 && !stop; ++i) {
        int id = 3 - i;
        if (!res[id]) continue;
        int32_t count = node.counts[id], lf = node.children[id];
        if (count > -1) {
          for (int32_t j = 0; j < count && !stop; ++j) stop = cb(idx[lf + j], p.t, user_data);
        } else if (lf > -1) {
          if (sp + 1 >= kHostStack) return StackOverflow;
          stack[++sp] = lf;
        }
      }
      if (stop || sp < 0) break;
      current = stack[sp--];
      h_quad4(nodes[current], p, res);
    }
  }
  for (int i = 0; i < 4; ++i) t[i] = p.t[i];
  return Ok;
}

void free_bvh(RTBvh bvh) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (bvh.id < g_bvh.size() && g_bvh[bvh.id]) {
    g_bvh[bvh.id]->release();
  } else {
    fprintf(stderr, "Could not free bvh with id: %u\n", bvh.id);
  }
}

void free_mbvh(RTMbvh bvh) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (bvh.id < g_mbvh.size() && g_mbvh[bvh.id]) {
    g_mbvh[bvh.id]->release();
  } else {
    fprintf(stderr, "Could not free bvh with id: %u\n", bvh.id);
  }
}

// =================================================================== part 2

ResultCode rtbvh_gpu_create_bvh_from_triangles(const float* vertices, uintptr_t prim_count, uintptr_t prims_per_leaf,
                                               BvhType bvh_type, uint32_t flags, rtbvh_stream_t stream,
                                               RTBvh* result) {
  if (result == nullptr || (vertices == nullptr && prim_count > 0)) return Error;
  if (prim_count == 0) return NoPrimitives;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch<DAabb> d_a;
  Scratch<float4> d_c4;
  cudaError_t e;
  if ((e = d_a.alloc(prim_count, s)) || (e = d_c4.alloc(prim_count, s))) return cuda_rc(e);
  if ((e = launch_triangle_prep(vertices, prim_count, d_a.ptr, d_c4.ptr, s))) return cuda_rc(e);
  return build_and_store(d_a.ptr, d_c4.ptr, prim_count, prims_per_leaf, bvh_type, vertices, flags, s, result);
}

ResultCode rtbvh_gpu_create_spatial_bvh(const float* vertices, uintptr_t prim_count, const RTAabb* aabbs,
                                        const float* centers, uintptr_t center_stride, uintptr_t prims_per_leaf,
                                        uint32_t fixes, uint32_t flags, rtbvh_stream_t stream, RTBvh* result) {
  if (result == nullptr || (vertices == nullptr && prim_count > 0)) return Error;
  if (centers && (center_stride % 4 != 0 || center_stride < 12 || center_stride > 16)) return Error;
  if (fixes & ~RTBVH_SPATIAL_FIX_ALL) return InvalidArgument;
  if (prim_count == 0) return NoPrimitives;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch<DAabb> d_a;
  Scratch<float4> d_c4;
  cudaError_t e;
  if ((e = d_a.alloc(prim_count, s)) || (e = d_c4.alloc(prim_count, s))) return cuda_rc(e);
  if ((e = launch_triangle_prep(vertices, prim_count, d_a.ptr, d_c4.ptr, s))) return cuda_rc(e);
  if (centers && (e = launch_pack_centers(centers, center_stride / 4, prim_count, d_c4.ptr, s))) return cuda_rc(e);
  const DAabb* boxes = aabbs ? reinterpret_cast<const DAabb*>(aabbs) : d_a.ptr;
  return spatial_and_store(boxes, d_c4.ptr, vertices, prim_count, prims_per_leaf, fixes, flags, s, result);
}

ResultCode rtbvh_gpu_create_bvh(const RTAabb* aabbs, uintptr_t prim_count, const float* centers,
                                uintptr_t center_stride, uintptr_t prims_per_leaf, BvhType bvh_type, uint32_t flags,
                                rtbvh_stream_t stream, RTBvh* result) {
  if (result == nullptr || centers == nullptr || aabbs == nullptr) return Error;
  if (center_stride % 4 != 0 || center_stride < 12 || center_stride > 16) return Error;
  if (prim_count == 0) return NoPrimitives;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch<float4> d_c4;
  cudaError_t e;
  if ((e = d_c4.alloc(prim_count, s))) return cuda_rc(e);
  if ((e = launch_pack_centers(centers, center_stride / 4, prim_count, d_c4.ptr, s))) return cuda_rc(e);
  return build_and_store(reinterpret_cast<const DAabb*>(aabbs), d_c4.ptr, prim_count, prims_per_leaf, bvh_type,
                         nullptr, flags, s, result);
}

ResultCode rtbvh_gpu_create_mbvh(RTBvh bvh, uint32_t flags, rtbvh_stream_t stream, RTMbvh* result) {
  if (result == nullptr) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DAabb* d_nodes;
  uint32_t node_count, prim_count, vertex_count, build_type;
  bool lower_bound, cover;
  const uint32_t* d_indices;
  const float4* d_tris;
  const float* d_vertices;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* src = lookup(bvh.id, false);
    if (!src) return Error;
    d_nodes = src->d_nodes;
    node_count = src->node_count;
    prim_count = src->prim_count;
    vertex_count = src->vertex_count;
    lower_bound = src->vertex_lower_bound;
    build_type = src->build_type;
    cover = src->boxes_cover;
    d_indices = src->d_indices;
    d_tris = src->d_tris;
    d_vertices = src->d_vertices;
  }
  auto e = std::make_unique<Entry>();
  e->alive = true;
  e->prim_count = prim_count;
  e->vertex_count = vertex_count;
  e->vertex_lower_bound = lower_bound;
  e->build_type = build_type;
  e->boxes_cover = cover;
  e->source_bvh = bvh.id;
  ResultCode rc;
  cudaError_t err;
  e->bvh_node_count = node_count;
  if ((err = device_alloc(&e->d_status, 4, s)) || (err = cudaMemsetAsync(e->d_status, 0, 16, s)) ||
      (err = device_alloc(&e->d_indices, prim_count, s)) ||
      (err = cudaMemcpyAsync(e->d_indices, d_indices, (size_t)prim_count * 4, cudaMemcpyDeviceToDevice, s)) ||
      (err = device_alloc(&e->d_nodes, node_count, s)) ||
      (err = cudaMemcpyAsync(e->d_nodes, d_nodes, (size_t)node_count * sizeof(DAabb), cudaMemcpyDeviceToDevice,
                             s))) {
    e->release();
    return cuda_rc(err);
  }
  if (d_tris) {
    if ((err = device_alloc(&e->d_tris, (size_t)kTriFloat4 * prim_count, s)) ||
        (err = cudaMemcpyAsync(e->d_tris, d_tris, 16 * (size_t)kTriFloat4 * prim_count, cudaMemcpyDeviceToDevice,
                               s)) ||
        (err = device_alloc(&e->d_vertices, 9 * (size_t)vertex_count, s)) ||
        (err = cudaMemcpyAsync(e->d_vertices, d_vertices, 36 * (size_t)vertex_count, cudaMemcpyDeviceToDevice,
                               s))) {
      e->release();
      return cuda_rc(err);
    }
  }
  if ((rc = collapse_entry(*e, s, &e->d_mnodes, &e->node_count)) != Ok) {
    e->release();
    return rc;
  }
  if (!(flags & RTBVH_FLAG_NO_HOST_MIRROR)) {
    if ((rc = mirror_mbvh(*e, s)) != Ok) {
      e->release();
      return rc;
    }
  } else if ((err = cudaStreamSynchronize(s))) {
    e->release();
    return cuda_rc(err);
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* raw = e.get();
  uint32_t id = store(std::move(e), true);
  *result = mbvh_handle(id, *raw);
  return Ok;
}

ResultCode rtbvh_gpu_set_triangles(uint32_t structure_id, int is_mbvh, const float* vertices, uintptr_t prim_count,
                                   rtbvh_stream_t stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* e = lookup(structure_id, is_mbvh != 0);
  if (!e || vertices == nullptr) return Error;
  // a structure loaded from bytes knows only a lower bound of its
  // primitive count (its largest index + 1)
  if (e->vertex_lower_bound ? prim_count < e->vertex_count : prim_count != e->vertex_count)
    return InequalAabbsAndPrimitives;
  cudaError_t err;
  if (e->d_vertices && prim_count != e->vertex_count) {
    void* const old_arrays[] = {e->d_vertices};
    pool_free_now(old_arrays, 1);
    e->d_vertices = nullptr;
  }
  e->vertex_count = (uint32_t)prim_count;
  e->vertex_lower_bound = false;
  if (!e->d_vertices && (err = device_alloc(&e->d_vertices, 9 * (size_t)prim_count, s))) return cuda_rc(err);
  if (!e->d_tris && (err = device_alloc(&e->d_tris, (size_t)kTriFloat4 * e->prim_count, s))) return cuda_rc(err);
  if ((err = cudaMemcpyAsync(e->d_vertices, vertices, 36 * (size_t)prim_count, cudaMemcpyDeviceToDevice, s)) ||
      (err = launch_gather_triangles(e->d_vertices, e->d_indices, e->prim_count, e->d_tris, s)))
    return cuda_rc(err);
  // the boxes promise nothing about these triangles: an Mbvh's traversal
  // tree is rebuilt from them (gated where the boxes miss them)
  e->boxes_cover = false;
  if (!is_mbvh) return Ok;
  {
    // the old tree may still be read by traversals on other streams
    void* const old_arrays[] = {e->d_qnodes, e->d_wnodes, e->d_tboxes};
    pool_free_now(old_arrays, 3);
  }
  // the quad nodes come out as they are (same BVH2 nodes); only the
  // traversal tree and the escape flags are kept
  DMNode* same = nullptr;
  uint32_t count = 0;
  const ResultCode rc = collapse_entry(*e, s, &same, &count);
  pool_free(same, s);
  return rc;
}

static ResultCode trace_common(uint32_t id, bool mbvh, const float* rays, const float* t_max, uintptr_t ray_count,
                               float* hits, uint32_t flags, uint32_t* stats, cudaStream_t s) {
  TraceArgs a;
  const bool walk_stats = (flags & RTBVH_TRACE_WALK_STATS) != 0;
  if (walk_stats && (!mbvh || (flags & (RTBVH_TRACE_STATS | RTBVH_TRACE_ANY_HIT | RTBVH_TRACE_EXACT_NODES |
                                        RTBVH_TRACE_REORDER))))
    return InvalidArgument;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(id, mbvh);
    if (!e) return Error;
    if (!e->d_tris && e->node_count > 0) return InvalidArgument;
    a.mnodes = e->d_mnodes;
    if (!(flags & RTBVH_TRACE_EXACT_NODES) && mbvh) {
      a.qnodes = e->d_qnodes;
      a.qexact = e->d_wnodes;
      a.q_count = e->wcount;
      a.q_gates = e->q_gates;
      a.tboxes = e->q_gates ? e->d_tboxes : nullptr;
    }
    if (walk_stats && (a.qnodes == nullptr || a.q_count == 0)) return InvalidArgument;
    a.nodes = e->d_nodes;
    a.node_count = e->node_count;
    a.tris = e->d_tris;
    a.prim_count = e->prim_count;
    a.status = e->d_status;
  }
  if (ray_count == 0) return Ok;
  if (rays == nullptr || hits == nullptr) return Error;
  a.rays = rays;
  a.t_max = t_max;
  a.ray_count = ray_count;
  a.hits = reinterpret_cast<float4*>(hits);
  if (walk_stats && stats == nullptr) return Error;
  a.stats = (flags & RTBVH_TRACE_STATS) ? stats : nullptr;
  a.walk_stats = walk_stats ? stats : nullptr;
  a.any_hit = (flags & RTBVH_TRACE_ANY_HIT) != 0;
  a.reorder = (flags & RTBVH_TRACE_REORDER) != 0;
  cudaError_t err = mbvh ? launch_trace_mbvh(a, s) : launch_trace_bvh(a, s);
  return cuda_rc(err);
}

ResultCode rtbvh_gpu_intersect_mbvh(RTMbvh mbvh, const float* rays, const float* t_max, uintptr_t ray_count,
                                    float* hits, uint32_t flags, uint32_t* stats, rtbvh_stream_t stream) {
  return trace_common(mbvh.id, true, rays, t_max, ray_count, hits, flags, stats, static_cast<cudaStream_t>(stream));
}

ResultCode rtbvh_gpu_intersect_bvh(RTBvh bvh, const float* rays, const float* t_max, uintptr_t ray_count,
                                   float* hits, uint32_t flags, uint32_t* stats, rtbvh_stream_t stream) {
  return trace_common(bvh.id, false, rays, t_max, ray_count, hits, flags, stats, static_cast<cudaStream_t>(stream));
}

static ResultCode packets_common(uint32_t id, bool mbvh, const float* const origin[3],
                                 const float* const direction[3], float* t, uintptr_t packet_count, float* hits,
                                 uint32_t flags, uint32_t* stats, cudaStream_t s) {
  if (flags & (RTBVH_TRACE_ANY_HIT | RTBVH_TRACE_REORDER)) return InvalidArgument;
  PacketArgs a;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(id, mbvh);
    if (!e) return Error;
    if (!e->d_tris && e->node_count > 0) return InvalidArgument;
    a.mnodes = e->d_mnodes;
    a.nodes = e->d_nodes;
    a.node_count = e->node_count;
    a.tris = e->d_tris;
    a.prim_count = e->prim_count;
    a.status = e->d_status;
  }
  if (packet_count == 0) return Ok;
  for (int k = 0; k < 3; ++k) {
    if (origin[k] == nullptr || direction[k] == nullptr) return Error;
    a.origin[k] = origin[k];
    a.direction[k] = direction[k];
  }
  if (t == nullptr) return Error;
  if ((flags & RTBVH_TRACE_STATS) && stats == nullptr) return Error;
  a.t = t;
  a.packet_count = packet_count;
  a.hits = reinterpret_cast<float4*>(hits);
  a.stats = (flags & RTBVH_TRACE_STATS) ? stats : nullptr;
  return cuda_rc(launch_trace_packets(a, mbvh, s));
}

ResultCode rtbvh_gpu_intersect_mbvh_packets(RTMbvh mbvh, const float* origin_x, const float* origin_y,
                                            const float* origin_z, const float* direction_x, const float* direction_y,
                                            const float* direction_z, float* t, uintptr_t packet_count, float* hits,
                                            uint32_t flags, uint32_t* stats, rtbvh_stream_t stream) {
  const float* o[3] = {origin_x, origin_y, origin_z};
  const float* d[3] = {direction_x, direction_y, direction_z};
  return packets_common(mbvh.id, true, o, d, t, packet_count, hits, flags, stats, static_cast<cudaStream_t>(stream));
}

ResultCode rtbvh_gpu_intersect_bvh_packets(RTBvh bvh, const float* origin_x, const float* origin_y,
                                           const float* origin_z, const float* direction_x, const float* direction_y,
                                           const float* direction_z, float* t, uintptr_t packet_count, float* hits,
                                           uint32_t flags, uint32_t* stats, rtbvh_stream_t stream) {
  const float* o[3] = {origin_x, origin_y, origin_z};
  const float* d[3] = {direction_x, direction_y, direction_z};
  return packets_common(bvh.id, false, o, d, t, packet_count, hits, flags, stats, static_cast<cudaStream_t>(stream));
}

static ResultCode candidates_common(uint32_t id, bool mbvh, const float* rays, const float* t_max,
                                    uintptr_t ray_count, uint32_t max_per_ray, uint32_t* candidates,
                                    uint32_t* counts, cudaStream_t s) {
  CandArgs a;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(id, mbvh);
    if (!e) return Error;
    a.mnodes = e->d_mnodes;
    a.nodes = e->d_nodes;
    a.node_count = e->node_count;
    a.indices = e->d_indices;
    a.prim_count = e->prim_count;
    a.status = e->d_status;
  }
  if (ray_count == 0) return Ok;
  if (rays == nullptr || counts == nullptr) return Error;
  if (candidates != nullptr && max_per_ray == 0) return InvalidArgument;
  a.rays = rays;
  a.t_max = t_max;
  a.ray_count = ray_count;
  a.max_per_ray = candidates ? max_per_ray : 0u;
  a.out = candidates;
  a.counts = counts;
  return cuda_rc(launch_candidates(a, mbvh, s));
}

ResultCode rtbvh_gpu_mbvh_candidates(RTMbvh mbvh, const float* rays, const float* t_max, uintptr_t ray_count,
                                     uint32_t max_per_ray, uint32_t* candidates, uint32_t* counts,
                                     rtbvh_stream_t stream) {
  return candidates_common(mbvh.id, true, rays, t_max, ray_count, max_per_ray, candidates, counts,
                           static_cast<cudaStream_t>(stream));
}

ResultCode rtbvh_gpu_bvh_candidates(RTBvh bvh, const float* rays, const float* t_max, uintptr_t ray_count,
                                    uint32_t max_per_ray, uint32_t* candidates, uint32_t* counts,
                                    rtbvh_stream_t stream) {
  return candidates_common(bvh.id, false, rays, t_max, ray_count, max_per_ray, candidates, counts,
                           static_cast<cudaStream_t>(stream));
}

// Chunk schedule of the host-buffer trace: a small first chunk so that the
// GPU starts after a short upload, large middle chunks (few launch tails),
// and a small last chunk so that the final download is short (1M, 3M, then
// 6M rays, the remainder split to end with 1M).
static size_t next_chunk(size_t done, size_t remaining) {
  const size_t M = (size_t)1 << 20;
  if (remaining <= 2 * M) return remaining;
  if (done == 0) return M;
  if (done == M) return remaining > 4 * M ? 3 * M : remaining - M;
  if (remaining > 7 * M) return 6 * M;
  return remaining - M;
}

// Device address of page-locked host memory the GPU can read and write
// directly (pinned and mapped into the device's address space), else NULL.
static const void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (p == nullptr || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

ResultCode rtbvh_intersect_mbvh_batch(RTMbvh mbvh, const float* rays, const float* t_max, uintptr_t ray_count,
                                      float* hits, uint32_t flags) {
  if (ray_count == 0) return Ok;
  if (rays == nullptr || hits == nullptr) return Error;
  static cudaStream_t streams[2] = {nullptr, nullptr};
  static std::once_flag once;
  std::call_once(once, []() {
    cudaStreamCreateWithFlags(&streams[0], cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&streams[1], cudaStreamNonBlocking);
  });
  cudaError_t e;
  // Pinned, mapped host buffers: the traversal reads the rays and writes the
  // hits in host memory itself (40 bytes per ray over the CPU-GPU link,
  // overlapped with the walk), no staging copies.
  {
    const float* dr = static_cast<const float*>(mapped_host(rays));
    float* dh = static_cast<float*>(const_cast<void*>(mapped_host(hits)));
    const float* dt = t_max ? static_cast<const float*>(mapped_host(t_max)) : nullptr;
    if (dr && dh && (t_max == nullptr || dt)) {
      ResultCode rc = trace_common(mbvh.id, true, dr, dt, ray_count, dh, flags & ~(RTBVH_TRACE_STATS | RTBVH_TRACE_WALK_STATS), nullptr,
                                   streams[0]);
      if ((e = cudaStreamSynchronize(streams[0]))) return cuda_rc(e);
      return rc;
    }
  }
  size_t per = 0;
  for (size_t done = 0; done < ray_count;) {
    const size_t c = next_chunk(done, ray_count - done);
    per = c > per ? c : per;
    done += c;
  }
  Scratch<float> d_rays[2], d_tmax[2];
  Scratch<float4> d_hits[2];
  for (int k = 0; k < 2; ++k) {
    if ((e = d_rays[k].alloc(6 * per, streams[k])) || (e = d_hits[k].alloc(per, streams[k]))) return cuda_rc(e);
    if (t_max && (e = d_tmax[k].alloc(per, streams[k]))) return cuda_rc(e);
  }
  ResultCode rc = Ok;
  int k = 0;
  for (size_t c0 = 0; c0 < ray_count; k ^= 1) {
    const size_t cnt = next_chunk(c0, ray_count - c0);
    cudaStream_t s = streams[k];
    if ((e = cudaMemcpyAsync(d_rays[k].ptr, rays + 6 * c0, 24 * cnt, cudaMemcpyHostToDevice, s))) return cuda_rc(e);
    if (t_max && (e = cudaMemcpyAsync(d_tmax[k].ptr, t_max + c0, 4 * cnt, cudaMemcpyHostToDevice, s)))
      return cuda_rc(e);
    rc = trace_common(mbvh.id, true, d_rays[k].ptr, t_max ? d_tmax[k].ptr : nullptr, cnt,
                      reinterpret_cast<float*>(d_hits[k].ptr), flags & ~(RTBVH_TRACE_STATS | RTBVH_TRACE_WALK_STATS), nullptr, s);
    if (rc != Ok) break;
    if ((e = cudaMemcpyAsync(hits + 4 * c0, d_hits[k].ptr, 16 * cnt, cudaMemcpyDeviceToHost, s))) return cuda_rc(e);
    c0 += cnt;
  }
  if ((e = cudaStreamSynchronize(streams[0])) || (e = cudaStreamSynchronize(streams[1]))) return cuda_rc(e);
  return rc;
}

ResultCode rtbvh_gpu_status(uint32_t structure_id, int is_mbvh) {
  uint32_t* d_status;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(structure_id, is_mbvh != 0);
    if (!e) return Error;
    d_status = e->d_status;
  }
  uint32_t st = 0;
  cudaError_t err;
  if ((err = cudaDeviceSynchronize()) || (err = cudaMemcpy(&st, d_status, 4, cudaMemcpyDeviceToHost)) ||
      (err = cudaMemset(d_status, 0, 4)))
    return cuda_rc(err);
  if (st & kStatusStackOverflow) return StackOverflow;
  if (st & kStatusTimeout) return Timeout;
  if (st) return Error;
  return Ok;
}

ResultCode rtbvh_gpu_view(uint32_t structure_id, int is_mbvh, RTGpuView* view) {
  if (view == nullptr) return Error;
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* e = lookup(structure_id, is_mbvh != 0);
  if (!e) return Error;
  view->nodes = is_mbvh ? static_cast<const void*>(e->d_mnodes) : static_cast<const void*>(e->d_nodes);
  view->node_count = e->node_count;
  view->indices = e->d_indices;
  view->index_count = e->prim_count;
  view->leaf_triangles = reinterpret_cast<const float*>(e->d_tris);
  return Ok;
}

ResultCode rtbvh_gpu_traversal_tree(RTMbvh mbvh, const RTMbvhNode** exact, const void** compact, uint32_t* count) {
  if (exact == nullptr || compact == nullptr || count == nullptr) return Error;
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* e = lookup(mbvh.id, true);
  if (!e) return Error;
  *exact = reinterpret_cast<const RTMbvhNode*>(e->d_wnodes);
  *compact = e->d_qnodes;
  *count = e->wcount;
  return Ok;
}

// Re-collapses Mbvh entry m from BVH2 nodes after a refit: fresh quad nodes
// (same count and topology), a fresh traversal tree, triangles re-laid from
// `vertices` when given, and the host mirror refreshed.
static ResultCode recollapse(Entry* m, const float* vertices, cudaStream_t s) {
  const size_t n = m->vertex_count, slots = m->prim_count;
  ResultCode rc;
  cudaError_t err;
  {
    // the old arrays may still be read by traversals on other streams
    void* const old_arrays[] = {m->d_mnodes, m->d_qnodes, m->d_wnodes, m->d_tboxes};
    pool_free_now(old_arrays, 4);
  }
  const uint32_t expected = m->node_count;
  m->d_mnodes = nullptr;
  m->d_qnodes = nullptr;
  m->d_wnodes = nullptr;
  m->d_tboxes = nullptr;
  m->wcount = 0;
  m->q_gates = false;
  if (vertices) {
    if (!m->d_vertices && (err = device_alloc(&m->d_vertices, 9 * n, s))) return cuda_rc(err);
    if (!m->d_tris && (err = device_alloc(&m->d_tris, (size_t)kTriFloat4 * slots, s))) return cuda_rc(err);
    if ((err = cudaMemcpyAsync(m->d_vertices, vertices, 36 * n, cudaMemcpyDeviceToDevice, s)) ||
        (err = launch_gather_triangles(m->d_vertices, m->d_indices, slots, m->d_tris, s)))
      return cuda_rc(err);
  }
  // recollapse follows a refit: from triangles, every box now contains
  // them; from boxes, the attached triangles (if any) may lie outside
  m->boxes_cover = vertices != nullptr;
  DMNode* fresh = nullptr;
  uint32_t count = 0;
  if ((rc = collapse_entry(*m, s, &fresh, &count)) != Ok) {
    pool_free(fresh, s);
    return rc;
  }
  m->d_mnodes = fresh;
  m->node_count = count;
  if (count != expected) return Error;  // same topology, same quad count
  if (m->mirrored && (rc = mirror_mbvh(*m, s)) != Ok) return rc;
  return Ok;
}

// New primitive boxes from device triangles (written to `boxes`) or taken
// from device aabbs.
static cudaError_t refit_boxes(const float* vertices, const RTAabb* aabbs, size_t n, Scratch<DAabb>& d_a,
                               Scratch<float4>& d_c4, const DAabb** boxes, cudaStream_t s) {
  *boxes = reinterpret_cast<const DAabb*>(aabbs);
  if (!vertices) return cudaSuccess;
  cudaError_t err;
  if ((err = d_a.alloc(n, s)) || (err = d_c4.alloc(n, s))) return err;
  if ((err = launch_triangle_prep(vertices, n, d_a.ptr, d_c4.ptr, s))) return err;
  *boxes = d_a.ptr;
  return cudaSuccess;
}

ResultCode rtbvh_gpu_refit_mbvh(uint32_t mbvh_id, const float* vertices, const RTAabb* aabbs, rtbvh_stream_t stream) {
  if ((vertices == nullptr) == (aabbs == nullptr)) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* m = lookup(mbvh_id, true);
  if (!m || !m->d_nodes) return Error;
  Scratch<DAabb> d_a;
  Scratch<float4> d_c4;
  const DAabb* boxes = nullptr;
  cudaError_t err;
  if ((err = refit_boxes(vertices, aabbs, m->vertex_count, d_a, d_c4, &boxes, s))) return cuda_rc(err);
  ResultCode rc = refit_bvh(m->d_nodes, m->bvh_node_count, m->d_indices, m->prim_count, m->vertex_count, boxes, s);
  if (rc != Ok) return rc;
  return recollapse(m, vertices, s);
}

ResultCode rtbvh_gpu_refit(uint32_t bvh_id, const float* vertices, const RTAabb* aabbs, uint32_t mbvh_id,
                           rtbvh_stream_t stream) {
  if ((vertices == nullptr) == (aabbs == nullptr)) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* b = lookup(bvh_id, false);
  if (!b) return Error;
  Entry* m = nullptr;
  if (mbvh_id != UINT32_MAX) {
    m = lookup(mbvh_id, true);
    if (!m || m->source_bvh != bvh_id) return Error;
  }
  const size_t n = b->vertex_count;
  Scratch<DAabb> d_a;
  Scratch<float4> d_c4;
  const DAabb* boxes = reinterpret_cast<const DAabb*>(aabbs);
  cudaError_t err;
  if (vertices) {
    if ((err = d_a.alloc(n, s)) || (err = d_c4.alloc(n, s))) return cuda_rc(err);
    if ((err = launch_triangle_prep(vertices, n, d_a.ptr, d_c4.ptr, s))) return cuda_rc(err);
    boxes = d_a.ptr;
    if (b->d_vertices) {
      if ((err = cudaMemcpyAsync(b->d_vertices, vertices, 36 * n, cudaMemcpyDeviceToDevice, s)) ||
          (err = launch_gather_triangles(b->d_vertices, b->d_indices, b->prim_count, b->d_tris, s)))
        return cuda_rc(err);
    }
  }
  ResultCode rc = refit_bvh(b->d_nodes, b->node_count, b->d_indices, b->prim_count, b->vertex_count, boxes, s);
  if (rc != Ok) return rc;
  b->boxes_cover = vertices != nullptr;
  if (m) {
    if (m->d_nodes && (err = cudaMemcpyAsync(m->d_nodes, b->d_nodes, (size_t)b->node_count * sizeof(DAabb),
                                             cudaMemcpyDeviceToDevice, s)))
      return cuda_rc(err);
    if ((rc = recollapse(m, vertices, s)) != Ok) return rc;
  }
  if (b->mirrored && (rc = mirror_bvh(*b, s)) != Ok) return rc;
  return Ok;
}

ResultCode rtbvh_gpu_refit_noalloc(uint32_t bvh_id, const RTAabb* aabbs, rtbvh_stream_t stream) {
  if (aabbs == nullptr) return Error;
  // The structure lock is held while the (asynchronous) work is queued, so a
  // concurrent free_bvh cannot release the arrays in between; the queued
  // kernels report index errors in the Bvh's own status word, which
  // rtbvh_gpu_status reads.
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* b = lookup(bvh_id, false);
  if (!b) return Error;
  const ResultCode rc = refit_bvh_noalloc(b->d_nodes, b->node_count, b->d_indices, b->prim_count, b->vertex_count,
                                          reinterpret_cast<const DAabb*>(aabbs), b->d_status,
                                          static_cast<cudaStream_t>(stream));
  // boxes from aabbs promise nothing about attached triangles
  b->boxes_cover = false;
  return rc;
}

ResultCode rtbvh_gpu_intersect_backward(const float* vertices, uintptr_t prim_count, const float* rays,
                                        const float* hits, const float* grad_tuv, uintptr_t ray_count,
                                        float* grad_vertices, float* grad_rays, rtbvh_stream_t stream) {
  if (vertices == nullptr || rays == nullptr || hits == nullptr || grad_tuv == nullptr || grad_vertices == nullptr)
    return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return cuda_rc(launch_intersect_backward(vertices, prim_count, rays, reinterpret_cast<const float4*>(hits),
                                           grad_tuv, ray_count, grad_vertices, grad_rays, s));
}

const char* rtbvh_gpu_version(void) { return "rtbvh-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"

// ============================================================ on-disk format
// The serde derives of the crate (src/bvh.rs:141-147, :318-324,
// src/bvh_node.rs:9-14, src/mbvh_node.rs:26-38, src/aabb.rs:12-20) encoded
// with bincode 1's default options: little-endian fixed-width integers, a
// u64 length before every Vec, glam's Vec3 as three f32, enums as a u32
// variant index. So a BvhNode is the 32-byte RTAabb record, an MbvhNode the
// 128-byte RTMbvhNode record, and
//   Bvh  = u64 N, N nodes, u64 M, M u32 indices, u32 BuildType
//   Mbvh = u64 N, N nodes, u64 Q, Q quad nodes, u64 M, M u32 indices
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "the serialized layout assumes a little-endian host"
#endif

namespace {

struct ByteWriter {
  uint8_t* out;
  size_t cap, n = 0;
  void put(const void* src, size_t k) {
    if (out && n + k <= cap) std::memcpy(out + n, src, k);
    n += k;
  }
  void u64(uint64_t v) { put(&v, 8); }
  void u32(uint32_t v) { put(&v, 4); }
};

struct ByteReader {
  const uint8_t* in;
  size_t size, n = 0;
  bool ok = true;
  const uint8_t* take(size_t k) {
    if (!ok || k > size - n) {
      ok = false;
      return nullptr;
    }
    const uint8_t* p = in + n;
    n += k;
    return p;
  }
  uint64_t u64() {
    uint64_t v = 0;
    if (const uint8_t* p = take(8)) std::memcpy(&v, p, 8);
    return v;
  }
  uint32_t u32() {
    uint32_t v = 0;
    if (const uint8_t* p = take(4)) std::memcpy(&v, p, 4);
    return v;
  }
};

template <class T>
ResultCode fetch_device(std::vector<T>& out, const T* d, size_t count) {
  out.resize(count);
  if (count == 0) return Ok;
  cudaError_t e;
  if ((e = cudaDeviceSynchronize()) || (e = cudaMemcpy(out.data(), d, count * sizeof(T), cudaMemcpyDeviceToHost)))
    return cuda_rc(e);
  return Ok;
}

// Leaf ranges inside [0, prim_count), children pairs inside the node array.
bool nodes_valid(const RTAabb* nodes, uint64_t count, uint64_t prim_count) {
  for (uint64_t i = 0; i < count; ++i) {
    const RTAabb& b = nodes[i];
    if (b.count >= 0) {
      if (b.left_first < 0 || (uint64_t)b.left_first + (uint64_t)b.count > prim_count) return false;
    } else if (b.left_first >= 0 && (uint64_t)b.left_first + 1 >= count) {
      return false;
    }
  }
  return true;
}

bool indices_valid(const uint32_t* idx, uint64_t count) {
  for (uint64_t i = 0; i < count; ++i)
    if (idx[i] >= count) return false;
  return true;
}

// Uploads nodes and indices into a new entry (status word, host mirror).
ResultCode upload_entry(Entry& e, const RTAabb* nodes, uint64_t node_count, const uint32_t* idx, uint64_t prim_count,
                        cudaStream_t s) {
  uint32_t largest = 0;
  for (uint64_t i = 0; i < prim_count; ++i) largest = std::max(largest, idx[i]);
  e.vertex_count = largest + 1;
  e.vertex_lower_bound = true;
  cudaError_t err;
  if ((err = device_alloc(&e.d_status, 4, s)) || (err = cudaMemsetAsync(e.d_status, 0, 16, s)) ||
      (err = device_alloc(&e.d_nodes, node_count, s)) ||
      (err = cudaMemcpyAsync(e.d_nodes, nodes, node_count * sizeof(DAabb), cudaMemcpyHostToDevice, s)) ||
      (err = device_alloc(&e.d_indices, prim_count, s)) ||
      (err = cudaMemcpyAsync(e.d_indices, idx, prim_count * 4, cudaMemcpyHostToDevice, s)) ||
      (err = cudaStreamSynchronize(s)))
    return cuda_rc(err);
  return Ok;
}

}  // namespace

ResultCode rtbvh_serialize_bvh(RTBvh bvh, uint8_t* buffer, uintptr_t capacity, uintptr_t* size) {
  if (size == nullptr) return Error;
  std::vector<DAabb> nodes;
  std::vector<uint32_t> idx;
  uint32_t build_type;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(bvh.id, false);
    if (!e) return Error;
    build_type = e->build_type;
    ResultCode rc;
    if ((rc = fetch_device(nodes, e->d_nodes, e->node_count)) != Ok ||
        (rc = fetch_device(idx, e->d_indices, e->prim_count)) != Ok)
      return rc;
  }
  ByteWriter w{buffer, buffer ? (size_t)capacity : 0};
  w.u64(nodes.size());
  w.put(nodes.data(), nodes.size() * sizeof(DAabb));
  w.u64(idx.size());
  w.put(idx.data(), idx.size() * 4);
  w.u32(build_type);
  *size = w.n;
  if (buffer && w.n > capacity) return InvalidArgument;
  return Ok;
}

ResultCode rtbvh_deserialize_bvh(const uint8_t* buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                 RTBvh* result) {
  if (buffer == nullptr || result == nullptr) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ByteReader r{buffer, (size_t)size};
  const uint64_t nn = r.u64();
  const RTAabb* nodes = nn <= (size - r.n) / 32 ? reinterpret_cast<const RTAabb*>(r.take(nn * 32)) : nullptr;
  const uint64_t ni = r.ok ? r.u64() : 0;
  const uint8_t* ip = ni <= (size - r.n) / 4 ? r.take(ni * 4) : nullptr;
  const uint32_t bt = r.u32();
  if (!r.ok || !nodes || !ip || r.n != size || bt > 3) return InvalidArgument;
  if (nn == 0 || ni == 0) return NoPrimitives;
  if (nn > 0xffffffffull || ni > 0xffffffffull) return InvalidArgument;
  // the buffer may be unaligned: copy into aligned host arrays
  std::vector<RTAabb> hn(nn);
  std::vector<uint32_t> hi(ni);
  std::memcpy(hn.data(), nodes, nn * 32);
  std::memcpy(hi.data(), ip, ni * 4);
  if (!nodes_valid(hn.data(), nn, ni) || !indices_valid(hi.data(), ni)) return InvalidArgument;
  auto e = std::make_unique<Entry>();
  e->alive = true;
  e->node_count = (uint32_t)nn;
  e->prim_count = (uint32_t)ni;
  e->build_type = bt;
  e->boxes_cover = false;  // triangles come later (rtbvh_gpu_set_triangles)
  ResultCode rc = upload_entry(*e, hn.data(), nn, hi.data(), ni, s);
  if (rc == Ok && !(flags & RTBVH_FLAG_NO_HOST_MIRROR)) rc = mirror_bvh(*e, s);
  if (rc != Ok) {
    e->release();
    return rc;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* raw = e.get();
  uint32_t id = store(std::move(e), false);
  *result = bvh_handle(id, *raw);
  return Ok;
}

ResultCode rtbvh_serialize_mbvh(RTMbvh mbvh, uint8_t* buffer, uintptr_t capacity, uintptr_t* size) {
  if (size == nullptr) return Error;
  std::vector<DAabb> nodes;
  std::vector<DMNode> mnodes;
  std::vector<uint32_t> idx;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    Entry* e = lookup(mbvh.id, true);
    if (!e || !e->d_nodes) return Error;
    ResultCode rc;
    if ((rc = fetch_device(nodes, e->d_nodes, e->bvh_node_count)) != Ok ||
        (rc = fetch_device(mnodes, e->d_mnodes, e->node_count)) != Ok ||
        (rc = fetch_device(idx, e->d_indices, e->prim_count)) != Ok)
      return rc;
  }
  ByteWriter w{buffer, buffer ? (size_t)capacity : 0};
  w.u64(nodes.size());
  w.put(nodes.data(), nodes.size() * sizeof(DAabb));
  w.u64(mnodes.size());
  w.put(mnodes.data(), mnodes.size() * sizeof(DMNode));
  w.u64(idx.size());
  w.put(idx.data(), idx.size() * 4);
  *size = w.n;
  if (buffer && w.n > capacity) return InvalidArgument;
  return Ok;
}

ResultCode rtbvh_deserialize_mbvh(const uint8_t* buffer, uintptr_t size, uint32_t flags, rtbvh_stream_t stream,
                                  RTMbvh* result) {
  if (buffer == nullptr || result == nullptr) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ByteReader r{buffer, (size_t)size};
  const uint64_t nn = r.u64();
  const uint8_t* np = nn <= (size - r.n) / 32 ? r.take(nn * 32) : nullptr;
  const uint64_t nq = r.ok ? r.u64() : 0;
  const uint8_t* qp = nq <= (size - r.n) / 128 ? r.take(nq * 128) : nullptr;
  const uint64_t ni = r.ok ? r.u64() : 0;
  const uint8_t* ip = ni <= (size - r.n) / 4 ? r.take(ni * 4) : nullptr;
  if (!r.ok || !np || !qp || !ip || r.n != size) return InvalidArgument;
  if (nn == 0 || ni == 0) return NoPrimitives;
  if (nn > 0xffffffffull || nq > 0xffffffffull || ni > 0xffffffffull) return InvalidArgument;
  std::vector<RTAabb> hn(nn);
  std::vector<RTMbvhNode> hq(nq);
  std::vector<uint32_t> hi(ni);
  std::memcpy(hn.data(), np, nn * 32);
  std::memcpy(hq.data(), qp, nq * 128);
  std::memcpy(hi.data(), ip, ni * 4);
  if (!nodes_valid(hn.data(), nn, ni) || !indices_valid(hi.data(), ni)) return InvalidArgument;
  auto e = std::make_unique<Entry>();
  e->alive = true;
  e->prim_count = (uint32_t)ni;
  e->bvh_node_count = (uint32_t)nn;
  ResultCode rc = upload_entry(*e, hn.data(), nn, hi.data(), ni, s);
  // the quad nodes must be the collapse of the BVH2 nodes (Mbvh::construct):
  // collapse again on the device and compare bit for bit
  if (rc == Ok) rc = build_mbvh(e->d_nodes, e->bvh_node_count, s, &e->d_mnodes, &e->node_count);
  if (rc == Ok) {
    std::vector<DMNode> check;
    if ((rc = fetch_device(check, e->d_mnodes, e->node_count)) == Ok &&
        (check.size() != nq || std::memcmp(check.data(), hq.data(), nq * 128) != 0))
      rc = InvalidArgument;
  }
  // no triangles yet: the traversal tree is built when they are attached
  if (rc == Ok && !(flags & RTBVH_FLAG_NO_HOST_MIRROR)) rc = mirror_mbvh(*e, s);
  if (rc != Ok) {
    e->release();
    return rc;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  Entry* raw = e.get();
  uint32_t id = store(std::move(e), true);
  *result = mbvh_handle(id, *raw);
  return Ok;
}
