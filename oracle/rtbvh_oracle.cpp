// rtbvh oracle -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the CPU algorithms of meirbon/rtbvh (Rust crate
// `rtbvh` 0.6.2 plus its `rtbvh_ffi` wrapper) for the BVH construction and
// single-ray traversal path. It exists to check the CUDA implementation in
// `rtbvh_gb300/` and to serve as the timed CPU baseline. Only `tests/`,
// `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` may load it;
// the product library never links or calls it.
//
// Each function names the reference file:line it follows (paths relative to
// the reference project root).
//
// Parity status of this restatement:
//  * pinned by the reference's own known-answer tests: morton_split
//    (src/morton.rs:109-115), prefix_sum (src/utils.rs:295-345), build input
//    errors (src/lib.rs:28-64), builder structural checks on the teapot
//    (src/builders/binned_sah.rs:407-458, src/builders/locb.rs:336-388), the
//    five-triangle case (src/lib.rs:246-311) and the FFI quad hit at t == 1
//    (rtbvh_ffi/src/lib.rs:945-1060);
//  * unpinned: exact node layouts, split choices, hit ids and t values on real
//    scenes. No reference test pins them and the Rust crate cannot be compiled
//    here (no cargo/rustc), so they follow the reference source line by line.
//
// Floating-point conventions (the reference leans on `glam`, whose version is
// not pinned by the reference):
//  * Vec3 is scalar: dot is ((x*x') + (y*y')) + (z*z'), cross is the standard
//    component formula, no FMA contraction (this file must be compiled with
//    -ffp-contract=off).
//  * Vec3::min/max follow Rust f32::min/max: a NaN operand is ignored. For the
//    unspecified -0.0/+0.0 tie this restatement returns -0.0 for min and +0.0
//    for max, which keeps unions order-independent.
//  * Vec4 (SSE) min/max follow _mm_min_ps/_mm_max_ps: min(a,b) = a<b ? a : b,
//    max(a,b) = a>b ? a : b (NaN selects the second operand).
//  * `f32 as i32` / `as usize` saturate and map NaN to 0 (Rust semantics).

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- scalars
inline float rs_min(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
inline float rs_max(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}
inline float sse_min(float a, float b) { return a < b ? a : b; }
inline float sse_max(float a, float b) { return a > b ? a : b; }

// Rust `f32 as i32`.
inline int32_t rs_f32_to_i32(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}
// Rust `f32 as usize` (64-bit).
inline uint64_t rs_f32_to_usize(float f) {
  if (f != f) return 0;
  if (f <= 0.0f) return 0;
  if (f >= 18446744073709551616.0f) return UINT64_MAX;
  return (uint64_t)f;
}

struct V3 {
  float x, y, z;
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float dot(V3 a, V3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

// ---------------------------------------------------------------- Aabb
// src/aabb.rs:13-20 -- {min, extra1, max, extra2}, 32 bytes.
struct Aabb {
  float min[3];
  int32_t extra1;
  float max[3];
  int32_t extra2;
};
static_assert(sizeof(Aabb) == 32, "Aabb must be 32 bytes");

// src/aabb.rs:49-57
inline Aabb aabb_new() {
  Aabb a;
  for (int i = 0; i < 3; ++i) { a.min[i] = 1e34f; a.max[i] = -1e34f; }
  a.extra1 = 0;
  a.extra2 = 0;
  return a;
}
// src/aabb.rs:251-261
inline void aabb_grow(Aabb& a, V3 p) {
  for (int i = 0; i < 3; ++i) { a.min[i] = rs_min(a.min[i], p[i]); a.max[i] = rs_max(a.max[i], p[i]); }
}
// src/aabb.rs:263-273
inline void aabb_grow_bb(Aabb& a, const Aabb& b) {
  for (int i = 0; i < 3; ++i) { a.min[i] = rs_min(a.min[i], b.min[i]); a.max[i] = rs_max(a.max[i], b.max[i]); }
}
// src/aabb.rs:73-86 (extras take Default, i.e. 0)
inline Aabb aabb_union_of(const Aabb& a, const Aabb& b) {
  Aabb r;
  for (int i = 0; i < 3; ++i) { r.min[i] = rs_min(a.min[i], b.min[i]); r.max[i] = rs_max(a.max[i], b.max[i]); }
  r.extra1 = 0;
  r.extra2 = 0;
  return r;
}
// src/aabb.rs:312-321 (with_offset at :300-310 is the same arithmetic)
inline void aabb_offset_by(Aabb& a, float d) {
  for (int i = 0; i < 3; ++i) { a.min[i] = a.min[i] - d; a.max[i] = a.max[i] + d; }
}
// src/aabb.rs:342-346
inline float aabb_half_area(const Aabb& a) {
  float d0 = a.max[0] - a.min[0], d1 = a.max[1] - a.min[1], d2 = a.max[2] - a.min[2];
  float t = (d0 + d1) * d2;
  float u = d0 * d1;
  return t + u;
}
// src/aabb.rs:353-363, extend at :387-390
inline int aabb_longest_axis(const Aabb& a) {
  int ax = 0;
  if ((a.max[1] - a.min[1]) > (a.max[0] - a.min[0])) ax = 1;
  if ((a.max[2] - a.min[2]) > (a.max[ax] - a.min[ax])) ax = 2;
  return ax;
}
// src/aabb.rs:124-131
inline Aabb aabb_union_of_list(const Aabb* boxes, size_t n) {
  Aabb a = aabb_new();
  for (size_t i = 0; i < n; ++i) aabb_grow_bb(a, boxes[i]);
  aabb_offset_by(a, 0.0001f);
  return a;
}
// src/aabb.rs:141-143 (Vec3A cmple: NaN compares false)
inline bool aabb_is_valid(const Aabb& a) {
  return a.min[0] <= a.max[0] && a.min[1] <= a.max[1] && a.min[2] <= a.max[2];
}
// src/aabb.rs:246-249
inline bool aabb_contains(const Aabb& a, V3 p) {
  return p.x > a.min[0] && p.x < a.max[0] && p.y > a.min[1] && p.y < a.max[1] && p.z > a.min[2] &&
         p.z < a.max[2];
}

// ---------------------------------------------------------------- BvhNode
// src/bvh_node.rs:12-14 -- a node is an Aabb: extra1 = count (-1: interior),
// extra2 = left_first (-1: invalid). Accessors at src/bvh_node.rs:79-147.
typedef Aabb BvhNode;
inline bool node_is_leaf(const BvhNode& n) { return n.extra1 >= 0; }
inline BvhNode node_new() { return aabb_new(); }  // src/bvh_node.rs:62-66

// ---------------------------------------------------------------- Ray
// src/ray.rs:9-16, Ray::new at src/ray.rs:166-182.
struct Ray {
  V3 origin;
  float t_min;
  V3 direction;
  float t;
  V3 inv_direction;
  uint8_t signs[4];
};
inline Ray ray_new(V3 o, V3 d) {
  Ray r;
  r.origin = o;
  r.direction = d;
  r.t_min = 1e-4f;
  r.t = 1e34f;
  r.inv_direction = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  r.signs[0] = d.x < 0.0f;
  r.signs[1] = d.y < 0.0f;
  r.signs[2] = d.z < 0.0f;
  r.signs[3] = 0;
  return r;
}
inline bool v3_is_nan(V3 v) { return v.x != v.x || v.y != v.y || v.z != v.z; }

// src/aabb.rs:145-181 -- sign-indexed slab test; returns the FAR t.
inline bool aabb_intersect(const Aabb& a, const Ray& r, float* out) {
  auto sel = [&](int s, int axis) { return s == 0 ? a.min[axis] : a.max[axis]; };
  float ray_min = (sel(r.signs[0], 0) - r.origin.x) * r.inv_direction.x;
  float ray_max = (sel(1 - r.signs[0], 0) - r.origin.x) * r.inv_direction.x;
  float y_min = (sel(r.signs[1], 1) - r.origin.y) * r.inv_direction.y;
  float y_max = (sel(1 - r.signs[1], 1) - r.origin.y) * r.inv_direction.y;
  if ((ray_min > y_max) || (y_min > ray_max)) return false;
  if (y_min > ray_min) ray_min = y_min;
  if (y_max < ray_max) ray_max = y_max;
  float z_min = (sel(r.signs[2], 2) - r.origin.z) * r.inv_direction.z;
  float z_max = (sel(1 - r.signs[2], 2) - r.origin.z) * r.inv_direction.z;
  if ((ray_min > z_max) || (z_min > ray_max)) return false;
  if (z_max < ray_max) ray_max = z_max;
  if (ray_max > r.t_min) { *out = ray_max; return true; }
  return false;
}

// ---------------------------------------------------------------- MbvhNode
// src/mbvh_node.rs:29-38, 128 bytes.
struct MbvhNode {
  float min_x[4], max_x[4], min_y[4], max_y[4], min_z[4], max_z[4];
  int32_t children[4];
  int32_t counts[4];
};
static_assert(sizeof(MbvhNode) == 128, "MbvhNode must be 128 bytes");

// src/mbvh_node.rs:56-78
inline MbvhNode mnode_new() {
  MbvhNode m;
  for (int i = 0; i < 4; ++i) {
    m.min_x[i] = m.min_y[i] = m.min_z[i] = 1e34f;
    m.max_x[i] = m.max_y[i] = m.max_z[i] = -1e34f;
    m.children[i] = -1;
    m.counts[i] = -1;
  }
  return m;
}
// src/mbvh_node.rs:40-53 (Default, used by the final resize)
inline MbvhNode mnode_default() {
  MbvhNode m;
  std::memset(&m, 0, sizeof(m));
  for (int i = 0; i < 4; ++i) { m.children[i] = -1; m.counts[i] = -1; }
  return m;
}
// src/mbvh_node.rs:161-174
inline void mnode_set_bounds_bb(MbvhNode& m, int i, const Aabb& b) {
  m.min_x[i] = b.min[0]; m.min_y[i] = b.min[1]; m.min_z[i] = b.min[2];
  m.max_x[i] = b.max[0]; m.max_y[i] = b.max[1]; m.max_z[i] = b.max[2];
}

struct MbvhHit {
  uint8_t ids[4];
  bool result[4];
};

// src/mbvh_node.rs:176-240 -- 4-wide slab test with SSE min/max, then a
// 5-compare sorting network on t_min (the last compare swaps ids only).
inline MbvhHit mnode_intersect(const MbvhNode& m, const Ray& r) {
  float t_min[4];
  MbvhHit h;
  for (int i = 0; i < 4; ++i) {
    float tx0 = (m.min_x[i] - r.origin.x) * r.inv_direction.x;
    float tx1 = (m.max_x[i] - r.origin.x) * r.inv_direction.x;
    float ty0 = (m.min_y[i] - r.origin.y) * r.inv_direction.y;
    float ty1 = (m.max_y[i] - r.origin.y) * r.inv_direction.y;
    float tz0 = (m.min_z[i] - r.origin.z) * r.inv_direction.z;
    float tz1 = (m.max_z[i] - r.origin.z) * r.inv_direction.z;
    float tx_min = sse_min(tx0, tx1), tx_max = sse_max(tx0, tx1);
    float ty_min = sse_min(ty0, ty1), ty_max = sse_max(ty0, ty1);
    float tz_min = sse_min(tz0, tz1), tz_max = sse_max(tz0, tz1);
    float tmin = sse_max(tx_min, sse_max(ty_min, tz_min));
    float tmax = sse_min(tx_max, sse_min(ty_max, tz_max));
    t_min[i] = tmin;
    h.result[i] = (tmax >= tmin) && (tmin < r.t);
  }
  uint8_t ids[4] = {0, 1, 2, 3};
  if (t_min[0] > t_min[1]) { std::swap(t_min[0], t_min[1]); std::swap(ids[0], ids[1]); }
  if (t_min[2] > t_min[3]) { std::swap(t_min[2], t_min[3]); std::swap(ids[2], ids[3]); }
  if (t_min[0] > t_min[2]) { std::swap(t_min[0], t_min[2]); std::swap(ids[0], ids[2]); }
  if (t_min[1] > t_min[3]) { std::swap(t_min[1], t_min[3]); std::swap(ids[1], ids[3]); }
  if (t_min[2] > t_min[3]) { std::swap(ids[2], ids[3]); }
  for (int i = 0; i < 4; ++i) h.ids[i] = ids[i];
  return h;
}

// src/mbvh_node.rs:297-411
void merge_nodes(size_t m_index, size_t cur_node, const BvhNode* pool, size_t pool_len,
                 std::vector<MbvhNode>& mpool, size_t& pool_ptr) {
  for (int i = 0; i < 4; ++i) mnode_set_bounds_bb(mpool[m_index], i, pool[cur_node]);
  int32_t nodes[4] = {-1, -1, -1, -1};
  int32_t leafs[4] = {-1, -1, -1, -1};
  if (pool[cur_node].extra2 >= 0) {
    uint32_t left_first = (uint32_t)pool[cur_node].extra2;
    size_t child[2] = {left_first, (size_t)left_first + 1};
    for (int side = 0; side < 2; ++side) {
      const int s0 = side * 2;
      if (child[side] < pool_len) {
        const BvhNode& cn = pool[child[side]];
        if (cn.extra2 >= 0) {
          uint32_t lf = (uint32_t)cn.extra2;
          if (node_is_leaf(cn)) {
            nodes[s0] = (int32_t)lf;
            leafs[s0] = cn.extra1;
          } else {
            for (int k = 0; k < 2; ++k) {
              const BvhNode& g = pool[lf + k];
              if (node_is_leaf(g)) {
                nodes[s0 + k] = g.extra2;
                leafs[s0 + k] = g.extra1;
              } else {
                nodes[s0 + k] = (int32_t)(lf + k);
              }
              mnode_set_bounds_bb(mpool[m_index], s0 + k, g);
            }
          }
        }
      }
    }
  }
  for (int i = 0; i < 4; ++i) {
    int32_t node = nodes[i];
    int32_t count = leafs[i];
    if (node >= 0 && count >= 0) {
      mpool[m_index].children[i] = node;
      mpool[m_index].counts[i] = count;
      continue;
    } else if (node == -1) {
      continue;
    }
    const BvhNode& bn = pool[(size_t)node];
    if (node_is_leaf(bn)) {
      mpool[m_index].children[i] = bn.extra2;
      mpool[m_index].counts[i] = bn.extra1;
      mnode_set_bounds_bb(mpool[m_index], i, bn);
    } else {
      size_t new_m = pool_ptr++;
      mpool[m_index].children[i] = (int32_t)new_m;
      mnode_set_bounds_bb(mpool[m_index], i, bn);
      merge_nodes(new_m, (size_t)node, pool, pool_len, mpool, pool_ptr);
    }
  }
}

// ---------------------------------------------------------------- Morton
// src/utils.rs:12-22
uint32_t round_up_log2(uint32_t bits, uint32_t offset) {
  if (bits == 0) return offset;
  while ((1u << offset) < bits) offset += 1;
  return offset;
}
// src/morton.rs:10-25 (usize is 64 bits)
uint32_t morton_split(uint32_t v) {
  uint32_t log_bits = round_up_log2(32, 0);
  uint64_t x = v;
  uint64_t mask = ~(uint64_t)0;
  uint64_t i = log_bits;
  uint64_t n = (uint64_t)1 << log_bits;
  while (i > 0) {
    mask = (mask | (mask << n)) & ~(mask << (n / 2));
    x = (x | (x << n)) & mask;
    n >>= 1;
    i -= 1;
  }
  return (uint32_t)x;
}

struct MortonEncoder {
  V3 world_to_grid, grid_offset;
  uint32_t grid_dim;
};
// src/morton.rs:36-46
MortonEncoder morton_encoder_new(const Aabb& a, uint32_t grid_dim) {
  MortonEncoder e;
  float g = (float)grid_dim;
  V3 inv = v3(1.0f / (a.max[0] - a.min[0]), 1.0f / (a.max[1] - a.min[1]), 1.0f / (a.max[2] - a.min[2]));
  e.world_to_grid = v3(g * inv.x, g * inv.y, g * inv.z);
  e.grid_offset = v3(-a.min[0] * e.world_to_grid.x, -a.min[1] * e.world_to_grid.y, -a.min[2] * e.world_to_grid.z);
  e.grid_dim = grid_dim;
  return e;
}
// src/morton.rs:48-61
uint32_t morton_encode_point(const MortonEncoder& e, V3 p) {
  float gp[3] = {p.x * e.world_to_grid.x + e.grid_offset.x, p.y * e.world_to_grid.y + e.grid_offset.y,
                 p.z * e.world_to_grid.z + e.grid_offset.z};
  int32_t lim = (int32_t)(e.grid_dim - 1);
  uint32_t c[3];
  for (int i = 0; i < 3; ++i) c[i] = (uint32_t)std::min(lim, std::max(rs_f32_to_i32(gp[i]), 0));
  return morton_split(c[0]) | (morton_split(c[1]) << 1) | (morton_split(c[2]) << 2);
}

// ---------------------------------------------------------------- Bvh
struct Bvh {
  std::vector<BvhNode> nodes;
  std::vector<uint32_t> prim_indices;
};

// src/utils.rs:74-96 (Lomuto partition over a sub-slice)
template <class F>
size_t partition(uint32_t* slice, size_t len, F check) {
  size_t count = 0;
  for (size_t i = 0; i < len; ++i) {
    if (check(slice[i])) {
      std::swap(slice[i], slice[count]);
      count += 1;
    }
  }
  return count;
}

struct SahBin {
  Aabb aabb;
  uint64_t prim_count;
  float right_cost;
};
struct SahSplit {
  float cost;
  uint32_t count;
};

struct BinnedCfg {
  const Aabb* aabbs;
  const V3* centers;
  size_t max_depth, bin_count, max_leaf_size;
  float traversal_cost;
};

// src/builders/binned_sah.rs:119-128
inline size_t compute_bin_index(V3 center, size_t bin_count, V3 bin_offset, V3 center_to_bin, int axis) {
  float bin_index = center[axis] * center_to_bin[axis] + bin_offset[axis];
  uint64_t b = rs_f32_to_usize(rs_max(bin_index, 0.0f));
  return (size_t)std::min<uint64_t>((uint64_t)(bin_count - 1), b);
}

// src/builders/mod.rs:59-76 -- pair allocation; one shared counter.
struct NodeAlloc {
  std::atomic<size_t>* counter;
  size_t len;
};

struct SahTask {
  size_t node, begin, end, depth;
};


constexpr float F32_MAX = 3.40282347e+38f;  // f32::MAX

// src/builders/binned_sah.rs:80-114
SahSplit find_split(SahBin* bins, size_t bin_count) {
  Aabb cur = aabb_new();
  uint64_t cnt = 0;
  for (size_t i = bin_count - 1; i > 0; --i) {
    aabb_grow_bb(cur, bins[i].aabb);
    cnt += bins[i].prim_count;
    bins[i].right_cost = aabb_half_area(cur) * (float)cnt;
  }
  cur = aabb_new();
  cnt = 0;
  SahSplit best{F32_MAX, (uint32_t)bin_count};
  for (size_t i = 0; i + 1 < bin_count; ++i) {
    aabb_grow_bb(cur, bins[i].aabb);
    cnt += bins[i].prim_count;
    float cost = aabb_half_area(cur) * (float)cnt + bins[i + 1].right_cost;
    if (cost < best.cost) best = SahSplit{cost, (uint32_t)(i + 1)};
  }
  return best;
}

// src/builders/binned_sah.rs:132-282 -- one build task. Returns true and fills
// (ta, tb) when the node was split.
bool sah_task_run(const BinnedCfg& cfg, BvhNode* nodes, size_t nodes_len, uint32_t* prim_indices,
                  std::atomic<size_t>& counter, const SahTask& t, SahTask& ta, SahTask& tb,
                  std::vector<SahBin>& bin_store) {
  BvhNode& node = nodes[t.node];
  aabb_offset_by(node, 0.0001f);
  auto make_leaf = [&]() {
    aabb_offset_by(node, 0.0001f);
    node.extra2 = (int32_t)t.begin;
    node.extra1 = (int32_t)(t.end - t.begin);
  };
  const size_t ws = t.end - t.begin;
  if (ws <= 1 || t.depth >= cfg.max_depth) {
    make_leaf();
    return false;
  }
  const size_t bc = cfg.bin_count;
  V3 c2b, off;
  {
    float inv[3];
    for (int a = 0; a < 3; ++a) inv[a] = 1.0f / (node.max[a] - node.min[a]);
    c2b = v3(inv[0] * (float)bc, inv[1] * (float)bc, inv[2] * (float)bc);
    off = v3(-node.min[0] * c2b.x, -node.min[1] * c2b.y, -node.min[2] * c2b.z);
  }
  bin_store.resize(3 * bc);
  SahBin* bins[3] = {&bin_store[0], &bin_store[bc], &bin_store[2 * bc]};
  for (int a = 0; a < 3; ++a)
    for (size_t i = 0; i < bc; ++i) { bins[a][i].aabb = aabb_new(); bins[a][i].prim_count = 0; bins[a][i].right_cost = F32_MAX; }

  uint32_t* slice = prim_indices + t.begin;
  for (size_t i = 0; i < ws; ++i) {
    size_t p = slice[i];
    for (int a = 0; a < 3; ++a) {
      size_t bi = compute_bin_index(cfg.centers[p], bc, off, c2b, a);
      bins[a][bi].prim_count += 1;
      aabb_grow_bb(bins[a][bi].aabb, cfg.aabbs[p]);
    }
  }
  SahSplit best_splits[3];
  for (int a = 0; a < 3; ++a) best_splits[a] = find_split(bins[a], bc);
  int best_axis = 0;
  if (best_splits[0].cost > best_splits[1].cost) best_axis = 1;
  if (best_splits[best_axis].cost > best_splits[2].cost) best_axis = 2;

  size_t split_index = best_splits[best_axis].count;
  float max_split_cost = aabb_half_area(node) * ((float)ws - cfg.traversal_cost);
  if ((size_t)best_splits[best_axis].count == bc || best_splits[best_axis].cost >= max_split_cost) {
    if (ws > cfg.max_leaf_size) {
      best_axis = aabb_longest_axis(node);
      uint64_t count = 0;
      for (size_t i = 0; i + 1 < bc; ++i) {
        count += bins[best_axis][i].prim_count;
        if (count >= (uint64_t)(ws * 2 / 5 + 1)) {
          split_index = i + 1;
          break;
        }
      }
    } else {
      make_leaf();
      return false;
    }
  }
  const int ax = best_axis;
  size_t left_n = partition(slice, ws, [&](uint32_t id) {
    return compute_bin_index(cfg.centers[id], bc, off, c2b, ax) < split_index;
  });
  size_t begin_right = t.begin + left_n;
  if (begin_right > t.begin && begin_right < t.end) {
    size_t left = counter.fetch_add(2);
    if (left + 1 >= nodes_len + 1 || left >= nodes_len) return false;  // reference: unwrap() panics
    node.extra2 = (int32_t)left;
    node.extra1 = -1;
    Aabb left_box = aabb_new(), right_box = aabb_new();
    for (size_t i = 0; i < (size_t)best_splits[best_axis].count; ++i) aabb_grow_bb(left_box, bins[best_axis][i].aabb);
    for (size_t i = split_index; i < bc; ++i) aabb_grow_bb(right_box, bins[best_axis][i].aabb);
    nodes[left] = left_box;
    nodes[left + 1] = right_box;
    ta = SahTask{left, t.begin, begin_right, t.depth + 1};
    tb = SahTask{left + 1, begin_right, t.end, t.depth + 1};
    return true;
  }
  make_leaf();
  return false;
}

// src/utils.rs:243-288 -- TaskSpawner::run_task. With spawn_threshold = SIZE_MAX
// nothing is spawned and the visit order (hence node numbering) is the one a
// single worker produces.
void run_task(const BinnedCfg& cfg, BvhNode* nodes, size_t nodes_len, uint32_t* prim_indices,
              std::atomic<size_t>& counter, SahTask first, size_t spawn_threshold) {
  std::vector<std::thread> sub;
  std::vector<SahTask> stack{first};
  std::vector<SahBin> bins;
  while (!stack.empty()) {
    SahTask w = stack.back();
    stack.pop_back();
    SahTask a, b;
    if (sah_task_run(cfg, nodes, nodes_len, prim_indices, counter, w, a, b, bins)) {
      if ((a.end - a.begin) < (b.end - b.begin)) std::swap(a, b);
      stack.push_back(b);
      if ((a.end - a.begin) <= spawn_threshold) {
        stack.push_back(a);
        continue;
      }
      sub.emplace_back([&cfg, nodes, nodes_len, prim_indices, &counter, a, spawn_threshold]() {
        run_task(cfg, nodes, nodes_len, prim_indices, counter, a, spawn_threshold);
      });
    }
  }
  while (!sub.empty()) {
    sub.back().join();
    sub.pop_back();
  }
}

// src/builders/binned_sah.rs:305-318 (defaults) and :346-400 (build)
Bvh build_binned_sah(const Aabb* aabbs, const V3* centers, size_t n, size_t prims_per_leaf,
                     size_t spawn_threshold) {
  Bvh b;
  if (n == 0) return b;
  BinnedCfg cfg{aabbs, centers, 64, 16, prims_per_leaf == 0 ? 1 : prims_per_leaf, 1.0f};
  b.nodes.assign(2 * n - 1, node_new());
  b.prim_indices.resize(n);
  for (size_t i = 0; i < n; ++i) b.prim_indices[i] = (uint32_t)i;
  std::atomic<size_t> counter{1};
  b.nodes[0] = aabb_union_of_list(aabbs, n);
  run_task(cfg, b.nodes.data(), b.nodes.size(), b.prim_indices.data(), counter, SahTask{0, 0, n, 0},
           spawn_threshold);
  b.nodes.resize(counter.load());
  return b;
}

// ---------------------------------------------------------------- LOCB
// src/builders/locb.rs:36-45
inline void locb_search_range(size_t i, size_t begin, size_t end, size_t radius, size_t& sb, size_t& se) {
  sb = (i > begin + radius) ? i - radius : begin;
  se = std::min(i + radius + 1, end);
}

// src/builders/locb.rs:48-245. The reference caches the pair distances in a
// rolling matrix; every cached entry equals half_area(union(in[lo], in[hi]))
// for the pair, which is what is computed here directly. Returns false when
// a node has no neighbour (all distances NaN or >= f32::MAX).
bool locb_cluster(const BvhNode* in, BvhNode* out, uint32_t* nb, uint32_t* merged, size_t begin, size_t end,
                  size_t previous_end, size_t radius, size_t& next_begin, size_t& next_end) {
  for (size_t i = begin; i < end; ++i) {
    size_t sb, se;
    locb_search_range(i, begin, end, radius, sb, se);
    float best_d = F32_MAX;
    int64_t best_j = -1;
    for (size_t j = sb; j < i; ++j) {
      float d = aabb_half_area(aabb_union_of(in[j], in[i]));
      if (d < best_d) { best_d = d; best_j = (int64_t)j; }
    }
    for (size_t j = i + 1; j < se; ++j) {
      float d = aabb_half_area(aabb_union_of(in[i], in[j]));
      if (d < best_d) { best_d = d; best_j = (int64_t)j; }
    }
    if (best_j < 0) return false;
    nb[i] = (uint32_t)best_j;
  }
  for (size_t i = begin; i < end; ++i) {
    size_t j = nb[i];
    merged[i] = (i < j && (size_t)nb[j] == i) ? 1u : 0u;
  }
  // src/utils.rs:42-57 inclusive prefix sum
  uint32_t sum = 0;
  for (size_t i = begin; i < end; ++i) { sum += merged[i]; merged[i] = sum; }
  size_t merged_count = merged[end - 1];
  size_t unmerged_count = end - begin - merged_count;
  size_t children_count = merged_count * 2;
  size_t children_begin = end - children_count;
  size_t unmerged_begin = end - (children_count + unmerged_count);
  for (size_t i = begin; i < end; ++i) {
    size_t j = nb[i];
    if ((size_t)nb[j] == i) {
      if (i < j) {
        BvhNode& u = out[unmerged_begin + j - begin - merged[j]];
        size_t first_child = children_begin + ((size_t)merged[i] - 1) * 2;
        u = aabb_union_of(in[j], in[i]);
        u.extra1 = -1;
        u.extra2 = (int32_t)first_child;
        out[first_child] = in[i];
        out[first_child + 1] = in[j];
      }
    } else {
      out[unmerged_begin + i - begin - merged[i]] = in[i];
    }
  }
  for (size_t k = end; k < previous_end; ++k) out[k] = in[k];
  next_begin = unmerged_begin;
  next_end = children_begin;
  return merged_count > 0;
}

// src/morton.rs:63-102 -- codes, then a stable sort of the indices by code.
void morton_sorted(const MortonEncoder& enc, const V3* centers, size_t n, std::vector<uint32_t>& idx,
                   std::vector<uint32_t>& codes, unsigned threads) {
  codes.resize(n);
  idx.resize(n);
  if (threads <= 1 || n < 65536) {
    for (size_t i = 0; i < n; ++i) codes[i] = morton_encode_point(enc, centers[i]);
  } else {
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < threads; ++t)
      ts.emplace_back([&, t]() {
        for (size_t i = t; i < n; i += threads) codes[i] = morton_encode_point(enc, centers[i]);
      });
    for (auto& th : ts) th.join();
  }
  for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; });
}

// src/builders/locb.rs:18-29 (new) and :249-328 (build). Returns an empty
// Bvh and sets *err on a level without neighbours or merges.
Bvh build_locb(const Aabb* aabbs, const V3* centers, size_t n, int* err, unsigned threads) {
  Bvh b;
  *err = 0;
  if (n == 0) return b;
  Aabb world = aabb_union_of_list(aabbs, n);
  MortonEncoder enc = morton_encoder_new(world, 1u << 10);
  if (n <= 2) {
    BvhNode root = world;
    root.extra2 = 0;
    root.extra1 = (int32_t)n;
    b.nodes.push_back(root);
    for (size_t i = 0; i < n; ++i) b.prim_indices.push_back((uint32_t)i);
    return b;
  }
  std::vector<uint32_t> codes;
  morton_sorted(enc, centers, n, b.prim_indices, codes, threads);
  const size_t node_count = 2 * n - 1;
  BvhNode init;
  for (int i = 0; i < 3; ++i) { init.min[i] = 0.0f; init.max[i] = 0.0f; }
  init.extra1 = -1;
  init.extra2 = 0;
  std::vector<BvhNode> nodes(node_count, init), nodes_copy(node_count, init);
  std::vector<uint32_t> aux(node_count * 3, (uint32_t)node_count);
  uint32_t* nb = aux.data();
  uint32_t* merged = aux.data() + node_count;
  size_t begin = node_count - n, end = node_count, previous_end = end;
  for (size_t i = 0; i < n; ++i) {
    BvhNode& nd = nodes[begin + i];
    nd = aabbs[b.prim_indices[i]];
    aabb_offset_by(nd, 0.0001f);
    nd.extra1 = 1;
    nd.extra2 = (int32_t)i;
  }
  while (end - begin > 1) {
    size_t nbg, nen;
    if (!locb_cluster(nodes.data(), nodes_copy.data(), nb, merged, begin, end, previous_end, 14, nbg, nen)) {
      *err = 1;
      return Bvh();
    }
    std::swap(nodes, nodes_copy);
    previous_end = end;
    begin = nbg;
    end = nen;
  }
  b.nodes = std::move(nodes);
  return b;
}

// ---------------------------------------------------------------- Mbvh
// src/bvh.rs:381-404
std::vector<MbvhNode> mbvh_construct(const BvhNode* nodes, size_t node_count) {
  std::vector<MbvhNode> m;
  if (node_count == 0) return m;
  m.assign(node_count, mnode_new());
  size_t pool_ptr = 1;
  merge_nodes(0, 0, nodes, node_count, m, pool_ptr);
  m.resize(pool_ptr, mnode_default());
  return m;
}

// ---------------------------------------------------------------- refit / validate
// src/bvh.rs:176-205. Faithful: the fresh Aabb::new() carries extras of 0, so
// the reference overwrites every node's count/left_first with 0.
void refit(BvhNode* nodes, size_t node_count, const uint32_t* prim_indices, const Aabb* new_aabbs) {
  for (size_t ii = node_count; ii-- > 0;) {
    Aabb aabb = aabb_new();
    if (nodes[ii].extra2 >= 0) {
      uint32_t left_first = (uint32_t)nodes[ii].extra2;
      int32_t count = nodes[ii].extra1;
      if (node_is_leaf(nodes[ii])) {
        for (int32_t i = 0; i < count; ++i) aabb_grow_bb(aabb, new_aabbs[prim_indices[left_first + (uint32_t)i]]);
      } else {
        aabb_grow_bb(aabb, nodes[left_first]);
        aabb_grow_bb(aabb, nodes[left_first + 1]);
      }
      aabb_offset_by(aabb, 0.0001f);
    }
    nodes[ii] = aabb;
  }
}

// src/bvh.rs:207-244
void traverse_check(const BvhNode* nodes, const uint32_t* idx, const BvhNode& cur, uint8_t* checks, size_t n,
                    bool& ok) {
  if (cur.extra2 >= 0) {
    uint32_t lf = (uint32_t)cur.extra2;
    if (node_is_leaf(cur)) {
      for (int32_t i = 0; i < cur.extra1; ++i) {
        uint32_t p = idx[(int32_t)lf + i];
        if (p >= n) { ok = false; continue; }
        checks[p] = 1;
      }
    } else {
      traverse_check(nodes, idx, nodes[lf], checks, n, ok);
      traverse_check(nodes, idx, nodes[lf + 1], checks, n, ok);
    }
  }
}

// ---------------------------------------------------------------- traversal
struct Hit {
  float t, u, v;
  int32_t prim;
};
struct Stats {
  uint64_t node_visits = 0, tri_tests = 0, deep_pushes = 0;
  uint32_t max_stack = 0;
};

// src/builders/spatial_sah.rs:132-163 (Moller-Trumbore, closest-hit update)
inline bool mt_intersect(const float* tri, Ray& ray, float t_min, float* pu, float* pv) {
  V3 v0 = v3(tri[0], tri[1], tri[2]), v1 = v3(tri[3], tri[4], tri[5]), v2 = v3(tri[6], tri[7], tri[8]);
  V3 edge1 = sub(v1, v0), edge2 = sub(v2, v0);
  V3 h = cross(ray.direction, edge2);
  float a = dot(edge1, h);
  if (a > -1e-5f && a < 1e-5f) return false;
  float f = 1.0f / a;
  V3 s = sub(ray.origin, v0);
  float u = f * dot(s, h);
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  V3 q = cross(s, edge1);
  float v = f * dot(ray.direction, q);
  if (v < 0.0f || (u + v) > 1.0f) return false;
  float t = f * dot(edge2, q);
  if (t > t_min && t < ray.t) {
    ray.t = t;
    *pu = u;
    *pv = v;
    return true;
  }
  return false;
}

constexpr int ORACLE_STACK = 4096;

// src/iter_indices.rs:212-313 (MbvhIndexIterator) driving the triangle test,
// as examples/benchmark.rs:15-41 and rtbvh_ffi/src/lib.rs:700-731 do.
void trace_mbvh_one(const MbvhNode* m, size_t mcount, const uint32_t* idx, const float* tris, Ray& ray,
                    float t_min_tri, bool any_hit, Hit& out, Stats& st) {
  out.t = ray.t; out.u = 0.0f; out.v = 0.0f; out.prim = -1;
  if (mcount == 0) return;
  int32_t stack[ORACLE_STACK];
  MbvhHit hit = mnode_intersect(m[0], ray);
  st.node_visits++;
  int32_t current = 0, i = 0, j = 0, sp = -1;
  for (;;) {
    const MbvhNode& node = m[current];
    if (i >= 4) {
      if (sp < 0) break;
      current = stack[sp--];
      hit = mnode_intersect(m[current], ray);
      st.node_visits++;
      i = 0;
    } else {
      int id = hit.ids[3 - i];
      if (hit.result[id]) {
        int32_t count = node.counts[id];
        int32_t lf = node.children[id];
        if (count > -1) {
          if (j < count) {
            uint32_t prim = idx[lf + j];
            j++;
            st.tri_tests++;
            float u, v;
            if (mt_intersect(tris + 9 * (size_t)prim, ray, t_min_tri, &u, &v)) {
              out.t = ray.t; out.u = u; out.v = v; out.prim = (int32_t)prim;
              if (any_hit) return;
            }
            continue;
          }
          j = 0;
        } else if (lf > -1) {
          if (sp + 1 >= ORACLE_STACK) { out.prim = -2; return; }
          stack[++sp] = lf;
          if ((uint32_t)(sp + 1) > st.max_stack) st.max_stack = (uint32_t)(sp + 1);
          if (sp >= 32) st.deep_pushes++;
        }
      }
      i++;
    }
  }
}

// src/bvh_node.rs:150-177
inline int32_t sort_nodes(bool lh, float lt, bool rh, float rt, int32_t* stack, int32_t sp, int32_t lf) {
  if (lh && rh) {
    sp += 1;
    if (lt < rt) { stack[sp] = lf; sp += 1; stack[sp] = lf + 1; }
    else { stack[sp] = lf + 1; sp += 1; stack[sp] = lf; }
  } else if (lh) {
    sp += 1; stack[sp] = lf;
  } else if (rh) {
    sp += 1; stack[sp] = lf + 1;
  }
  return sp;
}

// src/iter_indices.rs:18-107 (BvhIndexIterator) driving the triangle test.
void trace_bvh_one(const BvhNode* nodes, size_t ncount, const uint32_t* idx, const float* tris, Ray& ray,
                   float t_min_tri, bool any_hit, Hit& out, Stats& st) {
  out.t = ray.t; out.u = 0.0f; out.v = 0.0f; out.prim = -1;
  if (ncount == 0 || v3_is_nan(ray.origin) || v3_is_nan(ray.direction)) return;
  int32_t stack[ORACLE_STACK];
  stack[0] = 0;
  int32_t sp = 0, i = 0;
  for (;;) {
    if (sp < 0) break;
    const BvhNode& node = nodes[stack[sp]];
    sp -= 1;
    int32_t count = node.extra1, lf = node.extra2;
    if (count > -1) {
      if (i < count) {
        uint32_t prim = idx[lf + i];
        i += 1;
        sp += 1;
        st.tri_tests++;
        float u, v;
        if (mt_intersect(tris + 9 * (size_t)prim, ray, t_min_tri, &u, &v)) {
          out.t = ray.t; out.u = u; out.v = v; out.prim = (int32_t)prim;
          if (any_hit) return;
        }
        continue;
      }
      i = 0;
    } else if (lf > -1) {
      st.node_visits++;
      float lt = 0.0f, rt = 0.0f;
      bool lh = aabb_intersect(nodes[lf], ray, &lt);
      bool rh = aabb_intersect(nodes[lf + 1], ray, &rt);
      if (sp + 2 >= ORACLE_STACK) { out.prim = -2; return; }
      sp = sort_nodes(lh, lt, rh, rt, stack, sp, lf);
      if ((uint32_t)(sp + 1) > st.max_stack) st.max_stack = (uint32_t)(sp + 1);
    }
  }
}

// ---------------------------------------------------------------- packets
// src/ray.rs:44-61 -- RayPacket4: four rays in SoA form. The inverse
// directions are 1/d per lane (ray.rs:86-100; rtbvh_ffi/src/lib.rs:673-676).
struct Packet4 {
  float ox[4], oy[4], oz[4], dx[4], dy[4], dz[4], ix[4], iy[4], iz[4], t[4];
};

// src/aabb.rs:217-246 -- Aabb::intersect4: glam Vec4 min/max (SSE rules);
// Some(per-lane t_min) when any lane has t_max > 0, t_max > t_min and
// t_min < t.
inline bool aabb_intersect4(const Aabb& a, const Packet4& p, float tnear[4]) {
  bool any = false;
  for (int k = 0; k < 4; ++k) {
    float t1x = (a.min[0] - p.ox[k]) * p.ix[k], t1y = (a.min[1] - p.oy[k]) * p.iy[k];
    float t1z = (a.min[2] - p.oz[k]) * p.iz[k];
    float t2x = (a.max[0] - p.ox[k]) * p.ix[k], t2y = (a.max[1] - p.oy[k]) * p.iy[k];
    float t2z = (a.max[2] - p.oz[k]) * p.iz[k];
    float tmin = sse_max(sse_min(t1x, t2x), sse_max(sse_min(t1y, t2y), sse_min(t1z, t2z)));
    float tmax = sse_min(sse_max(t1x, t2x), sse_min(sse_max(t1y, t2y), sse_max(t1z, t2z)));
    tnear[k] = tmin;
    if (tmax > 0.0f && tmax > tmin && tmin < p.t[k]) any = true;
  }
  return any;
}

// src/mbvh_node.rs:242-295 -- MbvhNode::intersect4: slot i is hit when any
// lane has t_max > t_min and t_min < t. The axes are folded in x, y, z order
// (t_min = max(max(x, y), z)). ids stay [0, 1, 2, 3].
inline void mnode_intersect4(const MbvhNode& m, const Packet4& p, bool result[4]) {
  for (int i = 0; i < 4; ++i) result[i] = false;
  for (int k = 0; k < 4; ++k) {
    for (int i = 0; i < 4; ++i) {
      float x1 = (m.min_x[i] - p.ox[k]) * p.ix[k], x2 = (m.max_x[i] - p.ox[k]) * p.ix[k];
      float tmin = sse_min(x1, x2), tmax = sse_max(x1, x2);
      float y1 = (m.min_y[i] - p.oy[k]) * p.iy[k], y2 = (m.max_y[i] - p.oy[k]) * p.iy[k];
      tmin = sse_max(tmin, sse_min(y1, y2));
      tmax = sse_min(tmax, sse_max(y1, y2));
      float z1 = (m.min_z[i] - p.oz[k]) * p.iz[k], z2 = (m.max_z[i] - p.oz[k]) * p.iz[k];
      tmin = sse_max(tmin, sse_min(z1, z2));
      tmax = sse_min(tmax, sse_max(z1, z2));
      if (tmax > tmin && tmin < p.t[k]) result[i] = true;
    }
  }
}

// src/builders/spatial_sah.rs:165-244 -- SpatialTriangle::intersect4, the
// packet triangle test the reference's packet benchmark calls
// (examples/benchmark.rs:43-68): |det| >= 1e-6, u and v in [0, 1] with
// u + v <= 1, t_min <= t < packet t; accepted lanes take the new t.
inline uint32_t tri_intersect4(const float* tri, Packet4& p, float t_min, float pu[4], float pv[4]) {
  const float e1x = tri[3] - tri[0], e1y = tri[4] - tri[1], e1z = tri[5] - tri[2];
  const float e2x = tri[6] - tri[0], e2y = tri[7] - tri[1], e2z = tri[8] - tri[2];
  uint32_t mask = 0;
  for (int k = 0; k < 4; ++k) {
    const float hx = (p.dy[k] * e2z) - (p.dz[k] * e2y);
    const float hy = (p.dz[k] * e2x) - (p.dx[k] * e2z);
    const float hz = (p.dx[k] * e2y) - (p.dy[k] * e2x);
    const float a = ((e1x * hx) + (e1y * hy)) + (e1z * hz);
    if (!(a <= -1e-6f || a >= 1e-6f)) continue;
    const float f = 1.0f / a;
    const float sx = p.ox[k] - tri[0], sy = p.oy[k] - tri[1], sz = p.oz[k] - tri[2];
    const float u = f * (((sx * hx) + (sy * hy)) + (sz * hz));
    if (!(u >= 0.0f && u <= 1.0f)) continue;
    const float qx = sy * e1z - sz * e1y, qy = sz * e1x - sx * e1z, qz = sx * e1y - sy * e1x;
    const float v = f * (((p.dx[k] * qx) + (p.dy[k] * qy)) + (p.dz[k] * qz));
    if (!(v >= 0.0f && (u + v) <= 1.0f)) continue;
    const float t = f * (((e2x * qx) + (e2y * qy)) + (e2z * qz));
    if (!(t >= t_min && t < p.t[k])) continue;
    p.t[k] = t;
    pu[k] = u;
    pv[k] = v;
    mask |= 1u << k;
  }
  return mask;
}

struct PacketOut {
  float u[4], v[4];
  int32_t prim[4];
};

inline void packet_test(const float* tris, uint32_t prim, Packet4& p, float t_min, PacketOut& out, Stats& st) {
  st.tri_tests++;
  float u[4], v[4];
  const uint32_t m = tri_intersect4(tris + 9 * (size_t)prim, p, t_min, u, v);
  for (int k = 0; k < 4; ++k)
    if ((m >> k) & 1u) { out.u[k] = u[k]; out.v[k] = v[k]; out.prim[k] = (int32_t)prim; }
}

// src/iter_indices.rs:316-414 (MbvhPacketIndexIterator): slots visited 3..0,
// a hit leaf's primitives yielded at once, hit interior slots pushed; a popped
// node's mask is computed with the packet's t at that moment.
bool trace_mbvh_packet(const MbvhNode* m, size_t mcount, const uint32_t* idx, const float* tris, Packet4& p,
                       float t_min, PacketOut& out, Stats& st) {
  if (mcount == 0) return true;
  int32_t stack[ORACLE_STACK];
  bool res[4];
  mnode_intersect4(m[0], p, res);
  st.node_visits++;
  int32_t current = 0, sp = -1;
  for (;;) {
    const MbvhNode& node = m[current];
    for (int i = 0; i < 4; ++i) {
      const int id = 3 - i;
      if (!res[id]) continue;
      const int32_t count = node.counts[id], lf = node.children[id];
      if (count > -1) {
        for (int32_t j = 0; j < count; ++j) packet_test(tris, idx[lf + j], p, t_min, out, st);
      } else if (lf > -1) {
        if (sp + 1 >= ORACLE_STACK) return false;
        stack[++sp] = lf;
        if ((uint32_t)(sp + 1) > st.max_stack) st.max_stack = (uint32_t)(sp + 1);
      }
    }
    if (sp < 0) break;
    current = stack[sp--];
    mnode_intersect4(m[current], p, res);
    st.node_visits++;
  }
  return true;
}

// src/iter_indices.rs:110-200 (BvhPacketIndexIterator) with
// BvhNode::sort_nodes4 (src/bvh_node.rs:180-213): both children hit -> the
// left one is pushed first (the right one is visited first) when any lane's
// left t_min is below its right t_min, else the reverse. A packet with a NaN
// origin or direction component walks nothing.
bool trace_bvh_packet(const BvhNode* nodes, size_t ncount, const uint32_t* idx, const float* tris, Packet4& p,
                      float t_min, PacketOut& out, Stats& st) {
  bool nan = false;
  for (int k = 0; k < 4; ++k)
    nan = nan || p.ox[k] != p.ox[k] || p.oy[k] != p.oy[k] || p.oz[k] != p.oz[k] || p.dx[k] != p.dx[k] ||
          p.dy[k] != p.dy[k] || p.dz[k] != p.dz[k];
  if (ncount == 0 || nan) return true;
  int32_t stack[ORACLE_STACK];
  stack[0] = 0;
  int32_t sp = 0;
  while (sp >= 0) {
    const BvhNode& node = nodes[stack[sp--]];
    const int32_t count = node.extra1, lf = node.extra2;
    if (count > -1) {
      for (int32_t j = 0; j < count; ++j) packet_test(tris, idx[lf + j], p, t_min, out, st);
    } else if (lf > -1) {
      st.node_visits++;
      float lt[4], rt[4];
      const bool lh = aabb_intersect4(nodes[lf], p, lt), rh = aabb_intersect4(nodes[lf + 1], p, rt);
      if (sp + 2 >= ORACLE_STACK) return false;
      if (lh && rh) {
        bool any_less = false;
        for (int k = 0; k < 4; ++k) any_less = any_less || (lt[k] < rt[k]);
        if (any_less) { stack[++sp] = lf; stack[++sp] = lf + 1; }
        else { stack[++sp] = lf + 1; stack[++sp] = lf; }
      } else if (lh) {
        stack[++sp] = lf;
      } else if (rh) {
        stack[++sp] = lf + 1;
      }
      if ((uint32_t)(sp + 1) > st.max_stack) st.max_stack = (uint32_t)(sp + 1);
    }
  }
  return true;
}

// ---------------------------------------------------------------- spatial SAH
// src/builders/spatial_sah.rs, sequential. Tasks run depth first, the child
// with more references first (ties: the left one): the order of
// TaskSpawner::run_task (src/utils.rs:246-283) while no task is handed to
// another thread. The reference hands tasks of more than 1024 references to
// new threads, after which its node numbering and leaf placement depend on
// thread timing; this order is the schedule in which each spawned thread
// runs to completion first.
//
// `fixes` selects corrections of reference defects (0 = the reference as
// written): see SpatialFix.

// spatial_sah.rs:64-78
struct SRef {
  Aabb aabb;
  V3 center;
  uint32_t prim;
};

enum SpatialFix : uint32_t {
  kFixClip = 1,        // split_edge returns a + t*(b-a), not a*t*(b-a) (:90-93)
  kFixExitBin = 2,     // a reference leaves at its last bin, not its first (:545-546)
  kFixSweepBox = 4,    // the sweep's left box is the union of bins 0..i, not of their suffix unions (:549-570)
  kFixSplitSpace = 8,  // allocate_children hands the freed split space to the left child and keeps the right
                       // child on its moved references (:375-424)
  kFixFallback = 16,   // the equal-count fallback starts at the task's begin (:643-648)
};

// src/aabb.rs:288-298
inline void aabb_shrink(Aabb& a, const Aabb& b) {
  for (int i = 0; i < 3; ++i) { a.min[i] = rs_max(a.min[i], b.min[i]); a.max[i] = rs_min(a.max[i], b.max[i]); }
}
// src/aabb.rs:334-340
inline float aabb_area(const Aabb& a) {
  float ex = a.max[0] - a.min[0], ey = a.max[1] - a.min[1], ez = a.max[2] - a.min[2];
  float v = ((ex * ey) + (ex * ez)) + (ey * ez);
  return rs_max(0.0f, v);
}
// src/aabb.rs:329-332
inline V3 aabb_center(const Aabb& a) {
  return v3((a.min[0] + a.max[0]) * 0.5f, (a.min[1] + a.max[1]) * 0.5f, (a.min[2] + a.max[2]) * 0.5f);
}

// SpatialTriangle::split, spatial_sah.rs:85-129. tri = v0, v1, v2.
void tri_split(const float* tri, int axis, float position, bool fix_clip, Aabb& left, Aabb& right) {
  const V3 p[3] = {v3(tri[0], tri[1], tri[2]), v3(tri[3], tri[4], tri[5]), v3(tri[6], tri[7], tri[8])};
  left = aabb_new();
  right = aabb_new();
  auto split_edge = [&](V3 a, V3 b) -> V3 {
    float t = (position - a[axis]) / (b[axis] - a[axis]);
    V3 d = sub(b, a);
    if (fix_clip) return v3(a.x + t * d.x, a.y + t * d.y, a.z + t * d.z);
    return v3((a.x * t) * d.x, (a.y * t) * d.y, (a.z * t) * d.z);
  };
  const bool q0 = p[0][axis] <= position, q1 = p[1][axis] <= position, q2 = p[2][axis] <= position;
  aabb_grow(q0 ? left : right, p[0]);
  aabb_grow(q1 ? left : right, p[1]);
  aabb_grow(q2 ? left : right, p[2]);
  if (q0 != q1) { V3 m = split_edge(p[0], p[1]); aabb_grow(left, m); aabb_grow(right, m); }
  if (q1 != q2) { V3 m = split_edge(p[1], p[2]); aabb_grow(left, m); aabb_grow(right, m); }
  if (q2 != q0) { V3 m = split_edge(p[2], p[0]); aabb_grow(left, m); aabb_grow(right, m); }
}

struct SWork {  // WorkItem, spatial_sah.rs:247-277
  size_t node, begin, end, split_end, depth;
  bool sorted;
};
struct ObjSplit {  // spatial_sah.rs:25-44
  float cost;
  int64_t index;  // -1: None
  int axis;
  Aabb left, right;
};
struct SpSplit {  // spatial_sah.rs:46-61
  float cost, position;
  int axis;
};

// Builder defaults, spatial_sah.rs:865-881 (max_leaf_size from primitives_per_leaf).
constexpr int kSbBins = 16, kSbPasses = 2;
constexpr size_t kSbMaxDepth = 64;
constexpr float kSbTraversalCost = 1.0f, kSbAlpha = 1e-5f, kSbSplitFactor = 0.75f;

struct SpatialBuild {
  const float* tris = nullptr;  // n x 9
  size_t n = 0, max_ref = 0, max_leaf = 1;
  uint32_t fixes = 0;
  float threshold = 0.0f;
  std::vector<BvhNode> nodes;
  std::atomic<size_t> node_count{1};   // AtomicNodeStack's counter
  std::vector<uint32_t> prim_indices;
  std::atomic<size_t> ref_counter{0};  // make_leaf's reference_count
  std::vector<Aabb> acc;
  std::vector<SRef> refs[3];
  std::vector<size_t> work;  // work_size() of the WorkItem each node was created with
  std::atomic<int> err{0};   // 1: the reference panics or writes out of bounds here
  const float* tri(uint32_t p) const { return tris + 9 * (size_t)p; }
};

// reference_marks of apply_object_split, one array per thread (the
// reference allocates one per call; all entries are false between calls).
std::vector<uint8_t>& sb_marks(size_t size) {
  thread_local std::vector<uint8_t> marks;
  if (marks.size() < size) marks.assign(size, 0);
  return marks;
}

// spatial_sah.rs:314-368
ObjSplit sb_find_object_split(SpatialBuild& b, size_t begin, size_t end, bool sorted) {
  if (!sorted) {
    // sort_by with a comparator that answers Less exactly when a < b: the
    // standard library's stable sort only asks "is less", so this is a stable
    // sort on the centre coordinate.
    for (int axis = 0; axis < 3; ++axis)
      std::stable_sort(b.refs[axis].begin() + begin, b.refs[axis].begin() + end,
                       [axis](const SRef& x, const SRef& y) { return x.center[axis] < y.center[axis]; });
  }
  ObjSplit best{FLT_MAX, -1, 0, aabb_new(), aabb_new()};
  for (int axis = 0; axis < 3; ++axis) {
    const std::vector<SRef>& r = b.refs[axis];
    Aabb a = aabb_new();
    for (size_t i = end - 1; i > begin; --i) {
      aabb_grow_bb(a, r[i].aabb);
      b.acc[i] = a;
    }
    a = aabb_new();
    for (size_t i = begin; i + 1 < end; ++i) {
      aabb_grow_bb(a, r[i].aabb);
      float cost = aabb_half_area(a) * (float)(i + 1 - begin) + aabb_half_area(b.acc[i + 1]) * (float)(end - (i + 1));
      if (cost < best.cost) best = ObjSplit{cost, (int64_t)(i + 1), axis, a, b.acc[i + 1]};
    }
  }
  return best;
}

// spatial_sah.rs:491-583. Returns false for None; sets b.err where the
// reference would panic.
bool sb_binning_pass(SpatialBuild& b, SpSplit& split, int axis, size_t begin, size_t end, float mn, float mx,
                     float& next_lo, float& next_hi) {
  struct Bin {
    Aabb aabb;
    size_t entry, exit;
  } bins[kSbBins];
  for (auto& bin : bins) bin = Bin{aabb_new(), 0, 0};
  const float bin_size = (mx - mn) / (float)kSbBins;
  const float inv_size = 1.0f / bin_size;
  const bool fix_clip = b.fixes & kFixClip;
  for (size_t i = begin; i < end; ++i) {
    const SRef& ref = b.refs[0][i];
    size_t first = std::min((size_t)(kSbBins - 1), (size_t)rs_f32_to_usize(rs_max(inv_size * (ref.aabb.min[axis] - mn), 0.0f)));
    size_t last = std::min((size_t)(kSbBins - 1), (size_t)rs_f32_to_usize(rs_max(inv_size * (ref.aabb.max[axis] - mn), 0.0f)));
    if (!aabb_is_valid(ref.aabb)) break;
    if (first > last) { b.err = 1; return false; }  // bins[first..last] panics
    Aabb cur = ref.aabb;
    for (size_t j = 0; j < last - first; ++j) {
      Aabb lb, rb;
      tri_split(b.tri(ref.prim), axis, mn + (float)(j + first + 1) * bin_size, fix_clip, lb, rb);
      aabb_shrink(lb, cur);
      aabb_grow_bb(bins[first + j].aabb, lb);
      aabb_shrink(cur, rb);
    }
    aabb_grow_bb(bins[last].aabb, cur);
    bins[first].entry += 1;
    bins[(b.fixes & kFixExitBin) ? last : first].exit += 1;
  }
  Aabb suffix[kSbBins];
  Aabb cur = aabb_new();
  for (int i = kSbBins; i > 0; --i) {
    aabb_grow_bb(cur, bins[i - 1].aabb);
    suffix[i - 1] = cur;
  }
  size_t left_count = 0, right_count = end - begin;
  cur = aabb_new();
  bool found = false;
  for (int i = 0; i < kSbBins - 1; ++i) {
    left_count += bins[i].entry;
    right_count -= bins[i].exit;
    aabb_grow_bb(cur, (b.fixes & kFixSweepBox) ? bins[i].aabb : suffix[i]);
    float cost = (float)left_count * aabb_half_area(cur) + (float)right_count * aabb_half_area(suffix[i + 1]);
    if (cost < split.cost) {
      split.cost = cost;
      split.axis = axis;
      split.position = mn + (float)(i + 1) * bin_size;
      found = true;
    }
  }
  if (!found) return false;
  next_lo = split.position - bin_size;
  next_hi = split.position + bin_size;
  return true;
}

// spatial_sah.rs:585-603
SpSplit sb_find_spatial_split(SpatialBuild& b, const SWork& w) {
  const Aabb nb = b.nodes[w.node];
  SpSplit split{FLT_MAX, 0.0f, 0};
  for (int axis = 0; axis < 3 && !b.err; ++axis) {
    float mn = nb.min[axis], mx = nb.max[axis];
    for (int pass = 0; pass < kSbPasses; ++pass) {
      float lo, hi;
      if (!sb_binning_pass(b, split, axis, w.begin, w.end, mn, mx, lo, hi)) break;
      mn = lo;
      mx = hi;
    }
  }
  return split;
}

// spatial_sah.rs:370-438
bool sb_allocate_children(SpatialBuild& b, const SWork& w, size_t right_begin, size_t right_end, const Aabb& left_box,
                          const Aabb& right_box, bool sorted, SWork& lw, SWork& rw) {
  const size_t left = b.node_count.fetch_add(2);
  if (left + 1 >= b.nodes.size()) { b.err = 1; return false; }  // AtomicNodeStack::allocate -> None
  BvhNode& parent = b.nodes[w.node];
  parent.extra2 = (int32_t)left;
  parent.extra1 = -1;
  aabb_offset_by(parent, 0.0001f);
  b.nodes[left] = left_box;
  b.nodes[left + 1] = right_box;

  const size_t remaining = w.split_end - right_end;
  const float left_cost = aabb_half_area(left_box) * (float)(right_begin - w.begin);
  const float right_cost = aabb_half_area(right_box) * (float)(right_end - right_begin);
  const size_t lsc = remaining == 0 ? 0 : (size_t)rs_f32_to_usize((float)remaining * (left_cost / (left_cost + right_cost)));
  if (lsc > 0) {
    if (right_end + lsc > b.max_ref) { b.err = 1; return false; }
    for (int axis = 0; axis < 3; ++axis) {  // move_backward, src/utils.rs:59-72
      SRef* r = b.refs[axis].data();
      std::memmove(r + right_begin + lsc, r + right_begin, (right_end - right_begin) * sizeof(SRef));
    }
  }
  const bool fix = b.fixes & kFixSplitSpace;
  lw = SWork{left, w.begin, right_begin, fix ? right_begin + lsc : right_begin, w.depth + 1, sorted};
  rw = fix ? SWork{left + 1, right_begin + lsc, right_end + lsc, w.split_end, w.depth + 1, sorted}
           : SWork{left + 1, right_begin, right_end, w.split_end, w.depth + 1, sorted};
  b.work[left] = lw.end - lw.begin;
  b.work[left + 1] = rw.end - rw.begin;
  return true;
}

// spatial_sah.rs:440-489
bool sb_apply_object_split(SpatialBuild& b, const SWork& w, const ObjSplit& split, SWork& lw, SWork& rw) {
  const size_t s = (size_t)split.index;
  if (split.index < (int64_t)w.begin || s >= w.end) { b.err = 1; return false; }  // assert!
  std::vector<SRef>& r = b.refs[split.axis];
  std::vector<uint8_t>& marks = sb_marks(b.max_ref);
  for (size_t i = w.begin; i < s; ++i) marks[r[i].prim] = 1;
  for (size_t i = s; i < w.end; ++i) marks[r[i].prim] = 0;
  // sort_by with "Less exactly when a is marked and b is not": a stable
  // partition, marked references first.
  for (int o = 1; o <= 2; ++o) {
    std::vector<SRef>& q = b.refs[(split.axis + o) % 3];
    std::stable_partition(q.begin() + w.begin, q.begin() + w.end, [&marks](const SRef& x) { return marks[x.prim] != 0; });
  }
  for (int axis = 0; axis < 3; ++axis)  // the reference allocates fresh marks per call
    for (size_t i = w.begin; i < w.end; ++i) marks[b.refs[axis][i].prim] = 0;
  return sb_allocate_children(b, w, s, w.end, split.left, split.right, true, lw, rw);
}

// spatial_sah.rs:605-724
bool sb_apply_spatial_split(SpatialBuild& b, const SWork& w, const SpSplit& split, SWork& lw, SWork& rw) {
  const int ax = split.axis;
  const float pos = split.position;
  std::vector<SRef>& r = b.refs[ax];
  size_t left_end = w.begin, right_begin = w.end, right_end = w.end;
  Aabb left_box = aabb_new(), right_box = aabb_new();
  size_t i = w.begin;
  while (i < right_begin) {
    const Aabb a = r[i].aabb;
    if (a.max[ax] <= pos) {
      aabb_grow_bb(left_box, a);
      std::swap(r[i], r[left_end]);
      i += 1;
      left_end += 1;
    } else if (a.min[ax] >= pos) {
      aabb_grow_bb(right_box, a);
      right_begin -= 1;
      std::swap(r[i], r[right_begin]);
    } else {
      i += 1;
    }
  }
  size_t left_count = left_end - w.begin, right_count = right_end - right_begin;
  if ((left_count == 0 || right_count == 0) && left_end == right_begin) {
    if (left_count > 0) left_end = (b.fixes & kFixFallback) ? w.begin + left_count / 2 : left_count / 2;
    else left_end += right_count / 2;
    right_begin = left_end;
    if (left_end < w.begin || left_end > w.end) { b.err = 1; return false; }  // slice range panics
    left_box = aabb_new();
    right_box = aabb_new();
    for (size_t k = w.begin; k < left_end; ++k) aabb_grow_bb(left_box, r[k].aabb);
    for (size_t k = left_end; k < w.end; ++k) aabb_grow_bb(right_box, r[k].aabb);
  }
  const bool fix_clip = b.fixes & kFixClip;
  while (left_end < right_begin) {
    const SRef ref = r[left_end];
    Aabb lp, rp;
    tri_split(b.tri(ref.prim), ax, pos, fix_clip, lp, rp);
    aabb_shrink(lp, ref.aabb);
    aabb_shrink(rp, ref.aabb);
    if (w.split_end - right_end > 0) {
      aabb_grow_bb(left_box, lp);
      aabb_grow_bb(right_box, rp);
      r[right_end] = SRef{rp, aabb_center(rp), ref.prim};
      r[left_end] = SRef{lp, aabb_center(lp), ref.prim};
      right_end += 1;
      left_end += 1;
      left_count += 1;
      right_count += 1;
    } else if (left_count < right_count) {
      aabb_grow_bb(left_box, ref.aabb);
      left_end += 1;
      left_count += 1;
    } else {
      aabb_grow_bb(right_box, ref.aabb);
      right_begin -= 1;
      std::swap(r[right_begin], r[left_end]);
      right_count += 1;
    }
  }
  for (int o = 1; o <= 2; ++o)
    std::copy(r.begin() + w.begin, r.begin() + right_end, b.refs[(ax + o) % 3].begin() + w.begin);
  return sb_allocate_children(b, w, right_begin, right_end, left_box, right_box, false, lw, rw);
}

// make_leaf, spatial_sah.rs:733-744
void sb_make_leaf(SpatialBuild& b, const SWork& w) {
  const size_t count = w.end - w.begin;
  const size_t first = b.ref_counter.fetch_add(count);
  if (first + count > b.max_ref) { b.err = 1; return; }
  for (size_t i = 0; i < count; ++i) b.prim_indices[first + i] = b.refs[0][w.begin + i].prim;
  b.nodes[w.node].extra2 = (int32_t)first;
  b.nodes[w.node].extra1 = (int32_t)count;
}

// Task::run, spatial_sah.rs:726-838. Returns true with two child tasks.
bool sb_run(SpatialBuild& b, const SWork& w, SWork& lw, SWork& rw) {
  const size_t work = w.end - w.begin;
  if (work <= 1 || w.depth >= kSbMaxDepth) {
    sb_make_leaf(b, w);
    return false;
  }
  ObjSplit obj = sb_find_object_split(b, w.begin, w.end, w.sorted);
  SpSplit sp{FLT_MAX, 0.0f, 0};
  Aabb ov = obj.left;
  aabb_shrink(ov, obj.right);
  const float overlap = aabb_area(ov);
  if (overlap > b.threshold && (w.split_end - w.end) > 0) sp = sb_find_spatial_split(b, w);
  if (b.err) return false;
  const float best = rs_min(sp.cost, obj.cost);
  bool use_spatial = best < obj.cost;
  const Aabb nb = b.nodes[w.node];
  const float max_split_cost = aabb_half_area(nb) * ((float)work - kSbTraversalCost);
  if (best >= max_split_cost) {
    if (work > b.max_leaf) {
      use_spatial = false;
      obj.index = (int64_t)((w.begin + w.end) / 2);
      obj.axis = aabb_longest_axis(nb);
      obj.left = aabb_new();
      obj.right = aabb_new();
      for (size_t i = w.begin; i < (size_t)obj.index; ++i) aabb_grow_bb(obj.left, b.refs[obj.axis][i].aabb);
      for (size_t i = (size_t)obj.index; i < w.end; ++i) aabb_grow_bb(obj.right, b.refs[obj.axis][i].aabb);
    } else {
      sb_make_leaf(b, w);
      return false;
    }
  }
  if (use_spatial) return sb_apply_spatial_split(b, w, sp, lw, rw);
  if (obj.index >= 0) return sb_apply_object_split(b, w, obj, lw, rw);
  sb_make_leaf(b, w);
  return false;
}

// SpatialSahBuilder::build, spatial_sah.rs:926-1034. aabbs: n boxes (with
// their extras), centers: Primitive::center of each triangle.
void build_spatial(SpatialBuild& b, const Aabb* aabbs, const V3* centers) {
  const size_t n = b.n;
  b.max_ref = n + (size_t)rs_f32_to_usize((float)n * kSbSplitFactor);
  b.nodes.assign(2 * b.max_ref + 1, node_new());
  b.prim_indices.assign(b.max_ref, 0u);
  b.acc.assign(b.max_ref, aabb_new());
  b.work.assign(2 * b.max_ref + 1, 0);
  for (int axis = 0; axis < 3; ++axis) {
    b.refs[axis].assign(b.max_ref, SRef{aabb_new(), v3(0.0f, 0.0f, 0.0f), 0u});
    for (size_t i = 0; i < n; ++i) b.refs[axis][i] = SRef{aabbs[i], centers[i], (uint32_t)i};
  }
  const Aabb root = aabb_union_of_list(aabbs, n);
  b.threshold = kSbAlpha * 2.0f * aabb_half_area(root);
  b.node_count = 1;
  b.nodes[0] = root;
  b.work[0] = n;
  std::vector<SWork> stack{SWork{0, 0, n, b.max_ref, 0, false}};
  while (!stack.empty() && !b.err) {
    SWork w = stack.back();
    stack.pop_back();
    SWork a, c;
    if (sb_run(b, w, a, c)) {
      if (a.end - a.begin < c.end - c.begin) std::swap(a, c);
      stack.push_back(c);
      stack.push_back(a);
    }
  }
  if (!b.err) b.nodes.resize(b.node_count);
}

// TaskSpawner::run_task (src/utils.rs:246-283): the child with more
// references goes to a new thread when it has more than `threshold` of
// them, else onto this thread's stack after the other one; spawned threads
// are joined at the end. Tasks touch disjoint reference ranges and fresh
// nodes, so they run concurrently; numbers and leaf ranges come out in
// thread-timing order and sb_canonical renumbers them.
void sb_run_task_threads(SpatialBuild& b, SWork root, size_t threshold) {
  std::vector<std::thread> spawned;
  std::vector<SWork> stack{root};
  while (!stack.empty() && !b.err) {
    SWork w = stack.back();
    stack.pop_back();
    SWork a, c;
    if (sb_run(b, w, a, c)) {
      if (a.end - a.begin < c.end - c.begin) std::swap(a, c);
      stack.push_back(c);
      if (a.end - a.begin <= threshold) {
        stack.push_back(a);
        continue;
      }
      spawned.emplace_back([&b, a, threshold]() { sb_run_task_threads(b, a, threshold); });
    }
  }
  for (auto& t : spawned) t.join();
}

// Renumbers a finished tree in the single-thread order of build_spatial:
// node pairs handed out in pre-order with the child of larger work first,
// leaf index ranges in the same order.
void sb_canonical(SpatialBuild& b) {
  std::vector<BvhNode> out(b.node_count);
  std::vector<uint32_t> idx(b.max_ref, 0u);
  std::vector<std::pair<size_t, size_t>> stack{{0, 0}};  // (old id, new id)
  size_t next_pair = 1, next_ref = 0;
  while (!stack.empty()) {
    const std::pair<size_t, size_t> top = stack.back();
    stack.pop_back();
    BvhNode nd = b.nodes[top.first];
    if (nd.extra1 < 0) {
      const size_t old_left = (size_t)nd.extra2, pair = next_pair;
      next_pair += 2;
      nd.extra2 = (int32_t)pair;
      size_t a = old_left, c = old_left + 1, na = pair, nc = pair + 1;
      if (b.work[a] < b.work[c]) {
        std::swap(a, c);
        std::swap(na, nc);
      }
      stack.push_back({c, nc});
      stack.push_back({a, na});
    } else {
      const size_t count = (size_t)nd.extra1, first = (size_t)nd.extra2;
      for (size_t k = 0; k < count; ++k) idx[next_ref + k] = b.prim_indices[first + k];
      nd.extra2 = (int32_t)next_ref;
      next_ref += count;
    }
    out[top.second] = nd;
  }
  b.nodes.swap(out);
  b.prim_indices.swap(idx);
}

// build_spatial with the reference's threading (spawn_threshold references:
// 1024 in TaskSpawner::new), numbered afterwards as build_spatial numbers.
void build_spatial_threads(SpatialBuild& b, const Aabb* aabbs, const V3* centers, size_t spawn_threshold) {
  const size_t n = b.n;
  b.max_ref = n + (size_t)rs_f32_to_usize((float)n * kSbSplitFactor);
  b.nodes.assign(2 * b.max_ref + 1, node_new());
  b.prim_indices.assign(b.max_ref, 0u);
  b.acc.assign(b.max_ref, aabb_new());
  b.work.assign(2 * b.max_ref + 1, 0);
  for (int axis = 0; axis < 3; ++axis) {
    b.refs[axis].assign(b.max_ref, SRef{aabb_new(), v3(0.0f, 0.0f, 0.0f), 0u});
    for (size_t i = 0; i < n; ++i) b.refs[axis][i] = SRef{aabbs[i], centers[i], (uint32_t)i};
  }
  const Aabb root = aabb_union_of_list(aabbs, n);
  b.threshold = kSbAlpha * 2.0f * aabb_half_area(root);
  b.node_count = 1;
  b.nodes[0] = root;
  b.work[0] = n;
  sb_run_task_threads(b, SWork{0, 0, n, b.max_ref, 0, false}, spawn_threshold);
  if (b.err) return;
  b.nodes.resize(b.node_count);
  sb_canonical(b);
}

void load_aabbs(const float* raw, size_t n, std::vector<Aabb>& out) {
  out.resize(n);
  if (n) std::memcpy(out.data(), raw, n * sizeof(Aabb));
}
void load_centers(const float* raw, size_t n, std::vector<V3>& out) {
  out.resize(n);
  for (size_t i = 0; i < n; ++i) out[i] = v3(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]);
}

}  // namespace

// ================================================================= C API
// Array layouts (all little-endian, float32 unless stated):
//   aabbs   n x 8  : RTAabb {min[3], i32 count, max[3], i32 left_first}
//   centers n x 3
//   nodes   m x 8  : RTBvhNode (same layout as RTAabb)
//   mnodes  k x 32 : RTMbvhNode {min_x[4],max_x[4],min_y[4],max_y[4],min_z[4],max_z[4], i32 children[4], i32 counts[4]}
//   tris    n x 9  : v0, v1, v2 of primitive i (primitive-id order)
//   rays    R x 6  : origin, direction
//   hits    R x 4  : t, u, v, i32 prim (-1: none)
//   stats   R x 3  : u32 node visits, u32 triangle tests, u32 max stack depth
extern "C" {

int32_t ror_abi_sizes(int32_t which) {
  switch (which) {
    case 0: return (int32_t)sizeof(Aabb);
    case 1: return (int32_t)sizeof(BvhNode);
    case 2: return (int32_t)sizeof(MbvhNode);
    default: return -1;
  }
}

uint32_t ror_morton_split(uint32_t v) { return morton_split(v); }

// Triangle::aabb and Triangle::center of the shared crate
// (shared/src/lib.rs:27-39; also src/lib.rs:166-178): the empty box grown by
// the three vertices, and ((v0 + v1) + v2) * (1/3).
void ror_triangle_prep(const float* tris, size_t n, float* aabbs_out, float* centers_out) {
  const float third = 1.0f / 3.0f;
  for (size_t i = 0; i < n; ++i) {
    const float* t = tris + 9 * i;
    Aabb a = aabb_new();
    aabb_grow(a, v3(t[0], t[1], t[2]));
    aabb_grow(a, v3(t[3], t[4], t[5]));
    aabb_grow(a, v3(t[6], t[7], t[8]));
    std::memcpy(aabbs_out + 8 * i, &a, sizeof(Aabb));
    for (int k = 0; k < 3; ++k) centers_out[3 * i + k] = ((t[k] + t[3 + k]) + t[6 + k]) * third;
  }
}

// src/utils.rs:42-57
uint32_t ror_prefix_sum_u32(const uint32_t* first, size_t count, uint32_t* output) {
  if (count == 0) return first[0];
  uint32_t sum = 0;
  for (size_t i = 0; i < count; ++i) { sum += first[i]; output[i] = sum; }
  return sum;
}

// src/aabb.rs:124-131
void ror_union_of_list(const float* aabbs, size_t n, float* out8) {
  std::vector<Aabb> a;
  load_aabbs(aabbs, n, a);
  Aabb r = aabb_union_of_list(a.data(), n);
  std::memcpy(out8, &r, sizeof(Aabb));
}

// Morton codes of the centres against the world box of the aabbs
// (src/builders/locb.rs:19-20 + src/morton.rs:63-102).
void ror_morton_codes(const float* aabbs, const float* centers, size_t n, uint32_t* codes_out,
                      uint32_t* sorted_idx_out) {
  std::vector<Aabb> a;
  std::vector<V3> c;
  load_aabbs(aabbs, n, a);
  load_centers(centers, n, c);
  Aabb world = aabb_union_of_list(a.data(), n);
  MortonEncoder enc = morton_encoder_new(world, 1u << 10);
  std::vector<uint32_t> idx, codes;
  morton_sorted(enc, c.data(), n, idx, codes, 1);
  if (n) {
    std::memcpy(codes_out, codes.data(), n * 4);
    std::memcpy(sorted_idx_out, idx.data(), n * 4);
  }
}

// Builds. nodes_out must hold 2n-1 nodes, idx_out n entries. Return value:
// node count (>= 0), -2 no primitives, -5 a LOCB level without a merge.
// build_type: 0 = locally ordered clustering, 1 = binned SAH.
// spawn_threshold: 0 = single worker (canonical numbering), else the
// TaskSpawner threshold (1024 in the reference).
int64_t ror_build(const float* aabbs, const float* centers, size_t n, size_t prims_per_leaf, int32_t build_type,
                  size_t spawn_threshold, uint32_t threads, float* nodes_out, uint32_t* idx_out) {
  if (n == 0) return -2;
  std::vector<Aabb> a;
  std::vector<V3> c;
  load_aabbs(aabbs, n, a);
  load_centers(centers, n, c);
  Bvh b;
  if (build_type == 0) {
    int err = 0;
    b = build_locb(a.data(), c.data(), n, &err, threads);
    if (err) return -5;
  } else {
    b = build_binned_sah(a.data(), c.data(), n, prims_per_leaf, spawn_threshold == 0 ? SIZE_MAX : spawn_threshold);
  }
  std::memcpy(nodes_out, b.nodes.data(), b.nodes.size() * sizeof(BvhNode));
  std::memcpy(idx_out, b.prim_indices.data(), b.prim_indices.size() * 4);
  return (int64_t)b.nodes.size();
}

// Spatial-split SAH (src/builders/spatial_sah.rs; see build_spatial for the
// task order). spawn_threshold: 0 = one thread, else TaskSpawner's
// threading with that threshold (same output). tris: n x 9 vertices,
// aabbs: n x 8, centers: n x 3. nodes_out
// holds nodes_cap nodes (2 * max_refs + 1 suffice), idx_out idx_cap entries
// (max_refs: the reference returns all of them, unused ones 0). Returns the
// node count, -2 no primitives, -3 an input on which the reference panics or
// writes out of bounds, -4 output too small.
uint64_t ror_spatial_max_refs(size_t n) { return n + rs_f32_to_usize((float)n * kSbSplitFactor); }

int64_t ror_build_spatial(const float* aabbs, const float* centers, const float* tris, size_t n, size_t prims_per_leaf,
                          uint32_t fixes, size_t spawn_threshold, float* nodes_out, size_t nodes_cap, uint32_t* idx_out,
                          size_t idx_cap) {
  if (n == 0) return -2;
  std::vector<Aabb> a;
  std::vector<V3> c;
  load_aabbs(aabbs, n, a);
  load_centers(centers, n, c);
  SpatialBuild b;
  b.tris = tris;
  b.n = n;
  b.max_leaf = prims_per_leaf == 0 ? 1 : prims_per_leaf;
  b.fixes = fixes;
  if (spawn_threshold == 0) build_spatial(b, a.data(), c.data());
  else build_spatial_threads(b, a.data(), c.data(), spawn_threshold);
  if (b.err) return -3;
  if (b.nodes.size() > nodes_cap || b.prim_indices.size() > idx_cap) return -4;
  std::memcpy(nodes_out, b.nodes.data(), b.nodes.size() * sizeof(BvhNode));
  std::memcpy(idx_out, b.prim_indices.data(), b.prim_indices.size() * 4);
  return (int64_t)b.nodes.size();
}

// src/bvh.rs:381-404. mnodes_out must hold node_count entries; returns the
// number of quad nodes.
int64_t ror_mbvh(const float* nodes, size_t node_count, float* mnodes_out) {
  std::vector<Aabb> nd;
  load_aabbs(nodes, node_count, nd);
  std::vector<MbvhNode> m = mbvh_construct(nd.data(), node_count);
  if (!m.empty()) std::memcpy(mnodes_out, m.data(), m.size() * sizeof(MbvhNode));
  return (int64_t)m.size();
}

// src/bvh.rs:176-205, in place.
void ror_refit(float* nodes, size_t node_count, const uint32_t* prim_indices, const float* new_aabbs,
               size_t prim_count) {
  std::vector<Aabb> nd, na;
  load_aabbs(nodes, node_count, nd);
  load_aabbs(new_aabbs, prim_count, na);
  refit(nd.data(), node_count, prim_indices, na.data());
  std::memcpy(nodes, nd.data(), node_count * sizeof(Aabb));
}

// src/bvh.rs:232-244
int32_t ror_validate(const float* nodes, size_t node_count, const uint32_t* idx, size_t prim_count) {
  if (node_count == 0) return 0;
  std::vector<Aabb> nd;
  load_aabbs(nodes, node_count, nd);
  std::vector<uint8_t> checks(prim_count, 0);
  bool ok = true;
  traverse_check(nd.data(), idx, nd[0], checks.data(), prim_count, ok);
  for (size_t i = 0; i < prim_count; ++i)
    if (!checks[i]) ok = false;
  return ok ? 1 : 0;
}

// Traversal of R rays (closest hit, or any hit when any_hit != 0). t_max is
// either one value per ray (t_max != NULL) or the Ray::new default of 1e34.
// t_min_tri is the triangle test's lower bound (Ray::t_min = 1e-4 in the
// crate; the FFI test callback uses 1e-5). structure: 0 = Mbvh, 1 = Bvh.
// threads > 1 splits the rays into chunks of 1000, as examples/benchmark.rs:25.
// Returns the number of rays whose traversal stack exceeded the oracle's
// bound (0 expected).
int64_t ror_trace(int32_t structure, const float* nodes, size_t node_count, const uint32_t* idx, const float* tris,
                  const float* rays, size_t nrays, const float* t_max, float t_min_tri, int32_t any_hit,
                  float* hits_out, uint32_t* stats_out, uint32_t threads) {
  std::atomic<int64_t> bad{0};
  std::atomic<size_t> next{0};
  const size_t chunk = 1000;
  auto worker = [&]() {
    for (;;) {
      size_t c0 = next.fetch_add(chunk);
      if (c0 >= nrays) break;
      size_t c1 = std::min(nrays, c0 + chunk);
      for (size_t r = c0; r < c1; ++r) {
        const float* rr = rays + 6 * r;
        Ray ray = ray_new(v3(rr[0], rr[1], rr[2]), v3(rr[3], rr[4], rr[5]));
        if (t_max) ray.t = t_max[r];
        Hit h;
        Stats st;
        if (structure == 0)
          trace_mbvh_one(reinterpret_cast<const MbvhNode*>(nodes), node_count, idx, tris, ray, t_min_tri,
                         any_hit != 0, h, st);
        else
          trace_bvh_one(reinterpret_cast<const BvhNode*>(nodes), node_count, idx, tris, ray, t_min_tri,
                        any_hit != 0, h, st);
        if (h.prim == -2) { bad.fetch_add(1); h.prim = -1; }
        if (hits_out) {
          float* ho = hits_out + 4 * r;
          ho[0] = h.t; ho[1] = h.u; ho[2] = h.v;
          std::memcpy(ho + 3, &h.prim, 4);
        }
        if (stats_out) {
          stats_out[3 * r + 0] = (uint32_t)st.node_visits;
          stats_out[3 * r + 1] = (uint32_t)st.tri_tests;
          stats_out[3 * r + 2] = st.max_stack;
        }
      }
    }
  };
  if (threads <= 1) {
    worker();
  } else {
    std::vector<std::thread> ts;
    for (uint32_t t = 0; t < threads; ++t) ts.emplace_back(worker);
    for (auto& th : ts) th.join();
  }
  return bad.load();
}

// Candidate lists: the primitives MbvhIndexIterator (src/iter_indices.rs:
// 212-313, structure 0) or BvhIndexIterator (:18-107, structure 1) yields for
// each ray when the callback never changes t (rtbvh_ffi/src/lib.rs:700-731
// with a callback that returns false and leaves t alone), in yield order.
// Ray r's first max_per_ray ids go to cand_out[r * max_per_ray ...];
// counts_out[r] is the full number of yields. Returns the number of rays
// whose stack exceeded the oracle's bound.
int64_t ror_candidates(int32_t structure, const float* nodes, size_t node_count, const uint32_t* idx,
                       const float* rays, size_t nrays, const float* t_max, uint32_t max_per_ray,
                       uint32_t* cand_out, uint32_t* counts_out) {
  int64_t bad = 0;
  for (size_t r = 0; r < nrays; ++r) {
    const float* rr = rays + 6 * r;
    Ray ray = ray_new(v3(rr[0], rr[1], rr[2]), v3(rr[3], rr[4], rr[5]));
    if (t_max) ray.t = t_max[r];
    uint32_t n = 0;
    auto yield = [&](uint32_t prim) {
      if (n < max_per_ray) cand_out[r * (size_t)max_per_ray + n] = prim;
      ++n;
    };
    int32_t stack[ORACLE_STACK];
    if (structure == 0) {
      const MbvhNode* m = reinterpret_cast<const MbvhNode*>(nodes);
      if (node_count > 0) {
        MbvhHit hit = mnode_intersect(m[0], ray);
        int32_t current = 0, sp = -1;
        for (;;) {
          const MbvhNode& node = m[current];
          for (int i = 0; i < 4; ++i) {
            const int id = hit.ids[3 - i];
            if (!hit.result[id]) continue;
            const int32_t count = node.counts[id], lf = node.children[id];
            if (count > -1) {
              for (int32_t j = 0; j < count; ++j) yield(idx[lf + j]);
            } else if (lf > -1) {
              if (sp + 1 >= ORACLE_STACK) { ++bad; sp = -1; break; }
              stack[++sp] = lf;
            }
          }
          if (sp < 0) break;
          current = stack[sp--];
          hit = mnode_intersect(m[current], ray);
        }
      }
    } else {
      const BvhNode* b = reinterpret_cast<const BvhNode*>(nodes);
      if (node_count > 0 && !v3_is_nan(ray.origin) && !v3_is_nan(ray.direction)) {
        stack[0] = 0;
        int32_t sp = 0;
        while (sp >= 0) {
          const BvhNode& node = b[stack[sp--]];
          const int32_t count = node.extra1, lf = node.extra2;
          if (count > -1) {
            for (int32_t j = 0; j < count; ++j) yield(idx[lf + j]);
          } else if (lf > -1) {
            float lt = 0.0f, rt = 0.0f;
            const bool lh = aabb_intersect(b[lf], ray, &lt), rh = aabb_intersect(b[lf + 1], ray, &rt);
            if (sp + 2 >= ORACLE_STACK) { ++bad; break; }
            sp = sort_nodes(lh, lt, rh, rt, stack, sp, lf);
          }
        }
      }
    }
    counts_out[r] = n;
  }
  return bad;
}

// Packet traversal of P packets of four rays (closest hit through the
// packet triangle test). soa = 6 arrays of 4P floats each (origin x, y, z,
// direction x, y, z; lane k of packet p at 4p + k); t is 4P floats, in/out
// (the FFI's t). hits_out: 4P x 4 (t, u, v, prim), stats_out: P x 3 (quad /
// BVH2 node tests, triangle yields, max stack depth). threads > 1 splits the
// packets into chunks of 1000, as examples/benchmark.rs:43-68. Returns the
// number of packets whose stack exceeded the oracle's bound.
int64_t ror_trace_packets(int32_t structure, const float* nodes, size_t node_count, const uint32_t* idx,
                          const float* tris, const float* const* soa, float* t, size_t npackets, float t_min_tri,
                          float* hits_out, uint32_t* stats_out, uint32_t threads) {
  std::atomic<int64_t> bad{0};
  std::atomic<size_t> next{0};
  const size_t chunk = 1000;
  auto worker = [&]() {
    for (;;) {
      size_t c0 = next.fetch_add(chunk);
      if (c0 >= npackets) break;
      size_t c1 = std::min(npackets, c0 + chunk);
      for (size_t q = c0; q < c1; ++q) {
        Packet4 p;
        PacketOut o;
        for (int k = 0; k < 4; ++k) {
          const size_t r = 4 * q + k;
          p.ox[k] = soa[0][r]; p.oy[k] = soa[1][r]; p.oz[k] = soa[2][r];
          p.dx[k] = soa[3][r]; p.dy[k] = soa[4][r]; p.dz[k] = soa[5][r];
          p.ix[k] = 1.0f / p.dx[k]; p.iy[k] = 1.0f / p.dy[k]; p.iz[k] = 1.0f / p.dz[k];
          p.t[k] = t[r];
          o.u[k] = o.v[k] = 0.0f;
          o.prim[k] = -1;
        }
        Stats st;
        const bool ok = structure == 0
                            ? trace_mbvh_packet(reinterpret_cast<const MbvhNode*>(nodes), node_count, idx, tris, p,
                                                t_min_tri, o, st)
                            : trace_bvh_packet(reinterpret_cast<const BvhNode*>(nodes), node_count, idx, tris, p,
                                               t_min_tri, o, st);
        if (!ok) bad.fetch_add(1);
        for (int k = 0; k < 4; ++k) {
          const size_t r = 4 * q + k;
          t[r] = p.t[k];
          if (hits_out) {
            float* ho = hits_out + 4 * r;
            ho[0] = p.t[k]; ho[1] = o.u[k]; ho[2] = o.v[k];
            std::memcpy(ho + 3, &o.prim[k], 4);
          }
        }
        if (stats_out) {
          stats_out[3 * q + 0] = (uint32_t)st.node_visits;
          stats_out[3 * q + 1] = (uint32_t)st.tri_tests;
          stats_out[3 * q + 2] = st.max_stack;
        }
      }
    }
  };
  if (threads <= 1) {
    worker();
  } else {
    std::vector<std::thread> ts;
    for (uint32_t k = 0; k < threads; ++k) ts.emplace_back(worker);
    for (auto& th : ts) th.join();
  }
  return bad.load();
}

}  // extern "C"
