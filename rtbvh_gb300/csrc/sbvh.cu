// Spatial-split SAH build (src/builders/spatial_sah.rs) on the GPU.
//
// The reference runs Task::run (:726-838) once per node; a task reads and
// writes only its own region [begin, split_end) of the three per-axis
// reference arrays (its references plus its split space), and the regions of
// live tasks are disjoint. So tasks are independent once created and their
// results do not depend on the order they run in -- except the node numbers
// and leaf index ranges, which the reference hands out from two atomic
// counters (AtomicNodeStack::allocate, make_leaf). Here:
//
//  * k_sb_build is a persistent kernel over a global task queue: a block
//    takes a task, runs the whole of Task::run for it (sorts, object-split
//    sweep, spatial binning passes, the chosen partition, allocate_children)
//    and queues the two children. Parallel parts use the block's threads;
//    the reference's in-place partitions whose result is a particular
//    permutation (the three-way swap loop and the straddler loop of
//    apply_spatial_split) are replayed by one thread on a permutation array
//    and then applied by all threads.
//  * k_sb_counts / k_sb_ranks / k_sb_write number the finished tree in the
//    order of the reference's single-thread schedule (depth first, the child
//    with more references first): interior node k of that order gets the
//    child pair 1 + 2k, leaves take index ranges in the same order.
//
// Reference records are values (two float4: min + prim, max), as in the
// reference, because its allocate_children leaves stale copies behind that
// later writes must not alias. A record whose prim carries kSbFrag is a
// split fragment; its centre is the centre of its box, otherwise the
// primitive's centre.
//
// `fixes` (RTBVH_SPATIAL_FIX_*) switches on corrections of reference
// defects; 0 reproduces the reference as written.
#include <algorithm>
#include <cfloat>

#include "lib_internal.h"

namespace rtbvh {
namespace {

constexpr int kSbThreads = 256;
constexpr int kSbWarps = kSbThreads / 32;
constexpr int kSbBins = 16;
constexpr int kSbPasses = 2;
constexpr uint32_t kSbMaxDepth = 64;
constexpr int kSbTile = 2048;  // keys sorted in shared memory at once
constexpr int kSbMergeItems = 8;
constexpr uint32_t kSbClsWords = 1024;            // shared class words: 16 classes each
constexpr uint32_t kSbClsCap = kSbClsWords * 16;  // tasks up to this size replay from shared memory
constexpr uint32_t kSbFrag = 0x80000000u;
constexpr uint32_t kSbNone = 0xffffffffu;
constexpr uint32_t kSbSpin = 1u << 22;  // queue waits (~1 us apart): a few seconds, then kStatusTimeout
constexpr float kSbTraversalCost = 1.0f, kSbAlpha = 1e-5f, kSbSplitFactor = 0.75f;
constexpr uint32_t kSbAbort = 1u << 31;  // in the control word: stop taking tasks
constexpr uint32_t kSbPanic = 1u << 5;   // an input on which the reference panics

constexpr uint32_t kFixClip = 1, kFixExitBin = 2, kFixSweepBox = 4, kFixSplitSpace = 8, kFixFallback = 16;

// Classes of apply_spatial_split's partition (:622-640).
constexpr uint8_t kClsLeft = 0, kClsRight = 1, kClsStraddle = 2;
// Permutation entries: source slot | kind << 30.
constexpr uint32_t kKindLeftFrag = 1u << 30, kKindRightFrag = 2u << 30, kSlotMask = (1u << 30) - 1;

struct SbRef {
  float4 lo;  // min.xyz, w = prim | kSbFrag
  float4 hi;  // max.xyz, w = 0
};

struct SbTask {
  uint32_t begin, end, split_end, meta;  // meta: depth | sorted << 8
  float4 lo;                             // the node's box as its parent set it; w = parent task (uint)
  float4 hi;                             // w unused
};

struct SbCtl {
  uint32_t head, tail, done, status;
  float threshold;  // spatial_threshold (:964): alpha * 2 * half area of the root bounds
};

struct SbArgs {
  SbRef* refs[3];
  SbRef* scr;
  unsigned long long* keys;
  unsigned long long* keys2;
  float* fbuf;
  uint32_t* perm;
  uint8_t* cls;
  uint32_t* hkeys;
  uint32_t* hvals;
  SbTask* tasks;
  uint32_t* ready;
  uint32_t* child;  // left child task (right = +1), kSbNone for a leaf
  SbCtl* ctl;
  const float* tris;     // n x 9
  const float4* centers;
  uint32_t n, max_ref, task_cap, max_leaf, fixes;
};

// ------------------------------------------------------------------ boxes
struct SbBox {
  float mn[3], mx[3];
};
__device__ __forceinline__ SbBox sb_empty() {
  SbBox b;
  for (int k = 0; k < 3; ++k) { b.mn[k] = 1e34f; b.mx[k] = -1e34f; }
  return b;
}
// Aabb::grow_bb (src/aabb.rs:263-273)
__device__ __forceinline__ void sb_grow(SbBox& a, const SbBox& b) {
  for (int k = 0; k < 3; ++k) { a.mn[k] = rs_min(a.mn[k], b.mn[k]); a.mx[k] = rs_max(a.mx[k], b.mx[k]); }
}
// Aabb::grow (src/aabb.rs:251-261)
__device__ __forceinline__ void sb_grow_pt(SbBox& a, float x, float y, float z) {
  a.mn[0] = rs_min(a.mn[0], x); a.mx[0] = rs_max(a.mx[0], x);
  a.mn[1] = rs_min(a.mn[1], y); a.mx[1] = rs_max(a.mx[1], y);
  a.mn[2] = rs_min(a.mn[2], z); a.mx[2] = rs_max(a.mx[2], z);
}
// Aabb::shrink (src/aabb.rs:288-298)
__device__ __forceinline__ void sb_shrink(SbBox& a, const SbBox& b) {
  for (int k = 0; k < 3; ++k) { a.mn[k] = rs_max(a.mn[k], b.mn[k]); a.mx[k] = rs_min(a.mx[k], b.mx[k]); }
}
__device__ __forceinline__ float sb_half_area(const SbBox& a) {
  return half_area(a.mn[0], a.mn[1], a.mn[2], a.mx[0], a.mx[1], a.mx[2]);
}
// Aabb::area (src/aabb.rs:334-340)
__device__ __forceinline__ float sb_area(const SbBox& a) {
  float ex = a.mx[0] - a.mn[0], ey = a.mx[1] - a.mn[1], ez = a.mx[2] - a.mn[2];
  float v = ((ex * ey) + (ex * ez)) + (ey * ez);
  return rs_max(0.0f, v);
}
// Aabb::is_valid (src/aabb.rs:141-143)
__device__ __forceinline__ bool sb_valid(const SbBox& a) {
  return a.mn[0] <= a.mx[0] && a.mn[1] <= a.mx[1] && a.mn[2] <= a.mx[2];
}
// Aabb::longest_axis (src/aabb.rs:353-363)
__device__ __forceinline__ int sb_longest_axis(const SbBox& a) {
  int ax = 0;
  if ((a.mx[1] - a.mn[1]) > (a.mx[0] - a.mn[0])) ax = 1;
  if ((a.mx[2] - a.mn[2]) > (a.mx[ax] - a.mn[ax])) ax = 2;
  return ax;
}
__device__ __forceinline__ float sb_axis(float x, float y, float z, int ax) { return ax == 0 ? x : (ax == 1 ? y : z); }

__device__ __forceinline__ SbRef sb_load(const SbRef* p) {
  SbRef r;
  r.lo = __ldcg(&p->lo);
  r.hi = __ldcg(&p->hi);
  return r;
}
__device__ __forceinline__ void sb_store(SbRef* p, const SbRef& r) {
  p->lo = r.lo;
  p->hi = r.hi;
}
__device__ __forceinline__ SbBox sb_ref_box(const SbRef& r) {
  SbBox b;
  b.mn[0] = r.lo.x; b.mn[1] = r.lo.y; b.mn[2] = r.lo.z;
  b.mx[0] = r.hi.x; b.mx[1] = r.hi.y; b.mx[2] = r.hi.z;
  return b;
}
__device__ __forceinline__ uint32_t sb_prim(const SbRef& r) { return __float_as_uint(r.lo.w) & ~kSbFrag; }
__device__ __forceinline__ SbRef sb_make_ref(const SbBox& b, uint32_t prim_flags) {
  SbRef r;
  r.lo = make_float4(b.mn[0], b.mn[1], b.mn[2], __uint_as_float(prim_flags));
  r.hi = make_float4(b.mx[0], b.mx[1], b.mx[2], 0.0f);
  return r;
}
// SpatialReference::center: Primitive::center of the triangle for an input
// reference, Aabb::center (src/aabb.rs:329-332) of the box for a fragment.
__device__ __forceinline__ float sb_center(const SbRef& r, int ax, const float4* centers) {
  const uint32_t w = __float_as_uint(r.lo.w);
  if (w & kSbFrag) {
    float a = sb_axis(r.lo.x, r.lo.y, r.lo.z, ax), b = sb_axis(r.hi.x, r.hi.y, r.hi.z, ax);
    return (a + b) * 0.5f;
  }
  const float4 c = __ldg(centers + w);
  return sb_axis(c.x, c.y, c.z, ax);
}

// SpatialTriangle::split (spatial_sah.rs:85-129).
__device__ void sb_tri_split(const float* tri, int axis, float position, bool fix_clip, SbBox& left, SbBox& right) {
  float p[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int k = 0; k < 3; ++k) p[v][k] = __ldg(tri + 3 * v + k);
  left = sb_empty();
  right = sb_empty();
  bool q[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    q[v] = p[v][axis] <= position;
    sb_grow_pt(q[v] ? left : right, p[v][0], p[v][1], p[v][2]);
  }
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int a = e, b = (e + 1) % 3;
    if (q[a] != q[b]) {
      const float t = (position - p[a][axis]) / (p[b][axis] - p[a][axis]);
      float m[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float d = p[b][k] - p[a][k];
        m[k] = fix_clip ? p[a][k] + t * d : (p[a][k] * t) * d;
      }
      sb_grow_pt(left, m[0], m[1], m[2]);
      sb_grow_pt(right, m[0], m[1], m[2]);
    }
  }
}

// The fragments of a straddling reference: the triangle split at `position`,
// each side shrunk to the reference's box (:659-663).
__device__ __forceinline__ SbRef sb_fragment(const SbArgs& A, const SbRef& r, int axis, float position, bool right) {
  SbBox lb, rb;
  sb_tri_split(A.tris + 9 * (size_t)sb_prim(r), axis, position, A.fixes & kFixClip, lb, rb);
  SbBox b = right ? rb : lb;
  sb_shrink(b, sb_ref_box(r));
  return sb_make_ref(b, sb_prim(r) | kSbFrag);
}

// Rust `f32 as usize`.
__device__ __forceinline__ unsigned long long sb_f2usize(float f) {
  if (!(f > 0.0f)) return 0ull;
  if (f >= 1.8446744073709552e19f) return ~0ull;
  return (unsigned long long)f;
}

// ------------------------------------------------------------------ block helpers
struct SbShared {
  // task scalars, broadcast by thread 0
  uint32_t task, begin, end, split_end, depth, sorted, n;
  float nb[6];
  uint32_t fail;
  // object split result
  float obj_cost;
  uint32_t obj_axis, obj_index;  // obj_index kSbNone: None
  // spatial split state (:46-61)
  float sp_cost, sp_pos;
  uint32_t sp_axis, found;
  float pass_lo, pass_hi;
  uint32_t first_invalid;
  // partition results (relative to begin)
  uint32_t le, rb, re;
  uint32_t lsc;
  uint32_t use_spatial;
  float boxes[2][6];
  // reductions
  float red[kSbWarps][6];
  uint32_t redu[kSbWarps][2];
  float redc[kSbWarps];
  uint32_t redk[kSbWarps][2];
  uint32_t cls2[kSbClsWords];  // spatial partition classes, 2 bits each
  union {
    unsigned long long tile[kSbTile];
    struct {
      uint32_t mn[kSbBins][3], mx[kSbBins][3];
      uint32_t entry[kSbBins], exit[kSbBins];
    } bins;
  } u;
};

__device__ __forceinline__ void sb_warp_union(SbBox& b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      b.mn[k] = rs_min(b.mn[k], __shfl_xor_sync(0xffffffffu, b.mn[k], o));
      b.mx[k] = rs_max(b.mx[k], __shfl_xor_sync(0xffffffffu, b.mx[k], o));
    }
  }
}

// Union of the boxes of refs [lo, hi) (Aabb::grow_bb over a range; the union
// is order-independent). Result in every thread.
__device__ SbBox sb_block_union(SbShared& sh, const SbRef* refs, uint32_t lo, uint32_t hi) {
  SbBox b = sb_empty();
  for (uint32_t i = lo + threadIdx.x; i < hi; i += kSbThreads) sb_grow(b, sb_ref_box(sb_load(refs + i)));
  sb_warp_union(b);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0)
    for (int k = 0; k < 3; ++k) { sh.red[w][k] = b.mn[k]; sh.red[w][3 + k] = b.mx[k]; }
  __syncthreads();
  SbBox r = sb_empty();
  for (int j = 0; j < kSbWarps; ++j)
    for (int k = 0; k < 3; ++k) { r.mn[k] = rs_min(r.mn[k], sh.red[j][k]); r.mx[k] = rs_max(r.mx[k], sh.red[j][3 + k]); }
  __syncthreads();
  return r;
}

__device__ uint32_t sb_block_min(SbShared& sh, uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh.redu[threadIdx.x >> 5][0] = v;
  __syncthreads();
  uint32_t r = sh.redu[0][0];
  for (int j = 1; j < kSbWarps; ++j) r = min(r, sh.redu[j][0]);
  __syncthreads();
  return r;
}

__device__ uint32_t sb_block_sum(SbShared& sh, uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh.redu[threadIdx.x >> 5][0] = v;
  __syncthreads();
  uint32_t r = 0;
  for (int j = 0; j < kSbWarps; ++j) r += sh.redu[j][0];
  __syncthreads();
  return r;
}

// Exclusive scan of one u32 per thread over the block; *total gets the sum.
__device__ uint32_t sb_block_exscan(SbShared& sh, uint32_t v, uint32_t* total) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (l >= o) x += y;
  }
  __syncthreads();
  if (l == 31) sh.redu[w][0] = x;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (int j = 0; j < kSbWarps; ++j) {
    if (j < w) before += sh.redu[j][0];
    all += sh.redu[j][0];
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

// Inclusive scan of boxes over the block in thread order; returns this
// thread's prefix union and sets *total to the union of all.
__device__ SbBox sb_block_scan_box(SbShared& sh, SbBox b, SbBox* total) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    SbBox y;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      y.mn[k] = __shfl_up_sync(0xffffffffu, b.mn[k], o);
      y.mx[k] = __shfl_up_sync(0xffffffffu, b.mx[k], o);
    }
    if (l >= o) sb_grow(b, y);
  }
  __syncthreads();
  if (l == 31)
    for (int k = 0; k < 3; ++k) { sh.red[w][k] = b.mn[k]; sh.red[w][3 + k] = b.mx[k]; }
  __syncthreads();
  SbBox before = sb_empty(), all = sb_empty();
  for (int j = 0; j < kSbWarps; ++j) {
    SbBox t;
    for (int k = 0; k < 3; ++k) { t.mn[k] = sh.red[j][k]; t.mx[k] = sh.red[j][3 + k]; }
    if (j < w) sb_grow(before, t);
    sb_grow(all, t);
  }
  __syncthreads();
  sb_grow(before, b);
  *total = all;
  return before;
}

// Copies refs [lo, hi) of `src` to `dst` (distinct arrays).
__device__ __forceinline__ void sb_copy(SbRef* dst, const SbRef* src, uint32_t lo, uint32_t hi) {
  for (uint32_t i = lo + threadIdx.x; i < hi; i += kSbThreads) sb_store(dst + i, sb_load(src + i));
}

// ------------------------------------------------------------------ sort
// Bitonic sort of `count` keys (count <= kSbTile) in shared memory, padded
// with the largest key to a power of two.
__device__ void sb_tile_sort(SbShared& sh, unsigned long long* keys, uint32_t count) {
  uint32_t p2 = 1;
  while (p2 < count) p2 <<= 1;
  for (uint32_t i = threadIdx.x; i < p2; i += kSbThreads) sh.u.tile[i] = i < count ? __ldcg(keys + i) : ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= p2; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < p2; i += kSbThreads) {
        const uint32_t ixj = i ^ j;
        if (ixj > i) {
          const unsigned long long a = sh.u.tile[i], b = sh.u.tile[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) { sh.u.tile[i] = b; sh.u.tile[ixj] = a; }
        }
      }
      __syncthreads();
    }
  }
  for (uint32_t i = threadIdx.x; i < count; i += kSbThreads) keys[i] = sh.u.tile[i];
  __syncthreads();
}

// One merge pass: sorted runs of `width` keys in src -> runs of 2 * width
// in dst (keys are distinct). Merge path: each thread finds where its
// kSbMergeItems outputs start and merges them.
__device__ void sb_merge_pass(const unsigned long long* src, unsigned long long* dst, uint32_t count, uint32_t width) {
  for (uint32_t lo = 0; lo < count; lo += 2 * width) {
    const uint32_t mid = min(lo + width, count), hi = min(lo + 2 * width, count);
    const unsigned long long* a = src + lo;
    const unsigned long long* b = src + mid;
    const uint32_t na = mid - lo, nb = hi - mid, total = hi - lo;
    for (uint32_t base = 0; base < total; base += kSbThreads * kSbMergeItems) {
      const uint32_t d = base + threadIdx.x * kSbMergeItems;
      if (d >= total) continue;
      uint32_t alo = d > nb ? d - nb : 0, ahi = min(d, na);
      while (alo < ahi) {
        const uint32_t m = (alo + ahi) >> 1;
        if (__ldcg(a + m) < __ldcg(b + (d - 1 - m))) alo = m + 1;
        else ahi = m;
      }
      uint32_t ia = alo, ib = d - alo;
      for (int k = 0; k < kSbMergeItems && d + k < total; ++k) {
        unsigned long long v;
        if (ib >= nb || (ia < na && __ldcg(a + ia) < __ldcg(b + ib))) v = __ldcg(a + ia++);
        else v = __ldcg(b + ib++);
        dst[lo + d + k] = v;
      }
    }
  }
  __syncthreads();
}

// find_object_split's sort (:316-331): references [begin, end) of axis `ax`
// stably ordered by centre. The comparator answers Less exactly when
// a < b, and the standard library's stable sort only asks "is less", so the
// order is the stable order on the centre (-0 and +0 equal). Keys are the
// order-preserving centre bits above the slot, so all keys differ.
__device__ void sb_sort_axis(const SbArgs& A, SbShared& sh, int ax, uint32_t begin, uint32_t n) {
  SbRef* refs = A.refs[ax];
  unsigned long long* k0 = A.keys + begin;
  unsigned long long* k1 = A.keys2 + begin;
  for (uint32_t i = threadIdx.x; i < n; i += kSbThreads) {
    float c = sb_center(sb_load(refs + begin + i), ax, A.centers);
    if (c == 0.0f) c = 0.0f;
    k0[i] = ((unsigned long long)float_to_ordered(c) << 32) | i;
  }
  __syncthreads();
  for (uint32_t t = 0; t < n; t += kSbTile) sb_tile_sort(sh, k0 + t, min((uint32_t)kSbTile, n - t));
  unsigned long long* src = k0;
  unsigned long long* dst = k1;
  for (uint32_t w = kSbTile; w < n; w <<= 1) {
    sb_merge_pass(src, dst, n, w);
    unsigned long long* t = src;
    src = dst;
    dst = t;
  }
  for (uint32_t i = threadIdx.x; i < n; i += kSbThreads)
    sb_store(A.scr + begin + i, sb_load(refs + begin + (uint32_t)(__ldcg(src + i) & 0xffffffffu)));
  __syncthreads();
  sb_copy(refs, A.scr, begin, begin + n);
  __syncthreads();
}

// ------------------------------------------------------------------ object split
// find_object_split's sweep (:333-365) over all three axes: the first
// minimum cost in (axis, index) order, strict `<` against f32::MAX, so NaN
// and infinite costs never win. fbuf holds the half areas of the suffix
// unions.
__device__ void sb_object_sweep(const SbArgs& A, SbShared& sh, uint32_t begin, uint32_t end) {
  float best = FLT_MAX;
  uint32_t best_axis = 0, best_index = kSbNone;
  for (int ax = 0; ax < 3; ++ax) {
    const SbRef* refs = A.refs[ax];
    // suffix unions, from the back: thread t takes element hi - 1 - t
    SbBox carry = sb_empty();
    for (uint32_t hi = end; hi > begin + 1; hi = hi > begin + 1 + kSbThreads ? hi - kSbThreads : begin + 1) {
      const uint32_t cnt = min((uint32_t)kSbThreads, hi - (begin + 1));
      SbBox b = sb_empty();
      const bool act = threadIdx.x < cnt;
      const uint32_t i = hi - 1 - threadIdx.x;
      if (act) b = sb_ref_box(sb_load(refs + i));
      SbBox total;
      SbBox s = sb_block_scan_box(sh, b, &total);
      sb_grow(s, carry);
      if (act) A.fbuf[i] = sb_half_area(s);
      sb_grow(carry, total);
    }
    __syncthreads();
    // prefix unions and costs
    carry = sb_empty();
    for (uint32_t lo = begin; lo + 1 < end; lo += kSbThreads) {
      const uint32_t cnt = min((uint32_t)kSbThreads, end - 1 - lo);
      const bool act = threadIdx.x < cnt;
      const uint32_t i = lo + threadIdx.x;
      SbBox b = sb_empty();
      if (act) b = sb_ref_box(sb_load(refs + i));
      SbBox total;
      SbBox s = sb_block_scan_box(sh, b, &total);
      sb_grow(s, carry);
      if (act) {
        const float cost = sb_half_area(s) * (float)(i + 1 - begin) + __ldcg(A.fbuf + i + 1) * (float)(end - (i + 1));
        if (cost < best) {
          best = cost;
          best_axis = ax;
          best_index = i + 1;
        }
      }
      sb_grow(carry, total);
    }
    __syncthreads();
  }
  // block arg-min: lowest cost, then lowest (axis, index)
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  unsigned long long key = ((unsigned long long)best_axis << 32) | best_index;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float c2 = __shfl_xor_sync(0xffffffffu, best, o);
    const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
    if (c2 < best || (c2 == best && k2 < key)) { best = c2; key = k2; }
  }
  if (l == 0) {
    sh.redc[w] = best;
    sh.redk[w][0] = (uint32_t)(key >> 32);
    sh.redk[w][1] = (uint32_t)key;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float bc = sh.redc[0];
    unsigned long long bk = ((unsigned long long)sh.redk[0][0] << 32) | sh.redk[0][1];
    for (int j = 1; j < kSbWarps; ++j) {
      const float c2 = sh.redc[j];
      const unsigned long long k2 = ((unsigned long long)sh.redk[j][0] << 32) | sh.redk[j][1];
      if (c2 < bc || (c2 == bc && k2 < bk)) { bc = c2; bk = k2; }
    }
    sh.obj_cost = bc;
    sh.obj_axis = (uint32_t)(bk >> 32);
    sh.obj_index = (uint32_t)bk;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ spatial binning
__device__ __forceinline__ void sb_bin_grow(SbShared& sh, uint32_t bin, const SbBox& b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (b.mn[k] == b.mn[k]) atomicMin(&sh.u.bins.mn[bin][k], float_to_ordered(b.mn[k]));
    if (b.mx[k] == b.mx[k]) atomicMax(&sh.u.bins.mx[bin][k], float_to_ordered(b.mx[k]));
  }
}
__device__ __forceinline__ SbBox sb_bin_box(const SbShared& sh, int bin) {
  SbBox b;
  for (int k = 0; k < 3; ++k) {
    b.mn[k] = ordered_to_float(sh.u.bins.mn[bin][k]);
    b.mx[k] = ordered_to_float(sh.u.bins.mx[bin][k]);
  }
  return b;
}

// find_spatial_split (:585-603) and run_binning_pass (:491-583). Binning
// covers references [begin, first invalid) of the axis-0 array (the
// reference breaks at the first invalid box); bins are unions, so the order
// of the atomic updates does not matter. Thread 0 runs the sweep.
__device__ void sb_spatial_search(const SbArgs& A, SbShared& sh, uint32_t begin, uint32_t end) {
  const SbRef* r0 = A.refs[0];
  uint32_t fi = end;
  for (uint32_t i = begin + threadIdx.x; i < end; i += kSbThreads)
    if (!sb_valid(sb_ref_box(sb_load(r0 + i)))) fi = min(fi, i);
  fi = sb_block_min(sh, fi);
  if (threadIdx.x == 0) {
    sh.sp_cost = FLT_MAX;
    sh.sp_pos = 0.0f;
    sh.sp_axis = 0;
  }
  const bool fix_clip = A.fixes & kFixClip;
  for (int ax = 0; ax < 3; ++ax) {
    if (threadIdx.x == 0) {
      sh.pass_lo = sh.nb[ax];
      sh.pass_hi = sh.nb[3 + ax];
    }
    __syncthreads();
    for (int pass = 0; pass < kSbPasses; ++pass) {
      const float mn = sh.pass_lo, mx = sh.pass_hi;
      const float bin_size = (mx - mn) / (float)kSbBins;
      const float inv_size = 1.0f / bin_size;
      if (threadIdx.x < kSbBins) {
        for (int k = 0; k < 3; ++k) {
          sh.u.bins.mn[threadIdx.x][k] = float_to_ordered(1e34f);
          sh.u.bins.mx[threadIdx.x][k] = float_to_ordered(-1e34f);
        }
        sh.u.bins.entry[threadIdx.x] = 0;
        sh.u.bins.exit[threadIdx.x] = 0;
      }
      __syncthreads();
      for (uint32_t i = begin + threadIdx.x; i < fi; i += kSbThreads) {
        const SbRef ref = sb_load(r0 + i);
        const SbBox box = sb_ref_box(ref);
        const uint32_t first = (uint32_t)min(15ull, sb_f2usize(rs_max(inv_size * (box.mn[ax] - mn), 0.0f)));
        const uint32_t last = (uint32_t)min(15ull, sb_f2usize(rs_max(inv_size * (box.mx[ax] - mn), 0.0f)));
        if (first > last) {  // bins[first..last] panics
          atomicOr(&sh.fail, kSbPanic);
          continue;
        }
        SbBox cur = box;
        const float* tri = A.tris + 9 * (size_t)sb_prim(ref);
        for (uint32_t j = 0; j < last - first; ++j) {
          SbBox lb, rb;
          sb_tri_split(tri, ax, mn + (float)(j + first + 1) * bin_size, fix_clip, lb, rb);
          sb_shrink(lb, cur);
          sb_bin_grow(sh, first + j, lb);
          sb_shrink(cur, rb);
        }
        sb_bin_grow(sh, last, cur);
        atomicAdd(&sh.u.bins.entry[first], 1u);
        atomicAdd(&sh.u.bins.exit[(A.fixes & kFixExitBin) ? last : first], 1u);
      }
      __syncthreads();
      if (threadIdx.x < 32) {
        // the 15-boundary sweep of :557-576 with one bin per lane: suffix
        // unions (the reference overwrites the bins with them), the left
        // boxes as unions of bins or of suffixes 0..i, counts as prefix
        // sums, then the first strict minimum below the incoming cost
        const int l = threadIdx.x;
        const bool in = l < kSbBins;
        const SbBox bin = in ? sb_bin_box(sh, l) : sb_empty();
        SbBox suf = bin;
#pragma unroll
        for (int o = 1; o < kSbBins; o <<= 1) {
          SbBox y;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            y.mn[k] = __shfl_down_sync(0xffffffffu, suf.mn[k], o);
            y.mx[k] = __shfl_down_sync(0xffffffffu, suf.mx[k], o);
          }
          if (l + o < kSbBins) sb_grow(suf, y);
        }
        SbBox lb = (A.fixes & kFixSweepBox) ? bin : suf;
        uint32_t ent = in ? sh.u.bins.entry[l] : 0u, ext = in ? sh.u.bins.exit[l] : 0u;
#pragma unroll
        for (int o = 1; o < kSbBins; o <<= 1) {
          SbBox y;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            y.mn[k] = __shfl_up_sync(0xffffffffu, lb.mn[k], o);
            y.mx[k] = __shfl_up_sync(0xffffffffu, lb.mx[k], o);
          }
          const uint32_t ye = __shfl_up_sync(0xffffffffu, ent, o), yx = __shfl_up_sync(0xffffffffu, ext, o);
          if (l >= o) {
            sb_grow(lb, y);
            ent += ye;
            ext += yx;
          }
        }
        SbBox rbox;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          rbox.mn[k] = __shfl_down_sync(0xffffffffu, suf.mn[k], 1);
          rbox.mx[k] = __shfl_down_sync(0xffffffffu, suf.mx[k], 1);
        }
        const float incoming = sh.sp_cost;
        float cost = FLT_MAX;
        bool ok = false;
        if (l < kSbBins - 1) {
          cost = (float)ent * sb_half_area(lb) + (float)((end - begin) - ext) * sb_half_area(rbox);
          ok = cost < incoming;
        }
        float bc = ok ? cost : FLT_MAX;
        int bl = ok ? l : 64;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float c2 = __shfl_xor_sync(0xffffffffu, bc, o);
          const int l2 = __shfl_xor_sync(0xffffffffu, bl, o);
          if (l2 < 64 && (bl == 64 || c2 < bc || (c2 == bc && l2 < bl))) {
            bc = c2;
            bl = l2;
          }
        }
        if (l == 0) {
          const uint32_t found = bl < 64 ? 1u : 0u;
          if (found) {
            sh.sp_cost = bc;
            sh.sp_axis = ax;
            sh.sp_pos = mn + (float)(bl + 1) * bin_size;
            sh.pass_lo = sh.sp_pos - bin_size;
            sh.pass_hi = sh.sp_pos + bin_size;
          }
          sh.found = found;
        }
      }
      __syncthreads();
      if (!sh.found) break;
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ tasks
__device__ __forceinline__ SbTask sb_load_task(const SbTask* p) {
  SbTask t;
  const uint4 a = __ldcg(reinterpret_cast<const uint4*>(p));
  t.begin = a.x;
  t.end = a.y;
  t.split_end = a.z;
  t.meta = a.w;
  t.lo = __ldcg(&p->lo);
  t.hi = __ldcg(&p->hi);
  return t;
}

__device__ __forceinline__ SbTask sb_make_task(uint32_t begin, uint32_t end, uint32_t split_end, uint32_t depth,
                                               bool sorted, const SbBox& b, uint32_t parent) {
  SbTask t;
  t.begin = begin;
  t.end = end;
  t.split_end = split_end;
  t.meta = depth | (sorted ? 1u << 8 : 0u);
  t.lo = make_float4(b.mn[0], b.mn[1], b.mn[2], __uint_as_float(parent));
  t.hi = make_float4(b.mx[0], b.mx[1], b.mx[2], 0.0f);
  return t;
}

// Stops the build: records the reason and makes waiting blocks leave.
__device__ __forceinline__ void sb_abort(const SbArgs& A, uint32_t t, uint32_t why) {
  if (threadIdx.x == 0) {
    A.child[t] = kSbNone;
    atomicOr(&A.ctl->status, why | kSbAbort);
  }
}

// allocate_children (:370-438) for references [begin, rb) (left) and
// [rb, re) (right), absolute positions; queues both children.
__device__ void sb_allocate_children(const SbArgs& A, SbShared& sh, uint32_t t, uint32_t rb, uint32_t re,
                                     const SbBox& left_box, const SbBox& right_box, bool sorted) {
  const uint32_t begin = sh.begin, split_end = sh.split_end;
  if (threadIdx.x == 0) {
    const uint32_t remaining = split_end - re;
    const float left_cost = sb_half_area(left_box) * (float)(rb - begin);
    const float right_cost = sb_half_area(right_box) * (float)(re - rb);
    const unsigned long long lsc =
        remaining == 0 ? 0ull : sb_f2usize((float)remaining * (left_cost / (left_cost + right_cost)));
    if (lsc > 0 && (unsigned long long)re + lsc > A.max_ref) sh.fail |= kSbPanic;  // move_backward out of bounds
    sh.lsc = (uint32_t)min(lsc, 0xffffffffull);
  }
  __syncthreads();
  if (sh.fail) {
    sb_abort(A, t, sh.fail);
    return;
  }
  const uint32_t lsc = sh.lsc;
  if (lsc > 0) {  // move_backward of the right references by lsc, all three arrays
    for (int ax = 0; ax < 3; ++ax) {
      sb_copy(A.scr, A.refs[ax], rb, re);
      __syncthreads();
      for (uint32_t i = rb + threadIdx.x; i < re; i += kSbThreads) sb_store(A.refs[ax] + i + lsc, sb_load(A.scr + i));
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    const bool fix = A.fixes & kFixSplitSpace;
    const SbTask l = sb_make_task(begin, rb, fix ? rb + lsc : rb, sh.depth + 1, sorted, left_box, t);
    const SbTask r = fix ? sb_make_task(rb + lsc, re + lsc, split_end, sh.depth + 1, sorted, right_box, t)
                         : sb_make_task(rb, re, split_end, sh.depth + 1, sorted, right_box, t);
    const uint32_t c = atomicAdd(&A.ctl->tail, 2u);
    if (c + 1 >= A.task_cap) {  // AtomicNodeStack::allocate returns None
      A.child[t] = kSbNone;
      atomicOr(&A.ctl->status, kSbPanic | kSbAbort);
    } else {
      A.tasks[c] = l;
      A.tasks[c + 1] = r;
      A.child[t] = c;
      __threadfence();
      atomicExch(A.ready + c, 1u);
      atomicExch(A.ready + c + 1, 1u);
    }
  }
  __syncthreads();
}

__device__ __forceinline__ uint32_t sb_hash(uint32_t p, uint32_t m) { return (uint32_t)((p * 2654435761u) % m); }

// apply_object_split (:440-489): reference_marks by primitive over the
// split axis (set for [begin, s), cleared for [s, end), last write wins;
// absent primitives unmarked), then a stable partition of the other two
// arrays, marked first. The marks live in a task-local hash table.
__device__ void sb_apply_object(const SbArgs& A, SbShared& sh, uint32_t t, int ax, uint32_t s, const SbBox& lb,
                                const SbBox& rbx) {
  const uint32_t begin = sh.begin, end = sh.end, n = end - begin, m = 2 * n;
  uint32_t* hk = A.hkeys + 2 * (size_t)begin;
  uint32_t* hv = A.hvals + 2 * (size_t)begin;
  for (uint32_t k = threadIdx.x; k < m; k += kSbThreads) {
    hk[k] = 0u;
    hv[k] = 1u;
  }
  __syncthreads();
  for (uint32_t i = begin + threadIdx.x; i < end; i += kSbThreads) {
    const uint32_t key = sb_prim(sb_load(A.refs[ax] + i)) + 1u;
    uint32_t h = sb_hash(key, m);
    for (uint32_t probe = 0; probe < m; ++probe) {
      const uint32_t cur = atomicCAS(hk + h, 0u, key);
      if (cur == 0u || cur == key) {
        atomicAnd(hv + h, i < s ? 1u : 0u);
        break;
      }
      h = h + 1 == m ? 0 : h + 1;
    }
  }
  __syncthreads();
  for (int o = 1; o <= 2; ++o) {
    SbRef* arr = A.refs[(ax + o) % 3];
    uint32_t local = 0;
    for (uint32_t i = begin + threadIdx.x; i < end; i += kSbThreads) {
      const uint32_t key = sb_prim(sb_load(arr + i)) + 1u;
      uint32_t h = sb_hash(key, m), mark = 0;
      for (uint32_t probe = 0; probe < m; ++probe) {
        const uint32_t cur = __ldcg(hk + h);
        if (cur == key) {
          mark = __ldcg(hv + h);
          break;
        }
        if (cur == 0u) break;
        h = h + 1 == m ? 0 : h + 1;
      }
      A.cls[i] = (uint8_t)mark;
      local += mark;
    }
    const uint32_t marked = sb_block_sum(sh, local);
    uint32_t before_t = 0, before_f = 0;
    for (uint32_t lo = begin; lo < end; lo += kSbThreads) {
      const uint32_t i = lo + threadIdx.x;
      const bool act = i < end;
      const uint32_t f = act ? (uint32_t)__ldcg(A.cls + i) : 0u;
      uint32_t tot;
      const uint32_t ex = sb_block_exscan(sh, f, &tot);
      if (act) {
        const uint32_t dest = f ? begin + before_t + ex : begin + marked + before_f + (threadIdx.x - ex);
        sb_store(A.scr + dest, sb_load(arr + i));
      }
      before_t += tot;
      before_f += min((uint32_t)kSbThreads, end - lo) - tot;
    }
    __syncthreads();
    sb_copy(arr, A.scr, begin, end);
    __syncthreads();
  }
  sb_allocate_children(A, sh, t, s, end, lb, rbx, true);
}

__device__ __forceinline__ uint32_t sb_cls_at(const SbShared& sh, uint32_t k) {
  return (sh.cls2[k >> 4] >> ((k & 15u) * 2u)) & 3u;
}

// Class bytes in global memory read through windows of 8 loaded at once
// (the replay walks them forwards from the front and backwards from the
// back), for tasks whose classes do not fit the shared words.
struct SbWin {
  unsigned long long bits;
  uint32_t base;
  bool valid;
};
__device__ __forceinline__ uint32_t sb_cls_fwd(const uint8_t* C, uint32_t n, SbWin& w, uint32_t k) {
  if (!w.valid || k < w.base || k >= w.base + 8) {
    w.base = k;
    w.valid = true;
    unsigned long long v = 0;
#pragma unroll
    for (uint32_t t = 0; t < 8; ++t)
      if (k + t < n) v |= (unsigned long long)__ldcg(C + k + t) << (8 * t);
    w.bits = v;
  }
  return (uint32_t)(w.bits >> (8 * (k - w.base))) & 0xffu;
}
__device__ __forceinline__ uint32_t sb_cls_bwd(const uint8_t* C, SbWin& w, uint32_t k) {
  if (!w.valid || k < w.base || k >= w.base + 8) {
    w.base = k >= 7 ? k - 7 : 0;
    w.valid = true;
    unsigned long long v = 0;
#pragma unroll
    for (uint32_t t = 0; t < 8; ++t)
      if (w.base + t <= k) v |= (unsigned long long)__ldcg(C + w.base + t) << (8 * t);
    w.bits = v;
  }
  return (uint32_t)(w.bits >> (8 * (k - w.base))) & 0xffu;
}
// Bits 0..15 of x to the even bit positions.
__device__ __forceinline__ uint32_t sb_spread16(uint32_t x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

constexpr uint32_t kSbRing = kSbTile * 2;  // straddler queue in the sort tile (u32 entries)

// The reference's partition loops (:622-702) replayed by thread 0 without
// moving references, writing the final order into P (slot | kind):
//  * the swap loop takes the front reference; a right one goes to the next
//    slot from the back and the reference there is taken next, a left one to
//    the next slot from the front, where the straddler it displaces moves
//    behind the others -- so left references keep their processing order,
//    right ones fill the back in processing order, and the straddlers form a
//    queue that every left reference processed after the first straddler
//    rotates by one;
//  * the fallback and the straddler loop then walk that queue from both
//    ends the same way.
// The queue (m <= kSbRing straddlers) lives in shared memory, the classes
// too (2 bits each) when `packed`, else they are read from C through
// windows. Returns false where the reference panics.
__device__ bool sb_replay_ring(const SbArgs& A, SbShared& sh, uint32_t n, uint32_t m, bool packed) {
  const uint32_t begin = sh.begin;
  uint32_t* P = A.perm + begin;
  const uint8_t* C = A.cls + begin;
  uint32_t* ring = reinterpret_cast<uint32_t*>(sh.u.tile);
  constexpr uint32_t mask = kSbRing - 1;
  uint32_t i = 0, j = 0, le = 0, rc = 0, qh = 0, qt = 0;
  SbWin fw{0ull, 0u, false}, bw{0ull, 0u, false};
  while (i + j < n) {
    uint32_t src = i, c = packed ? sb_cls_at(sh, i) : sb_cls_fwd(C, n, fw, i);
    bool done = false;
    while (c == kClsRight) {
      P[n - 1 - rc] = src;
      ++rc;
      ++j;
      if (i + j >= n) {
        done = true;
        break;
      }
      src = n - j;
      c = packed ? sb_cls_at(sh, src) : sb_cls_bwd(C, bw, src);
    }
    if (done) break;
    if (c == kClsLeft) {
      P[le++] = src;
      if (qt != qh) {
        ring[qt & mask] = ring[qh & mask];
        ++qt;
        ++qh;
      }
    } else {
      ring[qt & mask] = src;
      ++qt;
    }
    ++i;
  }
  uint32_t lc = le, rcnt = rc;
  if ((lc == 0 || rcnt == 0) && m == 0) {  // equal-count fallback (:643-658)
    if (lc > 0) {
      if (A.fixes & kFixFallback) le = lc / 2;
      else if (lc / 2 < begin) return false;  // left_end = left_count / 2 drops the begin: the slice panics
      else le = lc / 2 - begin;
    } else {
      le += rcnt / 2;
    }
    sh.le = le;
    sh.rb = le;
    sh.re = n;
    return true;
  }
  const uint32_t space = sh.split_end - begin;
  uint32_t re = n, a = 0, bp = m;
  uint32_t cur = m ? ring[qh & mask] : 0u;
  while (a < bp) {
    if (space - re > 0) {
      P[le + a] = cur | kKindLeftFrag;
      P[re++] = cur | kKindRightFrag;
      ++a;
      ++lc;
      ++rcnt;
      if (a < bp) cur = ring[(qh + a) & mask];
    } else if (lc < rcnt) {
      P[le + a] = cur;
      ++a;
      ++lc;
      if (a < bp) cur = ring[(qh + a) & mask];
    } else {
      --bp;
      P[le + bp] = cur;
      ++rcnt;
      if (a < bp) cur = ring[(qh + bp) & mask];
    }
  }
  sh.le = le + a;
  sh.rb = le + bp;
  sh.re = re;
  return true;
}

// The same replay with the references moved in P itself (any number of
// straddlers; one dependent global access per step).
__device__ bool sb_replay_global(const SbArgs& A, SbShared& sh, uint32_t n) {
  const uint32_t begin = sh.begin;
  uint32_t* P = A.perm + begin;
  const uint8_t* C = A.cls + begin;
  uint32_t i = 0, le = 0, rb = n, re = n;
  while (i < rb) {
    const uint32_t e = __ldcg(P + i);
    const uint8_t c = __ldcg(C + e);
    if (c == kClsLeft) {
      P[i] = __ldcg(P + le);
      P[le] = e;
      ++i;
      ++le;
    } else if (c == kClsRight) {
      --rb;
      P[i] = __ldcg(P + rb);
      P[rb] = e;
    } else {
      ++i;
    }
  }
  uint32_t lc = le, rc = re - rb;
  if ((lc == 0 || rc == 0) && le == rb) {
    if (lc > 0) {
      if (A.fixes & kFixFallback) le = lc / 2;
      else if (lc / 2 < begin) return false;
      else le = lc / 2 - begin;
    } else {
      le += rc / 2;
    }
    rb = le;
  }
  const uint32_t space = sh.split_end - begin;
  while (le < rb) {
    const uint32_t e = __ldcg(P + le);
    if (space - re > 0) {
      P[re] = e | kKindRightFrag;
      P[le] = e | kKindLeftFrag;
      ++re;
      ++le;
      ++lc;
      ++rc;
    } else if (lc < rc) {
      ++le;
      ++lc;
    } else {
      --rb;
      P[le] = __ldcg(P + rb);
      P[rb] = e;
      ++rc;
    }
  }
  sh.le = le;
  sh.rb = rb;
  sh.re = re;
  return true;
}

// apply_spatial_split (:605-724). The classes are computed in parallel, the
// partition is replayed by thread 0 into a permutation of slots, then every
// thread builds the new reference order (fragments clipped from the
// triangle) and all three arrays receive it.
__device__ void sb_apply_spatial(const SbArgs& A, SbShared& sh, uint32_t t) {
  const uint32_t begin = sh.begin, end = sh.end, n = end - begin;
  const int ax = (int)sh.sp_axis;
  const float pos = sh.sp_pos;
  SbRef* S = A.refs[ax];
  uint32_t* P = A.perm + begin;
  uint8_t* C = A.cls + begin;
  // classes: one reference per thread (coalesced); up to kSbClsCap
  // references they are packed 2 bits each into shared memory by warp
  // ballots, beyond that (and for the global replay) bytes in C
  uint32_t straddlers = 0;
  const bool packed = n <= kSbClsCap;
  for (uint32_t kb = 0; kb < n; kb += kSbThreads) {
    const uint32_t k = kb + threadIdx.x;
    uint32_t c = 0;
    if (k < n) {
      const SbBox b = sb_ref_box(sb_load(S + begin + k));
      c = b.mx[ax] <= pos ? kClsLeft : (b.mn[ax] >= pos ? kClsRight : kClsStraddle);
      C[k] = (uint8_t)c;
      straddlers += c == kClsStraddle;
    }
    if (packed) {
      const uint32_t b0 = __ballot_sync(0xffffffffu, c & 1u), b1 = __ballot_sync(0xffffffffu, c >> 1);
      const uint32_t w0 = (kb + (threadIdx.x & ~31u)) >> 4;
      if ((threadIdx.x & 31) == 0 && w0 < kSbClsWords) {
        sh.cls2[w0] = sb_spread16(b0) | (sb_spread16(b1) << 1);
        if (w0 + 1 < kSbClsWords) sh.cls2[w0 + 1] = sb_spread16(b0 >> 16) | (sb_spread16(b1 >> 16) << 1);
      }
    }
  }
  const uint32_t m = sb_block_sum(sh, straddlers);
  const bool ring = m <= kSbRing;
  if (!ring)
    for (uint32_t k = threadIdx.x; k < n; k += kSbThreads) P[k] = k;
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool ok = ring ? sb_replay_ring(A, sh, n, m, packed) : sb_replay_global(A, sh, n);
    if (!ok) sh.fail |= kSbPanic;
  }
  __syncthreads();
  if (sh.fail) {
    sb_abort(A, t, sh.fail);
    return;
  }
  const uint32_t le = sh.le, rb = sh.rb, re = sh.re;
  for (uint32_t k = threadIdx.x; k < re; k += kSbThreads) {
    const uint32_t e = __ldcg(P + k);
    const SbRef r = sb_load(S + begin + (e & kSlotMask));
    const uint32_t kind = e & ~kSlotMask;
    sb_store(A.scr + begin + k, kind == 0 ? r : sb_fragment(A, r, ax, pos, kind == kKindRightFrag));
  }
  __syncthreads();
  const SbBox lb = sb_block_union(sh, A.scr, begin, begin + le);
  const SbBox rbx = sb_block_union(sh, A.scr, begin + rb, begin + re);
  for (int o = 0; o < 3; ++o) sb_copy(A.refs[o], A.scr, begin, begin + re);
  __syncthreads();
  sb_allocate_children(A, sh, t, begin + rb, begin + re, lb, rbx, false);
}

// Task::run (:726-838) for queued task t.
__device__ void sb_run_task(const SbArgs& A, SbShared& sh, uint32_t t) {
  if (threadIdx.x == 0) {
    const SbTask task = sb_load_task(A.tasks + t);
    sh.begin = task.begin;
    sh.end = task.end;
    sh.split_end = task.split_end;
    sh.depth = task.meta & 0xffu;
    sh.sorted = (task.meta >> 8) & 1u;
    sh.nb[0] = task.lo.x; sh.nb[1] = task.lo.y; sh.nb[2] = task.lo.z;
    sh.nb[3] = task.hi.x; sh.nb[4] = task.hi.y; sh.nb[5] = task.hi.z;
    sh.fail = 0;
  }
  __syncthreads();
  const uint32_t begin = sh.begin, end = sh.end, split_end = sh.split_end, n = end - begin;
  if (n <= 1 || sh.depth >= kSbMaxDepth) {  // make_leaf
    if (threadIdx.x == 0) A.child[t] = kSbNone;
    return;
  }
  if (!sh.sorted)
    for (int ax = 0; ax < 3; ++ax) sb_sort_axis(A, sh, ax, begin, n);
  sb_object_sweep(A, sh, begin, end);
  SbBox ol = sb_empty(), orr = sb_empty();
  if (sh.obj_index != kSbNone) {
    ol = sb_block_union(sh, A.refs[sh.obj_axis], begin, sh.obj_index);
    orr = sb_block_union(sh, A.refs[sh.obj_axis], sh.obj_index, end);
  }
  SbBox ov = ol;
  sb_shrink(ov, orr);
  if (sb_area(ov) > __ldcg(&A.ctl->threshold) && split_end - end > 0) {
    sb_spatial_search(A, sh, begin, end);
  } else if (threadIdx.x == 0) {
    sh.sp_cost = FLT_MAX;
  }
  __syncthreads();
  if (sh.fail) {
    sb_abort(A, t, sh.fail);
    return;
  }
  SbBox nb;
  for (int k = 0; k < 3; ++k) { nb.mn[k] = sh.nb[k]; nb.mx[k] = sh.nb[3 + k]; }
  if (threadIdx.x == 0) {
    const float best = rs_min(sh.sp_cost, sh.obj_cost);
    const bool use_spatial = best < sh.obj_cost;
    const float max_split_cost = sb_half_area(nb) * ((float)n - kSbTraversalCost);
    uint32_t mode;  // 0 leaf, 1 object split, 2 spatial split, 3 median object split
    if (best >= max_split_cost) mode = n > A.max_leaf ? 3u : 0u;
    else mode = use_spatial ? 2u : (sh.obj_index != kSbNone ? 1u : 0u);
    sh.use_spatial = mode;
  }
  __syncthreads();
  const uint32_t mode = sh.use_spatial;
  if (mode == 0) {
    if (threadIdx.x == 0) A.child[t] = kSbNone;
  } else if (mode == 2) {
    sb_apply_spatial(A, sh, t);
  } else if (mode == 1) {
    sb_apply_object(A, sh, t, (int)sh.obj_axis, sh.obj_index, ol, orr);
  } else {
    // median split on the longest axis of the node (:773-788)
    const int ax = sb_longest_axis(nb);
    const uint32_t mid = (begin + end) / 2;
    const SbBox ml = sb_block_union(sh, A.refs[ax], begin, mid);
    const SbBox mr = sb_block_union(sh, A.refs[ax], mid, end);
    sb_apply_object(A, sh, t, ax, mid, ml, mr);
  }
}

// Persistent build kernel: blocks take tasks in queue order until every
// queued task has finished. Waits are bounded (kSbSpin polls).
__global__ void __launch_bounds__(kSbThreads) k_sb_build(SbArgs A) {
  __shared__ SbShared sh;
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t idx = atomicAdd(&A.ctl->head, 1u);
      uint32_t take = kSbNone;
      for (uint32_t it = 0;; ++it) {
        const uint32_t status = *(volatile uint32_t*)&A.ctl->status;
        if (status & kSbAbort) break;
        const uint32_t done = *(volatile uint32_t*)&A.ctl->done;
        __threadfence();
        const uint32_t tail = *(volatile uint32_t*)&A.ctl->tail;
        if (idx < tail && idx < A.task_cap && *(volatile uint32_t*)(A.ready + idx)) {
          take = idx;
          break;
        }
        // every queued task has finished, so no task can be queued any more
        if (done == tail && idx >= tail) break;
        if (it > kSbSpin) {
          atomicOr(&A.ctl->status, kStatusTimeout | kSbAbort);
          break;
        }
        __nanosleep(1024);
      }
      sh.task = take;
    }
    __syncthreads();
    const uint32_t t = sh.task;
    if (t == kSbNone) return;
    __threadfence();
    sb_run_task(A, sh, t);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&A.ctl->done, 1u);
    }
  }
}

// Initial references (build, :948-1002) and the root task.
__global__ void k_sb_init(SbArgs A, const DAabb* aabbs, const DAabb* world) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.max_ref) {
    SbRef r;
    if (i < A.n) {
      const DAabb a = load_aabb(aabbs + i);
      r.lo = make_float4(a.min[0], a.min[1], a.min[2], __uint_as_float(i));
      r.hi = make_float4(a.max[0], a.max[1], a.max[2], 0.0f);
    } else {  // SpatialReference::default: the empty box, centre 0, prim 0
      r.lo = make_float4(1e34f, 1e34f, 1e34f, __uint_as_float(kSbFrag));
      r.hi = make_float4(-1e34f, -1e34f, -1e34f, 0.0f);
    }
    for (int ax = 0; ax < 3; ++ax) sb_store(A.refs[ax] + i, r);
  }
  if (i < A.task_cap) A.ready[i] = 0u;
  if (i == 0) {
    const DAabb w = load_aabb(world);
    SbBox b;
    for (int k = 0; k < 3; ++k) { b.mn[k] = w.min[k]; b.mx[k] = w.max[k]; }
    A.tasks[0] = sb_make_task(0, A.n, A.max_ref, 0, false, b, kSbNone);
    A.ready[0] = 1u;
    A.ctl->head = 0;
    A.ctl->tail = 1;
    A.ctl->done = 0;
    A.ctl->status = 0;
    A.ctl->threshold = kSbAlpha * 2.0f * sb_half_area(b);
  }
}

// The root's find_object_split sort (:316-331) for one axis, before the
// build: keys are the order-preserving centre bits (-0 as +0), values the
// reference index; a stable LSD radix sort of (key, index) in index order
// gives the stable order on the centre.
__global__ void k_sb_root_keys(const float4* __restrict__ centers, uint32_t n, int ax, uint32_t* keys,
                               uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 c4 = __ldg(centers + i);
  float c = sb_axis(c4.x, c4.y, c4.z, ax);
  if (c == 0.0f) c = 0.0f;
  keys[i] = float_to_ordered(c);
  vals[i] = i;
}
__global__ void k_sb_root_gather(const DAabb* __restrict__ aabbs, const uint32_t* __restrict__ order, uint32_t n,
                                 SbRef* refs) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = order[k];
  const DAabb a = load_aabb(aabbs + i);
  SbRef r;
  r.lo = make_float4(a.min[0], a.min[1], a.min[2], __uint_as_float(i));
  r.hi = make_float4(a.max[0], a.max[1], a.max[2], 0.0f);
  sb_store(refs + k, r);
}
__global__ void k_sb_root_sorted(SbTask* tasks) { tasks[0].meta |= 1u << 8; }

// ------------------------------------------------------------------ numbering
struct SbNumArgs {
  const SbTask* tasks;
  const uint32_t* child;
  const SbCtl* ctl;
  uint32_t* arrive;
  uint32_t* ic;  // interior nodes in the subtree
  uint32_t* lr;  // leaf references in the subtree
  uint32_t* ib;  // interior nodes before the task in the single-thread order
  uint32_t* lb;  // leaf references before the task in that order
};

__device__ __forceinline__ uint32_t sb_parent(const SbTask* tasks, uint32_t t) {
  return __float_as_uint(__ldcg(&tasks[t].lo.w));
}
__device__ __forceinline__ uint32_t sb_work(const SbTask* tasks, uint32_t t) {
  const uint2 be = __ldcg(reinterpret_cast<const uint2*>(tasks + t));
  return be.y - be.x;
}

// Subtree sizes, bottom up: the second child to arrive at a parent fills it.
__global__ void k_sb_counts(SbNumArgs a) {
  const uint32_t total = __ldcg(&a.ctl->tail);
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= total || __ldcg(a.child + v) != kSbNone) return;
  a.ic[v] = 0;
  a.lr[v] = sb_work(a.tasks, v);
  __threadfence();
  uint32_t c = v;
  for (;;) {
    const uint32_t p = sb_parent(a.tasks, c);
    if (p == kSbNone) break;
    if (atomicAdd(a.arrive + p, 1u) == 0u) break;
    __threadfence();
    const uint32_t l = __ldcg(a.child + p);
    a.ic[p] = 1u + __ldcg(a.ic + l) + __ldcg(a.ic + l + 1);
    a.lr[p] = __ldcg(a.lr + l) + __ldcg(a.lr + l + 1);
    __threadfence();
    c = p;
  }
}

// Position of every task in TaskSpawner::run_task's single-thread order
// (src/utils.rs:246-283): the child with more references is popped first
// (the left one on a tie), its whole subtree before its sibling's.
__global__ void k_sb_ranks(SbNumArgs a) {
  const uint32_t total = __ldcg(&a.ctl->tail);
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= total) return;
  uint32_t ib = 0, lb = 0, c = v;
  for (;;) {
    const uint32_t p = sb_parent(a.tasks, c);
    if (p == kSbNone) break;
    const uint32_t l = __ldcg(a.child + p);
    const uint32_t first = sb_work(a.tasks, l) < sb_work(a.tasks, l + 1) ? l + 1 : l;
    ib += 1;
    if (c != first) {
      ib += __ldcg(a.ic + first);
      lb += __ldcg(a.lr + first);
    }
    c = p;
  }
  a.ib[v] = ib;
  a.lb[v] = lb;
}

// Writes the reference's node array and prim_indices: interior node k of
// the order gets children 1 + 2k (allocate, :375) and its box offset by
// 1e-4 (:382); leaves write their references' primitives at their range.
__global__ void k_sb_write(SbNumArgs a, const SbRef* refs0, DAabb* nodes, uint32_t* indices) {
  const uint32_t total = __ldcg(&a.ctl->tail);
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= total) return;
  const SbTask t = sb_load_task(a.tasks + v);
  uint32_t node = 0;
  const uint32_t p = __float_as_uint(t.lo.w);
  if (p != kSbNone) node = 1u + 2u * __ldcg(a.ib + p) + (__ldcg(a.child + p) == v ? 0u : 1u);
  DAabb out;
  out.min[0] = t.lo.x; out.min[1] = t.lo.y; out.min[2] = t.lo.z;
  out.max[0] = t.hi.x; out.max[1] = t.hi.y; out.max[2] = t.hi.z;
  if (__ldcg(a.child + v) != kSbNone) {
    for (int k = 0; k < 3; ++k) {
      out.min[k] = out.min[k] - 0.0001f;
      out.max[k] = out.max[k] + 0.0001f;
    }
    out.count = -1;
    out.left_first = (int32_t)(1u + 2u * __ldcg(a.ib + v));
  } else {
    const uint32_t count = t.end - t.begin, first = __ldcg(a.lb + v);
    out.count = (int32_t)count;
    out.left_first = (int32_t)first;
    for (uint32_t k = 0; k < count; ++k) indices[first + k] = sb_prim(sb_load(refs0 + t.begin + k));
  }
  store_aabb(nodes + node, out);
}

}  // namespace

// SpatialSahBuilder::build (:926-1034): max_reference_count =
// n + (n as f32 * split_factor) as usize.
uint64_t spatial_max_refs(size_t n) {
  const float f = (float)n * kSbSplitFactor;
  return (uint64_t)n + (f > 0.0f ? (uint64_t)f : 0ull);
}

ResultCode build_spatial_sah(const DAabb* aabbs, const float4* centers, const float* tris, size_t n,
                             size_t prims_per_leaf, uint32_t fixes, cudaStream_t s, BuildOutput* out,
                             uint32_t* index_count) {
  if (n == 0) return NoPrimitives;
  const uint64_t mr = spatial_max_refs(n);
  if (mr >= (uint64_t)kSlotMask / 2) return InvalidArgument;  // slots, task ids and 2x hash ranges fit 30 bits
  const uint32_t max_ref = (uint32_t)mr, task_cap = 2 * max_ref + 1;
  Scratch<SbRef> r0, r1, r2, scr;
  Scratch<unsigned long long> k0, k1;
  Scratch<float> fbuf;
  Scratch<uint32_t> perm, hk, hv, ready, child, arrive, ic, lr, ib, lb, acc6, rstat;
  Scratch<uint8_t> cls;
  Scratch<SbTask> tasks;
  Scratch<SbCtl> ctl;
  Scratch<DAabb> world;
  cudaError_t e;
  if ((e = r0.alloc(max_ref, s)) || (e = r1.alloc(max_ref, s)) || (e = r2.alloc(max_ref, s)) ||
      (e = scr.alloc(max_ref, s)) || (e = k0.alloc(max_ref, s)) || (e = k1.alloc(max_ref, s)) ||
      (e = fbuf.alloc(max_ref, s)) || (e = perm.alloc(max_ref, s)) || (e = cls.alloc(max_ref, s)) ||
      (e = hk.alloc(2 * (size_t)max_ref, s)) || (e = hv.alloc(2 * (size_t)max_ref, s)) ||
      (e = tasks.alloc(task_cap, s)) || (e = ready.alloc(task_cap, s)) || (e = child.alloc(task_cap, s)) ||
      (e = arrive.alloc(task_cap, s)) || (e = ic.alloc(task_cap, s)) || (e = lr.alloc(task_cap, s)) ||
      (e = ib.alloc(task_cap, s)) || (e = lb.alloc(task_cap, s)) || (e = ctl.alloc(1, s)) ||
      (e = world.alloc(1, s)) || (e = acc6.alloc(6, s)) || (e = rstat.alloc(1, s)) ||
      (e = cudaMemsetAsync(rstat.ptr, 0, 4, s)))
    return cuda_rc(e);
  if ((e = launch_world_bounds(aabbs, n, world.ptr, acc6.ptr, s))) return cuda_rc(e);
  SbArgs A;
  A.refs[0] = r0.ptr;
  A.refs[1] = r1.ptr;
  A.refs[2] = r2.ptr;
  A.scr = scr.ptr;
  A.keys = k0.ptr;
  A.keys2 = k1.ptr;
  A.fbuf = fbuf.ptr;
  A.perm = perm.ptr;
  A.cls = cls.ptr;
  A.hkeys = hk.ptr;
  A.hvals = hv.ptr;
  A.tasks = tasks.ptr;
  A.ready = ready.ptr;
  A.child = child.ptr;
  A.ctl = ctl.ptr;
  A.tris = tris;
  A.centers = centers;
  A.n = (uint32_t)n;
  A.max_ref = max_ref;
  A.task_cap = task_cap;
  A.max_leaf = prims_per_leaf == 0 ? 1u : (uint32_t)std::min<size_t>(prims_per_leaf, 0xffffffffu);
  A.fixes = fixes;
  k_sb_init<<<(task_cap + 255) / 256, 256, 0, s>>>(A, aabbs, world.ptr);
  if (n > 1) {  // the root's three sorts, device wide
    Scratch<uint32_t> rk, rv;
    Scratch<uint8_t> temp;
    const size_t tb = radix_sort_temp_bytes(n);
    if ((e = rk.alloc(n, s)) || (e = rv.alloc(n, s)) || (e = temp.alloc(tb, s))) return cuda_rc(e);
    const unsigned g = (unsigned)((n + 255) / 256);
    for (int ax = 0; ax < 3; ++ax) {
      k_sb_root_keys<<<g, 256, 0, s>>>(centers, (uint32_t)n, ax, rk.ptr, rv.ptr);
      if ((e = radix_sort_pairs(rk.ptr, rv.ptr, n, 32, temp.ptr, tb, rstat.ptr, s))) return cuda_rc(e);
      k_sb_root_gather<<<g, 256, 0, s>>>(aabbs, rv.ptr, (uint32_t)n, A.refs[ax]);
    }
    k_sb_root_sorted<<<1, 1, 0, s>>>(tasks.ptr);
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sb_build, kSbThreads, 0);
  k_sb_build<<<sm_count() * std::max(per_sm, 1), kSbThreads, 0, s>>>(A);
  if ((e = cudaGetLastError())) return cuda_rc(e);
  SbCtl h;
  uint32_t sort_status = 0;
  if ((e = cudaMemcpyAsync(&h, ctl.ptr, sizeof(SbCtl), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(&sort_status, rstat.ptr, 4, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
    return cuda_rc(e);
  if ((h.status | sort_status) & kStatusTimeout) return Timeout;
  if (h.status & kSbAbort) return Error;  // the reference panics on this input
  SbNumArgs na{tasks.ptr, child.ptr, ctl.ptr, arrive.ptr, ic.ptr, lr.ptr, ib.ptr, lb.ptr};
  const unsigned grid = (h.tail + 255) / 256;
  if ((e = cudaMemsetAsync(arrive.ptr, 0, (size_t)h.tail * 4, s))) return cuda_rc(e);
  k_sb_counts<<<grid, 256, 0, s>>>(na);
  uint32_t root[2];
  if ((e = cudaMemcpyAsync(root, ic.ptr, 4, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(root + 1, lr.ptr, 4, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
    return cuda_rc(e);
  if (root[1] > max_ref) return Error;  // make_leaf would write past prim_indices
  const uint32_t node_count = 1 + 2 * root[0];
  DAabb* nodes = nullptr;
  uint32_t* indices = nullptr;
  if ((e = device_alloc(&nodes, node_count, s)) || (e = device_alloc(&indices, max_ref, s)) ||
      (e = cudaMemsetAsync(indices, 0, (size_t)max_ref * 4, s))) {
    pool_free(nodes, s);
    pool_free(indices, s);
    return cuda_rc(e);
  }
  k_sb_ranks<<<grid, 256, 0, s>>>(na);
  k_sb_write<<<grid, 256, 0, s>>>(na, r0.ptr, nodes, indices);
  if ((e = cudaGetLastError())) {
    pool_free(nodes, s);
    pool_free(indices, s);
    return cuda_rc(e);
  }
  out->nodes = nodes;
  out->indices = indices;
  out->node_count = node_count;
  *index_count = max_ref;
  return Ok;
}

}  // namespace rtbvh
