// Single-ray traversal with the fused triangle test, one ray per thread.
//
// trace_mbvh follows MbvhIndexIterator::next (src/iter_indices.rs:264-313)
// step for step: the quad node's hit mask and slot order come from the
// 4-wide slab test (src/mbvh_node.rs:176-240) evaluated with the ray's
// current t when the node is entered; slots are visited far to near
// (ids[3..0]); a leaf slot's primitives are tested at once, an interior slot
// is pushed. The triangle test is SpatialTriangle::intersect
// (src/builders/spatial_sah.rs:132-163). With the same arithmetic (no FMA,
// IEEE division, SSE min/max rules) the hits, their order of discovery and
// the node/triangle counts equal the reference's.
//
// trace_bvh follows BvhIndexIterator::next (src/iter_indices.rs:66-107) with
// the sign-indexed slab test (src/aabb.rs:145-181) and sort_nodes
// (src/bvh_node.rs:150-177).
//
// Kernels are persistent. The stack lives in local memory with a hard bound;
// a ray that would exceed it stops, reports prim -2 and sets
// kStatusStackOverflow. A quad node (one 128-byte line) is read with four
// 256-bit loads (each lane reads its own node, so the load count per node
// sets the L1 wavefronts). Leaf triangles are 64 bytes ({v0, prim}, {e1},
// {e2}, pad): two 256-bit loads.
//
// Closest hit without statistics reads the 64-byte compact copies of the
// quad nodes (DQNode, two 256-bit loads) when they exist: the boxes contain
// the exact ones, so the nearest triangle and its t/u/v are unchanged, and
// only the winner among triangles hit at exactly the same t can differ from
// the reference's visit order. This halves the node bytes and the L1 fill
// traffic. Any hit, statistics and rays with a zero, non-finite or huge
// component use the exact nodes.
#include <cstdlib>

#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 128;
constexpr int kStack = 64;

struct RayState {
  float ox, oy, oz, dx, dy, dz, ix, iy, iz;
  float t;
  int32_t sx, sy, sz;
};

__device__ __forceinline__ RayState load_ray(const float* rays, size_t r, const float* t_max) {
  const float2* p = reinterpret_cast<const float2*>(rays + 6 * r);
  float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  RayState s;
  s.ox = a.x; s.oy = a.y; s.oz = b.x;
  s.dx = b.y; s.dy = c.x; s.dz = c.y;
  s.ix = 1.0f / s.dx; s.iy = 1.0f / s.dy; s.iz = 1.0f / s.dz;
  s.sx = s.dx < 0.0f; s.sy = s.dy < 0.0f; s.sz = s.dz < 0.0f;
  s.t = t_max ? __ldg(t_max + r) : 1e34f;
  return s;
}

// One 256-bit read-only load (sm_100+): 8 floats from a 32-byte aligned address.
__device__ __forceinline__ void ld8(const float* p, float (&v)[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}

// SpatialTriangle::intersect with a leaf-ordered triangle {v0,prim},{e1},{e2}.
__device__ __forceinline__ bool mt_test(const float4* tri, RayState& r, float& hu, float& hv, int32_t& prim) {
  float t0[8], t1[8];
  ld8(reinterpret_cast<const float*>(tri), t0);
  ld8(reinterpret_cast<const float*>(tri) + 8, t1);
  const float4 a = make_float4(t0[0], t0[1], t0[2], t0[3]), b = make_float4(t0[4], t0[5], t0[6], t0[7]);
  const float4 c = make_float4(t1[0], t1[1], t1[2], t1[3]);
  const float e1x = b.x, e1y = b.y, e1z = b.z;
  const float e2x = c.x, e2y = c.y, e2z = c.z;
  // h = d x e2
  const float hx = r.dy * e2z - e2y * r.dz;
  const float hy = r.dz * e2x - e2z * r.dx;
  const float hz = r.dx * e2y - e2x * r.dy;
  const float det = ((e1x * hx) + (e1y * hy)) + (e1z * hz);
  if (det > -1e-5f && det < 1e-5f) return false;
  const float f = 1.0f / det;
  const float sx = r.ox - a.x, sy = r.oy - a.y, sz = r.oz - a.z;
  const float u = f * (((sx * hx) + (sy * hy)) + (sz * hz));
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  // q = s x e1
  const float qx = sy * e1z - e1y * sz;
  const float qy = sz * e1x - e1z * sx;
  const float qz = sx * e1y - e1x * sy;
  const float v = f * (((r.dx * qx) + (r.dy * qy)) + (r.dz * qz));
  if (v < 0.0f || (u + v) > 1.0f) return false;
  const float t = f * (((e2x * qx) + (e2y * qy)) + (e2z * qz));
  if (t > 1e-4f && t < r.t) {
    r.t = t;
    hu = u;
    hv = v;
    prim = __float_as_int(a.w);
    return true;
  }
  return false;
}

// MbvhNode::intersect: mask bit i set when slot i is hit; ids packed as
// 2-bit fields, ascending by t_min after the 5-compare network.
//
// FAST: for a ray whose origin, direction and inverse direction are all
// finite, no slab value can be NaN ((m - o) * inv with finite factors), and
// then the SSE select rule (a < b ? a : b) and the native min/max instruction
// return the same value; at most the sign of a zero differs, which no later
// comparison can see. So the fast form takes every decision the exact form
// takes. Rays with a zero or non-finite component use the exact form.
template <bool FAST>
__device__ __forceinline__ void quad_intersect(const DMNode* node, const RayState& r, uint32_t& mask, uint32_t& ids,
                                               int4& children, int4& counts) {
  const float* q = reinterpret_cast<const float*>(node);
  float vx[8], vy[8], vz[8], vc[8];
  ld8(q, vx);
  ld8(q + 8, vy);
  ld8(q + 16, vz);
  ld8(q + 24, vc);
  const float4 mnx = make_float4(vx[0], vx[1], vx[2], vx[3]), mxx = make_float4(vx[4], vx[5], vx[6], vx[7]);
  const float4 mny = make_float4(vy[0], vy[1], vy[2], vy[3]), mxy = make_float4(vy[4], vy[5], vy[6], vy[7]);
  const float4 mnz = make_float4(vz[0], vz[1], vz[2], vz[3]), mxz = make_float4(vz[4], vz[5], vz[6], vz[7]);
  const float4 ch = make_float4(vc[0], vc[1], vc[2], vc[3]), ct = make_float4(vc[4], vc[5], vc[6], vc[7]);
  children = make_int4(__float_as_int(ch.x), __float_as_int(ch.y), __float_as_int(ch.z), __float_as_int(ch.w));
  counts = make_int4(__float_as_int(ct.x), __float_as_int(ct.y), __float_as_int(ct.z), __float_as_int(ct.w));
  float tmin[4];
  uint32_t m = 0;
  const float a_mnx[4] = {mnx.x, mnx.y, mnx.z, mnx.w}, a_mxx[4] = {mxx.x, mxx.y, mxx.z, mxx.w};
  const float a_mny[4] = {mny.x, mny.y, mny.z, mny.w}, a_mxy[4] = {mxy.x, mxy.y, mxy.z, mxy.w};
  const float a_mnz[4] = {mnz.x, mnz.y, mnz.z, mnz.w}, a_mxz[4] = {mxz.x, mxz.y, mxz.z, mxz.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float tx0 = (a_mnx[i] - r.ox) * r.ix, tx1 = (a_mxx[i] - r.ox) * r.ix;
    const float ty0 = (a_mny[i] - r.oy) * r.iy, ty1 = (a_mxy[i] - r.oy) * r.iy;
    const float tz0 = (a_mnz[i] - r.oz) * r.iz, tz1 = (a_mxz[i] - r.oz) * r.iz;
    float tn, tx;
    if (FAST) {
      tn = fmaxf(fminf(tx0, tx1), fmaxf(fminf(ty0, ty1), fminf(tz0, tz1)));
      tx = fminf(fmaxf(tx0, tx1), fminf(fmaxf(ty0, ty1), fmaxf(tz0, tz1)));
    } else {
      const float txn = sse_min(tx0, tx1), txx = sse_max(tx0, tx1);
      const float tyn = sse_min(ty0, ty1), tyx = sse_max(ty0, ty1);
      const float tzn = sse_min(tz0, tz1), tzx = sse_max(tz0, tz1);
      tn = sse_max(txn, sse_max(tyn, tzn));
      tx = sse_min(txx, sse_min(tyx, tzx));
    }
    tmin[i] = tn;
    if ((tx >= tn) && (tn < r.t)) m |= 1u << i;
  }
  uint32_t i0 = 0, i1 = 1, i2 = 2, i3 = 3;
  float t0 = tmin[0], t1 = tmin[1], t2 = tmin[2], t3 = tmin[3], tt;
  uint32_t ti;
  if (t0 > t1) { tt = t0; t0 = t1; t1 = tt; ti = i0; i0 = i1; i1 = ti; }
  if (t2 > t3) { tt = t2; t2 = t3; t3 = tt; ti = i2; i2 = i3; i3 = ti; }
  if (t0 > t2) { tt = t0; t0 = t2; t2 = tt; ti = i0; i0 = i2; i2 = ti; }
  if (t1 > t3) { tt = t1; t1 = t3; t3 = tt; ti = i1; i1 = i3; i3 = ti; }
  if (t2 > t3) { ti = i2; i2 = i3; i3 = ti; }
  mask = m;
  ids = i0 | (i1 << 2) | (i2 << 4) | (i3 << 6);
}

// Slot bound i of a DQNode axis word as a float (exact): 2^23 + q is
// assembled in the float's mantissa, then 2^23 is subtracted.
__device__ __forceinline__ float qbyte(uint32_t w, uint32_t i) {
  return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7440u + i)) - 8388608.0f;
}

__device__ __forceinline__ bool finite_ray(const RayState& r) {
  return isfinite(r.ox) && isfinite(r.oy) && isfinite(r.oz) && isfinite(r.dx) && isfinite(r.dy) && isfinite(r.dz) &&
         isfinite(r.ix) && isfinite(r.iy) && isfinite(r.iz);
}

__device__ __forceinline__ int sel4(const int4& v, uint32_t i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Per-lane ray refill shared by the persistent MBVH kernels: a lane whose ray
// has finished takes the next ray from a warp-local pool (refilled `batch`
// rays at a time from the global counter), so the warp's lanes stay busy
// instead of idling until the warp's slowest ray ends.
// Default rays per pool refill (TraceArgs::ray_batch). Small batches keep the
// end of a launch short (the last warps hold few rays); measured on one GB300
// against 128: the 1M incoherent scene +0.9 %, the 6,400-triangle sphere's
// camera +20 %, the 200k-triangle camera -4 % time (64, 16: less on one or
// the other; 256, 512: slower everywhere).
constexpr uint32_t kPoolBatch = 32;

struct WarpPool {
  uint32_t next = 0, end = 0;  // warp-uniform (ray counts < 2^32 - 2^25)
  bool exhausted = false;      // warp-uniform
  // Calls start(k) on every lane that is not active, for the next unclaimed
  // ray positions k; start decides whether the lane becomes active. A single
  // idle lane waits for a second one (unless no lane is active), so that the
  // ray set-up, which only the refilled lanes execute, runs for two or more
  // lanes at a time.
  template <class Start>
  __device__ __forceinline__ void refill(bool active, uint32_t batch, uint32_t ray_count, unsigned int* work,
                                         Start&& start) {
    const int lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t need = __ballot_sync(0xffffffffu, !active);
    if (!need || (__popc(need) < 2 && need != 0xffffffffu)) return;
    // first from what is left in the pool ...
    const uint32_t avail = end - next;
    if (avail) {
      const uint32_t rank = __popc(need & lt_mask);
      const bool mine = (need >> lane) & 1u;
      if (mine && rank < avail) start(next + rank);
      const uint32_t c = __popc(need);
      next += c < avail ? c : avail;
      need = __ballot_sync(0xffffffffu, mine && rank >= avail);
    }
    // ... then from a fresh batch of the global counter
    if (need) {
      unsigned int base = 0;
      if (lane == 0) base = atomicAdd(work, batch);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= ray_count) {
        exhausted = true;
      } else {
        next = base;
        end = (ray_count - base > batch) ? base + batch : ray_count;
        const uint32_t avail2 = end - next;
        const bool mine = (need >> lane) & 1u;
        const uint32_t rank = __popc(need & lt_mask);
        if (mine && rank < avail2) start(next + rank);
        const uint32_t c = __popc(need);
        next += c < avail2 ? c : avail2;
      }
    }
  }
};

// Mesh of ray r in a forest: m with seg_ray_off[m] <= r < seg_ray_off[m + 1].
__device__ __forceinline__ uint32_t ray_mesh(const TraceArgs& a, uint32_t r) {
  uint32_t lo = 0, hi = a.seg_count;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a.seg_ray_off + mid) <= r) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Hit mask of a quad node's subtree boxes (DTBox): slot i is set when the
// ray can enter its box at some t in [0, r.t). Finite rays within the
// compact walk's range only (the rounding argument of kCompactRange: a box
// that holds a triangle hit at t > 1e-4 passes).
__device__ __forceinline__ uint32_t subtree_mask(const DTBox* box, const RayState& r) {
  const float* q = reinterpret_cast<const float*>(box);
  float vx[8], vy[8], vz[8];
  ld8(q, vx);
  ld8(q + 8, vy);
  ld8(q + 16, vz);
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float tx0 = (vx[i] - r.ox) * r.ix, tx1 = (vx[4 + i] - r.ox) * r.ix;
    const float ty0 = (vy[i] - r.oy) * r.iy, ty1 = (vy[4 + i] - r.oy) * r.iy;
    const float tz0 = (vz[i] - r.oz) * r.iz, tz1 = (vz[4 + i] - r.oz) * r.iz;
    const float tn = fmaxf(fminf(tx0, tx1), fmaxf(fminf(ty0, ty1), fminf(tz0, tz1)));
    const float tx = fminf(fmaxf(tx0, tx1), fminf(fmaxf(ty0, ty1), fmaxf(tz0, tz1)));
    if (tx >= tn && tx >= 0.0f && tn < r.t) m |= 1u << i;
  }
  return m;
}

// Persistent MBVH traversal over the exact quad nodes with per-lane ray
// refill. Each loop iteration visits one quad node per lane; a ray's
// node/triangle order is the reference's. With ray_count_dev the number of
// rays is read from the device (the rays the compact kernel deferred).
//
// TCULL (closest hit over a binned-SAH tree's quad nodes with a.tboxes):
// a slot whose subtree box (from the triangles) the ray cannot enter below
// its current t is skipped. The reference would walk that subtree and
// accept no hit in it (every triangle lies inside the subtree box), so t
// and the order of all later tests are unchanged: the hit is the
// reference's bit for bit (the node counts are not, so STATS never culls).
template <bool ANY_HIT, bool STATS, bool TCULL = false>
__global__ void __launch_bounds__(kBlock) k_trace_mbvh(TraceArgs a, unsigned int* work) {
  RayState ray;
  float hu = 0.0f, hv = 0.0f;
  int32_t prim = -1;
  uint32_t visits = 0, tests = 0, max_depth = 0;
  // The node to visit next is kept in `next` instead of on the stack: the
  // last child a node pushes is always the next one popped, so holding it in
  // a register saves one store and one load per visited node. The logical
  // stack is stack[0..sp] followed by `next` (when next >= 0).
  int32_t stack[kStack];
  int sp = -1;
  int32_t next = -1;
  uint32_t r = 0;
  bool active = false, fast = true, cull = false;
  WarpPool pool;
  uint32_t batch = a.ray_batch ? a.ray_batch : kPoolBatch;
  const uint32_t ray_count = a.ray_count_dev ? *a.ray_count_dev : (uint32_t)a.ray_count;
  if (a.ray_count_dev) {
    // few rays (deferred by the compact walk): spread them over all warps,
    // down to one ray per refill, so that their walks run side by side
    const uint32_t warps = gridDim.x * (kBlock / 32u), even = ray_count / warps;
    batch = even < 1u ? 1u : (even < batch ? even : batch);
  }
  auto start_ray = [&](uint32_t rr) {
    r = a.order ? __ldg(a.order + rr) : rr;
    ray = load_ray(a.rays, r, a.t_max);
    fast = finite_ray(ray);
    if (TCULL && a.node_count > 0) {
      // |x| <= bound is false for NaN and infinities. Only rays that start
      // inside the scene's root box: boxes behind them are most of what the
      // cull saves; for rays from outside it costs more than it saves
      const DAabb root = load_aabb(a.nodes);
      cull = fabsf(ray.ox) <= kCompactRange && fabsf(ray.oy) <= kCompactRange && fabsf(ray.oz) <= kCompactRange &&
             fabsf(ray.dx) <= 3.0e38f && fabsf(ray.dy) <= 3.0e38f && fabsf(ray.dz) <= 3.0e38f &&
             fabsf(ray.ix) <= kQuantRange && fabsf(ray.iy) <= kQuantRange && fabsf(ray.iz) <= kQuantRange &&
             ray.ox >= root.min[0] && ray.oy >= root.min[1] && ray.oz >= root.min[2] && ray.ox <= root.max[0] &&
             ray.oy <= root.max[1] && ray.oz <= root.max[2];
    }
    hu = hv = 0.0f;
    prim = -1;
    visits = tests = max_depth = 0;
    if (a.node_count == 0) {
      a.hits[r] = make_float4(ray.t, 0.0f, 0.0f, __int_as_float(-1));
      if (STATS) {
        a.stats[3 * (size_t)r + 0] = 0;
        a.stats[3 * (size_t)r + 1] = 0;
        a.stats[3 * (size_t)r + 2] = 0;
      }
    } else {
      sp = -1;
      next = 0;
      active = true;
      if (a.seg_count) {
        const uint32_t m = ray_mesh(a, r);
        const uint32_t root = __ldg(a.seg_root + m);
        if (root == __ldg(a.seg_root + m + 1)) {
          active = false;
          a.hits[r] = make_float4(ray.t, 0.0f, 0.0f, __int_as_float(-1));
          if (STATS) {
            a.stats[3 * (size_t)r + 0] = 0;
            a.stats[3 * (size_t)r + 1] = 0;
            a.stats[3 * (size_t)r + 2] = 0;
          }
        }
        next = (int32_t)root;
      }
    }
  };
  for (;;) {
    if (!pool.exhausted) pool.refill(active, batch, ray_count, work, start_ray);
    if (!__any_sync(0xffffffffu, active)) {
      if (pool.exhausted) break;
      continue;
    }
    if (!active) continue;
    // ---- one quad node
    const int32_t current = next >= 0 ? next : stack[sp--];
    next = -1;
    if ((uint32_t)current >= a.node_count) {
      atomicOr(a.status, kStatusBadIndex);
      active = false;
      continue;
    }
    uint32_t mask, ids;
    int4 children, counts;
    bool done = false;
    if (fast) quad_intersect<true>(a.mnodes + current, ray, mask, ids, children, counts);
    else quad_intersect<false>(a.mnodes + current, ray, mask, ids, children, counts);
    if (TCULL && cull) mask &= subtree_mask(a.tboxes + current, ray);
    if (STATS) ++visits;
#pragma unroll 1
    for (int i = 0; i < 4; ++i) {
      const uint32_t id = (ids >> (2 * (3 - i))) & 3u;
      if (!((mask >> id) & 1u)) continue;
      const int32_t count = sel4(counts, id);
      const int32_t lf = sel4(children, id);
      if (count > -1) {
        if (lf < 0 || (uint32_t)lf + (uint32_t)count > a.prim_count) {
          atomicOr(a.status, kStatusBadIndex);
          done = true;
          break;
        }
        bool hit_stop = false;
        for (int32_t j = 0; j < count; ++j) {
          if (STATS) ++tests;
          if (mt_test(a.tris + kTriFloat4 * (size_t)(lf + j), ray, hu, hv, prim) && ANY_HIT) {
            hit_stop = true;
            break;
          }
        }
        if (hit_stop) {
          done = true;
          break;
        }
      } else if (lf > -1) {
        if (next >= 0) {
          if (sp + 1 >= kStack) {
            atomicOr(a.status, kStatusStackOverflow);
            prim = -2;
            done = true;
            break;
          }
          stack[++sp] = next;
        }
        next = lf;
        if (STATS && (uint32_t)(sp + 2) > max_depth) max_depth = (uint32_t)(sp + 2);
      }
    }
    if (done || (next < 0 && sp < 0)) {
      a.hits[r] = make_float4(ray.t, hu, hv, __int_as_float(prim));
      if (STATS) {
        a.stats[3 * (size_t)r + 0] = visits;
        a.stats[3 * (size_t)r + 1] = tests;
        a.stats[3 * (size_t)r + 2] = max_depth;
      }
      active = false;
    }
  }
}

// Interior slots of a traversal-tree node in near-to-far order. key[i] is
// the entry t of the i-th nearest interior slot the ray hits; other slots
// (missed, empty, or leaves) get +inf and sort last. Each key's child
// travels with it through the sorting network, so the caller reads children
// by position without run-time indexing. A hit slot's key is finite: it is
// below the ray's t (no NaN arises on the compact path's finite rays).
__device__ __forceinline__ void sort_slots(float (&key)[4], int32_t (&ch)[4]) {
  auto cswap = [&](int a, int b) {
    const bool s = key[b] < key[a];
    const float ka = key[a], kb = key[b];
    const int32_t ca = ch[a], cb = ch[b];
    key[a] = s ? kb : ka;
    key[b] = s ? ka : kb;
    ch[a] = s ? cb : ca;
    ch[b] = s ? ca : cb;
  };
  cswap(0, 1);
  cswap(2, 3);
  cswap(0, 2);
  cswap(1, 3);
  cswap(1, 2);
}

// Key of slot i (interior slots only) and its bit in the leaf mask.
//
// A slot whose box lies wholly behind the origin (exit t below 0) is
// skipped as well, which the reference's test does not do: every box of a
// traversal tree contains its triangles grown by 1e-4, so a triangle hit at
// t > 1e-4 (the triangle test's lower bound) lies inside its boxes with that
// margin, and the box's computed exit t stays above 0 (the slab rounding is
// below the margin, see kCompactRange). The cull removes no box that holds
// a hit; it saves the walks of rays that start inside the scene (secondary
// rays) through the boxes behind them.
__device__ __forceinline__ void slot_key(float tn, float tx, float t, int32_t child, int32_t count, int i,
                                         float& key, uint32_t& leaves) {
  const bool hit = tx >= tn && tx >= 0.0f && tn < t && child >= 0;
  key = (hit && count < 0) ? tn : __int_as_float(0x7f800000);
  leaves |= (hit && count >= 0) ? 1u << i : 0u;
}

// The slab test of quad_intersect<true> on a compact node: the plane of step
// q is at lo + q * step, so its ray parameter is q * (step * inv) +
// (lo - o) * inv (one fma). With a negative inverse direction the upper
// plane is the near one; the fma is monotonic in q, so selecting the planes
// by sign equals min/max of the two. Outputs: the sorted interior keys and
// children, the hit leaf slots as a mask over the node's own slot order, and
// the node's children and counts in that order.
__device__ __forceinline__ void slot_keys_q(const float (&h0)[8], const float (&h1)[8], const RayState& r,
                                            float (&key)[4], int32_t (&ich)[4], uint32_t& leaves,
                                            int32_t (&ch)[4], int32_t (&ct)[4]) {
  const uint32_t exps = __float_as_uint(h0[3]);
  const float sx = __uint_as_float((exps & 0xffu) << 23);
  const float sy = __uint_as_float(((exps >> 8) & 0xffu) << 23);
  const float sz = __uint_as_float(((exps >> 16) & 0xffu) << 23);
  const float ax = sx * r.ix, bx = (h0[0] - r.ox) * r.ix;
  const float ay = sy * r.iy, by = (h0[1] - r.oy) * r.iy;
  const float az = sz * r.iz, bz = (h0[2] - r.oz) * r.iz;
  const uint32_t xl = __float_as_uint(h0[4]), xh = __float_as_uint(h0[5]);
  const uint32_t yl = __float_as_uint(h0[6]), yh = __float_as_uint(h0[7]);
  const uint32_t zl = __float_as_uint(h1[0]), zh = __float_as_uint(h1[1]);
  const uint32_t xn = r.ix < 0.0f ? xh : xl, xf = r.ix < 0.0f ? xl : xh;
  const uint32_t yn = r.iy < 0.0f ? yh : yl, yf = r.iy < 0.0f ? yl : yh;
  const uint32_t zn = r.iz < 0.0f ? zh : zl, zf = r.iz < 0.0f ? zl : zh;
  const uint32_t c01 = __float_as_uint(h1[6]), c23 = __float_as_uint(h1[7]);
  ch[0] = __float_as_int(h1[2]);
  ch[1] = __float_as_int(h1[3]);
  ch[2] = __float_as_int(h1[4]);
  ch[3] = __float_as_int(h1[5]);
  ct[0] = (int32_t)(int16_t)(c01 & 0xffffu);
  ct[1] = (int32_t)(int16_t)(c01 >> 16);
  ct[2] = (int32_t)(int16_t)(c23 & 0xffffu);
  ct[3] = (int32_t)(int16_t)(c23 >> 16);
  leaves = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float tn = fmaxf(fmaf(qbyte(xn, i), ax, bx), fmaxf(fmaf(qbyte(yn, i), ay, by), fmaf(qbyte(zn, i), az, bz)));
    const float tx = fminf(fmaf(qbyte(xf, i), ax, bx), fminf(fmaf(qbyte(yf, i), ay, by), fmaf(qbyte(zf, i), az, bz)));
    slot_key(tn, tx, r.t, ch[i], ct[i], i, key[i], leaves);
    ich[i] = ch[i];
  }
  sort_slots(key, ich);
}

// The same from a node's exact (128-byte) copy, for compact nodes whose
// bounds did not fit the grid; FAST arithmetic (finite rays only).
__device__ __forceinline__ void slot_keys_exact(const DMNode* node, const RayState& r, float (&key)[4],
                                                int32_t (&ich)[4], uint32_t& leaves, int32_t (&ch)[4],
                                                int32_t (&ct)[4]) {
  const float* q = reinterpret_cast<const float*>(node);
  float vx[8], vy[8], vz[8], vc[8];
  ld8(q, vx);
  ld8(q + 8, vy);
  ld8(q + 16, vz);
  ld8(q + 24, vc);
  leaves = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    ch[i] = __float_as_int(vc[i]);
    ct[i] = __float_as_int(vc[4 + i]);
    const float tx0 = (vx[i] - r.ox) * r.ix, tx1 = (vx[4 + i] - r.ox) * r.ix;
    const float ty0 = (vy[i] - r.oy) * r.iy, ty1 = (vy[4 + i] - r.oy) * r.iy;
    const float tz0 = (vz[i] - r.oz) * r.iz, tz1 = (vz[4 + i] - r.oz) * r.iz;
    const float tn = fmaxf(fminf(tx0, tx1), fmaxf(fminf(ty0, ty1), fminf(tz0, tz1)));
    const float tx = fminf(fmaxf(tx0, tx1), fminf(fmaxf(ty0, ty1), fmaxf(tz0, tz1)));
    slot_key(tn, tx, r.t, ch[i], ct[i], i, key[i], leaves);
    ich[i] = ch[i];
  }
  sort_slots(key, ich);
}

// Closest hit over the compact (64-byte) nodes of the traversal tree, with
// the leaf tests taken out of the slot loop. A loop iteration has a node
// phase -- each lane with no untested leaf visits its next node, pushes the
// node's hit interior slots far to near (the nearest stays in `next`) and
// notes its hit leaf slots -- and a triangle phase -- each lane with noted
// leaves tests one of them. The lanes of a warp meet again before the
// triangle phase, so the warp runs it once per iteration for all of its
// lanes. A lane visits no node while it has untested leaves, so every node
// is entered with the t the reference-order loop would have after the
// previous node's leaves; only the order among one node's leaves (slot
// order here) differs, which can change the winner among triangles hit at
// exactly the same t.
//
// Rays the compact walk does not take -- a zero or non-finite component, an
// inverse direction beyond kQuantRange, an origin beyond kCompactRange, a
// node flagged out of range on the way or (GATES) a hit on a triangle
// flagged kTriEscape, see build_mbvh -- are appended to `deferred`
// and traced afterwards by k_trace_mbvh over the exact Mbvh.
// Nine resident blocks per SM (56 registers, 36 warps; a few bytes of
// spills): measured 4 % faster than the 64-register, 32-warp form.
//
// WSTATS: per-ray counts of this walk in a.walk_stats (traversal-tree node
// visits, triangle tests, 1 if the ray was handed to the exact walk).
template <int STACK, bool GATES, bool WSTATS>
__global__ void __launch_bounds__(kBlock, 9) k_trace_compact(TraceArgs a, unsigned int* work, uint32_t* deferred,
                                                           unsigned int* deferred_count) {
  RayState ray;
  float hu = 0.0f, hv = 0.0f;
  int32_t prim = -1;
  uint32_t w_visits = 0, w_tests = 0;
  int32_t stack[STACK];
  int sp = -1;
  int32_t next = -1;
  // the last visited node's hit leaf slots not yet tested, as bits of their
  // slots in lch / lct (first primitive slot, count)
  uint32_t pend = 0;
  int32_t lch[4] = {0, 0, 0, 0}, lct[4] = {0, 0, 0, 0};
  uint32_t r = 0;
  bool active = false;
  WarpPool pool;
  const uint32_t batch = a.ray_batch ? a.ray_batch : kPoolBatch;
  const uint32_t ray_count = (uint32_t)a.ray_count;
  auto write_stats = [&](uint32_t handed_on) {
    if (WSTATS) {
      a.walk_stats[3 * (size_t)r + 0] = w_visits;
      a.walk_stats[3 * (size_t)r + 1] = w_tests;
      a.walk_stats[3 * (size_t)r + 2] = handed_on;
    }
  };
  auto finish = [&]() {
    a.hits[r] = make_float4(ray.t, hu, hv, __int_as_float(prim));
    write_stats(0u);
    active = false;
  };
  auto defer = [&]() {
    deferred[atomicAdd(deferred_count, 1u)] = r;
    write_stats(1u);
    active = false;
  };
  auto start_ray = [&](uint32_t rr) {
    r = a.order ? __ldg(a.order + rr) : rr;
    ray = load_ray(a.rays, r, a.t_max);
    hu = hv = 0.0f;
    prim = -1;
    sp = -1;
    pend = 0;
    next = 0;
    w_visits = w_tests = 0;
    if (a.node_count == 0) {
      finish();
      return;
    }
    if (a.seg_count) {
      const uint32_t m = ray_mesh(a, r);
      if (__ldg(a.seg_root + m) == __ldg(a.seg_root + m + 1)) {
        finish();  // a mesh without nodes: a miss
        return;
      }
      next = (int32_t)__ldg(a.seg_qroot + m);
    }
    // |x| <= bound is false for NaN and infinities
    const bool ok = fabsf(ray.ox) <= kCompactRange && fabsf(ray.oy) <= kCompactRange &&
                    fabsf(ray.oz) <= kCompactRange && fabsf(ray.dx) <= 3.0e38f && fabsf(ray.dy) <= 3.0e38f &&
                    fabsf(ray.dz) <= 3.0e38f && fabsf(ray.ix) <= kQuantRange && fabsf(ray.iy) <= kQuantRange &&
                    fabsf(ray.iz) <= kQuantRange;
    if (!ok) {
      defer();
      return;
    }
    active = true;
  };
  for (;;) {
    if (!pool.exhausted) pool.refill(active, batch, ray_count, work, start_ray);
    const uint32_t amask = __ballot_sync(0xffffffffu, active);
    if (!amask) {
      if (pool.exhausted) break;
      continue;
    }
    if (!active) continue;
    // ---- node phase (no early exits: the lanes of amask meet below)
    if (pend == 0) {
      const int32_t current = next >= 0 ? next : stack[sp--];
      next = -1;
      if ((uint32_t)current >= a.q_count) {
        atomicOr(a.status, kStatusBadIndex);
        active = false;
      } else {
        const float* qn = reinterpret_cast<const float*>(a.qnodes + current);
        float h0[8], h1[8];
        ld8(qn, h0);
        ld8(qn + 8, h1);
        if (WSTATS) ++w_visits;
        const uint32_t flags = __float_as_uint(h0[3]) >> 24;
        if (flags & kQFlagOutOfRange) {
          defer();
        } else {
          float key[4];
          int32_t ich[4];
          if (!flags) slot_keys_q(h0, h1, ray, key, ich, pend, lch, lct);
          else slot_keys_exact(a.qexact + current, ray, key, ich, pend, lch, lct);
          bool overflow = false;
#pragma unroll
          for (int i = 3; i >= 0; --i) {  // far to near
            if (key[i] < __int_as_float(0x7f800000)) {
              if (next >= 0) {
                if (sp + 1 < STACK) stack[++sp] = next;
                else overflow = true;
              }
              next = ich[i];
            }
          }
          if (overflow) {
            atomicOr(a.status, kStatusStackOverflow);
            prim = -2;
            finish();
          }
        }
      }
    }
    __syncwarp(amask);
    // ---- triangle phase
    if (active && pend) {
      const uint32_t i = __ffs(pend) - 1;
      pend &= pend - 1u;
      const int32_t lf = i == 0 ? lch[0] : (i == 1 ? lch[1] : (i == 2 ? lch[2] : lch[3]));
      const int32_t count = i == 0 ? lct[0] : (i == 1 ? lct[1] : (i == 2 ? lct[2] : lct[3]));
      if (lf < 0 || (uint32_t)lf + (uint32_t)count > a.prim_count) {
        atomicOr(a.status, kStatusBadIndex);
        active = false;
      } else {
        for (int32_t j = 0; j < count; ++j) {
          const float4* tri = a.tris + kTriFloat4 * (size_t)(lf + j);
          if (WSTATS) ++w_tests;
          if (mt_test(tri, ray, hu, hv, prim) && GATES && (__float_as_uint(__ldg(&tri[1].w)) & kTriEscape)) {
            defer();  // an escaped triangle is hit: its hits are the exact walk's
            break;
          }
        }
      }
    }
    if (active && pend == 0 && next < 0 && sp < 0) finish();
  }
}

// Aabb::intersect (src/aabb.rs:145-181): far t or miss; t_min fixed at 1e-4.
__device__ __forceinline__ bool slab_far(const DAabb& b, const RayState& r, float& out) {
  float ray_min = ((r.sx ? b.max[0] : b.min[0]) - r.ox) * r.ix;
  float ray_max = ((r.sx ? b.min[0] : b.max[0]) - r.ox) * r.ix;
  const float y_min = ((r.sy ? b.max[1] : b.min[1]) - r.oy) * r.iy;
  const float y_max = ((r.sy ? b.min[1] : b.max[1]) - r.oy) * r.iy;
  if ((ray_min > y_max) || (y_min > ray_max)) return false;
  if (y_min > ray_min) ray_min = y_min;
  if (y_max < ray_max) ray_max = y_max;
  const float z_min = ((r.sz ? b.max[2] : b.min[2]) - r.oz) * r.iz;
  const float z_max = ((r.sz ? b.min[2] : b.max[2]) - r.oz) * r.iz;
  if ((ray_min > z_max) || (z_min > ray_max)) return false;
  if (z_max < ray_max) ray_max = z_max;
  if (ray_max > 1e-4f) {
    out = ray_max;
    return true;
  }
  return false;
}

// BvhIndexIterator::next (src/iter_indices.rs:66-107) for one ray: a step
// is one pop; a leaf's primitives are tested, an interior node's two
// children are tested with the far-t slab test (which never culls by t) and
// pushed in sort_nodes order. Stack entries hold the node's (left_first,
// count), read when its parent loaded both children (two 256-bit loads of
// the adjacent pair), so a pop needs no node load.
template <bool ANY_HIT, bool STATS>
__device__ __forceinline__ void trace_one_bvh(const TraceArgs& a, size_t r) {
  RayState ray = load_ray(a.rays, r, a.t_max);
  float hu = 0.0f, hv = 0.0f;
  int32_t prim = -1;
  uint32_t visits = 0, tests = 0, max_depth = 0;
  const bool nan = (ray.ox != ray.ox) || (ray.oy != ray.oy) || (ray.oz != ray.oz) || (ray.dx != ray.dx) ||
                   (ray.dy != ray.dy) || (ray.dz != ray.dz);
  int2 stack[kStack];
  int sp = -1;
  if (a.node_count > 0 && !nan) {
    const DAabb root = load_aabb(a.nodes);
    stack[0] = make_int2(root.left_first, root.count);
    sp = 0;
  }
  while (sp >= 0) {
    const int2 e = stack[sp--];
    const int32_t lf = e.x, count = e.y;
    if (count > -1) {
      if (lf < 0 || (uint32_t)lf + (uint32_t)count > a.prim_count) {
        atomicOr(a.status, kStatusBadIndex);
        break;
      }
      bool stop = false;
      for (int32_t j = 0; j < count; ++j) {
        if (STATS) ++tests;
        if (mt_test(a.tris + kTriFloat4 * (size_t)(lf + j), ray, hu, hv, prim) && ANY_HIT) {
          stop = true;
          break;
        }
      }
      if (stop) break;
    } else if (lf > -1) {
      if (STATS) ++visits;
      if ((uint32_t)lf + 1u >= a.node_count) {
        atomicOr(a.status, kStatusBadIndex);
        break;
      }
      float l8[8], r8[8];
      ld8(reinterpret_cast<const float*>(a.nodes + lf), l8);
      ld8(reinterpret_cast<const float*>(a.nodes + lf + 1), r8);
      DAabb lb, rb;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        lb.min[k] = l8[k];
        lb.max[k] = l8[4 + k];
        rb.min[k] = r8[k];
        rb.max[k] = r8[4 + k];
      }
      const int2 le = make_int2(__float_as_int(l8[7]), __float_as_int(l8[3]));
      const int2 re = make_int2(__float_as_int(r8[7]), __float_as_int(r8[3]));
      float lt = 0.0f, rt = 0.0f;
      const bool lh = slab_far(lb, ray, lt);
      const bool rh = slab_far(rb, ray, rt);
      if (sp + 2 >= kStack) {
        atomicOr(a.status, kStatusStackOverflow);
        prim = -2;
        break;
      }
      if (lh && rh) {
        if (lt < rt) { stack[++sp] = le; stack[++sp] = re; }
        else { stack[++sp] = re; stack[++sp] = le; }
      } else if (lh) {
        stack[++sp] = le;
      } else if (rh) {
        stack[++sp] = re;
      }
      if (STATS && (uint32_t)(sp + 1) > max_depth) max_depth = (uint32_t)(sp + 1);
    }
  }
  a.hits[r] = make_float4(ray.t, hu, hv, __int_as_float(prim));
  if (STATS) {
    a.stats[3 * (size_t)r + 0] = visits;
    a.stats[3 * (size_t)r + 1] = tests;
    a.stats[3 * (size_t)r + 2] = max_depth;
  }
}

// Warps take 32 consecutive rays at a time (adjacent camera rays walk the
// same nodes in step).
template <bool ANY_HIT, bool STATS>
__global__ void __launch_bounds__(kBlock) k_trace_bvh(TraceArgs a, unsigned int* work) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned int base = 0;
    if (lane == 0) base = atomicAdd(work, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((size_t)base >= a.ray_count) break;
    const size_t r = (size_t)base + lane;
    if (r < a.ray_count) trace_one_bvh<ANY_HIT, STATS>(a, r);
  }
}

// ------------------------------------------------------------------ candidate lists
// The primitives the reference's index iterators yield for a ray when the
// caller's callback leaves t unchanged: MbvhIndexIterator
// (src/iter_indices.rs:212-313) or BvhIndexIterator (:18-107) over the exact
// nodes, in yield order. This is the device form of intersect /
// intersect_mbvh with a user callback (rtbvh_ffi/src/lib.rs:551-581,
// 700-731) for primitives whose test the library does not know: the caller
// tests the listed primitives in its own kernel. One ray per thread.
template <bool MBVH>
__global__ void __launch_bounds__(kBlock) k_candidates(CandArgs a) {
  const size_t stride = (size_t)gridDim.x * kBlock;
  for (size_t r = (size_t)blockIdx.x * kBlock + threadIdx.x; r < a.ray_count; r += stride) {
    const RayState ray = load_ray(a.rays, r, a.t_max);
    uint32_t n = 0;
    bool bad = false;
    auto yield_range = [&](int32_t lf, int32_t count) {
      if (lf < 0 || (uint32_t)lf + (uint32_t)count > a.prim_count) {
        atomicOr(a.status, kStatusBadIndex);
        bad = true;
        return;
      }
      for (int32_t j = 0; j < count; ++j) {
        if (a.out && n < a.max_per_ray) a.out[r * a.max_per_ray + n] = __ldg(a.indices + lf + j);
        ++n;
      }
    };
    int32_t stack[kStack];
    int sp = -1;
    if (MBVH) {
      if (a.node_count > 0) {
        const bool fast = finite_ray(ray);
        int32_t current = 0;
        for (;;) {
          uint32_t mask, ids;
          int4 children, counts;
          if (fast) quad_intersect<true>(a.mnodes + current, ray, mask, ids, children, counts);
          else quad_intersect<false>(a.mnodes + current, ray, mask, ids, children, counts);
          for (int i = 0; i < 4 && !bad; ++i) {
            const uint32_t id = (ids >> (2 * (3 - i))) & 3u;
            if (!((mask >> id) & 1u)) continue;
            const int32_t count = sel4(counts, id), lf = sel4(children, id);
            if (count > -1) {
              yield_range(lf, count);
            } else if (lf > -1) {
              if (sp + 1 >= kStack) {
                atomicOr(a.status, kStatusStackOverflow);
                bad = true;
                break;
              }
              stack[++sp] = lf;
            }
          }
          if (bad || sp < 0) break;
          current = stack[sp--];
          if ((uint32_t)current >= a.node_count) {
            atomicOr(a.status, kStatusBadIndex);
            bad = true;
            break;
          }
        }
      }
    } else {
      const bool nan = (ray.ox != ray.ox) || (ray.oy != ray.oy) || (ray.oz != ray.oz) || (ray.dx != ray.dx) ||
                       (ray.dy != ray.dy) || (ray.dz != ray.dz);
      sp = (a.node_count == 0 || nan) ? -1 : 0;
      stack[0] = 0;
      while (sp >= 0 && !bad) {
        const int32_t ni = stack[sp--];
        if ((uint32_t)ni >= a.node_count) {
          atomicOr(a.status, kStatusBadIndex);
          bad = true;
          break;
        }
        const DAabb node = load_aabb(a.nodes + ni);
        if (node.count > -1) {
          yield_range(node.left_first, node.count);
        } else if (node.left_first > -1) {
          const int32_t lf = node.left_first;
          if ((uint32_t)lf + 1u >= a.node_count) {
            atomicOr(a.status, kStatusBadIndex);
            bad = true;
            break;
          }
          float lt = 0.0f, rt = 0.0f;
          const bool lh = slab_far(load_aabb(a.nodes + lf), ray, lt);
          const bool rh = slab_far(load_aabb(a.nodes + lf + 1), ray, rt);
          if (sp + 2 >= kStack) {
            atomicOr(a.status, kStatusStackOverflow);
            bad = true;
            break;
          }
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
    }
    a.counts[r] = bad ? 0xffffffffu : n;
  }
}

// ------------------------------------------------------------------ ray order
// Incoherent rays are traced in an order that groups rays with nearby
// origins and similar directions, so that the lanes of a warp walk similar
// nodes (fewer distinct cache lines per warp load, more L1 hits). Each ray's
// traversal is unchanged; only the assignment of rays to lanes differs, and
// hits are written to the ray's own slot.

__global__ void __launch_bounds__(256) k_ray_origin_bounds(const float* __restrict__ rays, size_t n,
                                                           uint32_t* __restrict__ acc) {
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2* p = reinterpret_cast<const float2*>(rays + 6 * i);
    const float2 a = __ldg(p), b = __ldg(p + 1);
    const float o[3] = {a.x, a.y, b.x};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (isfinite(o[k])) {
        mn[k] = fminf(mn[k], o[k]);
        mx[k] = fmaxf(mx[k], o[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      atomicMin(acc + k, float_to_ordered(mn[k]));
      atomicMax(acc + 3 + k, float_to_ordered(mx[k]));
    }
  }
}

__device__ __forceinline__ uint32_t spread3_bits(uint32_t v) {
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__device__ __forceinline__ uint32_t spread2_bits(uint32_t v) {
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
__device__ __forceinline__ uint32_t quant6(float x) {  // x in [0, 1]
  float q = x * 64.0f;
  return q >= 63.0f ? 63u : (q > 0.0f ? (uint32_t)q : 0u);
}

// key = Morton(origin cell, 6 bits per axis) << 12 | Morton(octahedral
// direction, 6 bits per coordinate)
__global__ void __launch_bounds__(256) k_ray_keys(const float* __restrict__ rays, size_t n,
                                                  const uint32_t* __restrict__ acc, uint32_t* __restrict__ keys,
                                                  uint32_t* __restrict__ vals) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float lo[3], inv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = ordered_to_float(__ldg(acc + k));
    const float ext = ordered_to_float(__ldg(acc + 3 + k)) - lo[k];
    inv[k] = ext > 0.0f ? 1.0f / ext : 0.0f;
  }
  const float2* p = reinterpret_cast<const float2*>(rays + 6 * i);
  const float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  const float o[3] = {a.x, a.y, b.x};
  const float d[3] = {b.y, c.x, c.y};
  uint32_t oc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) oc[k] = quant6((o[k] - lo[k]) * inv[k]);
  const float l1 = fabsf(d[0]) + fabsf(d[1]) + fabsf(d[2]);
  float u = 0.0f, v = 0.0f;
  if (l1 > 0.0f && isfinite(l1)) {
    u = d[0] / l1;
    v = d[1] / l1;
    if (d[2] < 0.0f) {
      const float uu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
      const float vv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
      u = uu;
      v = vv;
    }
  }
  const uint32_t du = quant6(u * 0.5f + 0.5f), dv = quant6(v * 0.5f + 0.5f);
  const uint32_t ko = spread3_bits(oc[0]) | (spread3_bits(oc[1]) << 1) | (spread3_bits(oc[2]) << 2);
  keys[i] = (ko << 12) | spread2_bits(du) | (spread2_bits(dv) << 1);
  vals[i] = (uint32_t)i;
}

// Persistent grid: resident blocks per SM (occupancy, capped by
// blocks_per_sm) on every SM, no more blocks than the rays need.
template <class K>
unsigned persistent_grid(K kern, const TraceArgs& a) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  if (a.blocks_per_sm > 0 && (int)a.blocks_per_sm < per_sm) per_sm = (int)a.blocks_per_sm;
  size_t grid = (size_t)sm_count() * per_sm;
  const size_t need = (a.ray_count + kBlock - 1) / kBlock;
  if (grid > need) grid = need;
  return (unsigned)grid;
}

template <bool MBVH, bool ANY_HIT, bool STATS>
cudaError_t launch3(const TraceArgs& a, cudaStream_t s, unsigned int* work) {
  auto kern = MBVH ? k_trace_mbvh<ANY_HIT, STATS> : k_trace_bvh<ANY_HIT, STATS>;
  kern<<<persistent_grid(kern, a), kBlock, 0, s>>>(a, work);
  return cudaGetLastError();
}

// Closest hit through the compact traversal tree, then the rays it deferred
// over the exact Mbvh. counters: [0] compact ray counter, [1] deferred rays,
// [2] exact ray counter (zeroed).
template <bool WSTATS>
auto compact_kernel(const TraceArgs& a) {
  return a.q_gates ? (a.stack_limit == 32   ? k_trace_compact<32, true, WSTATS>
                      : a.stack_limit == 48 ? k_trace_compact<48, true, WSTATS>
                                            : k_trace_compact<64, true, WSTATS>)
                   : (a.stack_limit == 32   ? k_trace_compact<32, false, WSTATS>
                      : a.stack_limit == 48 ? k_trace_compact<48, false, WSTATS>
                                            : k_trace_compact<64, false, WSTATS>);
}

cudaError_t launch_compact(const TraceArgs& a, cudaStream_t s, unsigned int* counters, uint32_t* deferred) {
  auto kern = a.walk_stats ? compact_kernel<true>(a) : compact_kernel<false>(a);
  kern<<<persistent_grid(kern, a), kBlock, 0, s>>>(a, counters, deferred, counters + 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  TraceArgs b = a;
  b.order = deferred;
  b.ray_count_dev = counters + 1;
  // at most 32 rays per refill (the kernel takes fewer when few rays were
  // deferred)
  b.ray_batch = 32;
  if (b.tboxes) {
    auto cull_kern = k_trace_mbvh<false, false, true>;
    cull_kern<<<persistent_grid(cull_kern, b), kBlock, 0, s>>>(b, counters + 2);
    return cudaGetLastError();
  }
  return launch3<true, false, false>(b, s, counters + 2);
}

template <bool MBVH>
cudaError_t launch_any(const TraceArgs& a0, cudaStream_t s) {
  if (a0.ray_count == 0) return cudaSuccess;
  // ray indices and the work counter are 32-bit; after the last batch every
  // warp adds one more ray_batch (<= 4096) to the counter, which must not wrap
  if (a0.ray_count > 0xffffffffull - (1ull << 25) || a0.ray_batch > 4096u) return cudaErrorInvalidValue;
  if (a0.stack_limit != 0 && a0.stack_limit != 32 && a0.stack_limit != 48 && a0.stack_limit != 64)
    return cudaErrorInvalidValue;
  TraceArgs a = a0;
  // any hit: most walks end after a few nodes, so refills are frequent and
  // larger pools cost fewer counter atomics (128: 34.0 against 28.7 Grays/s
  // with 32 on the 1M incoherent scene's occlusion rays)
  if (a.any_hit && a.ray_batch == 0) a.ray_batch = 128u;
  Scratch<unsigned int> work;
  Scratch<uint32_t> keys, order, acc, deferred;
  Scratch<char> sort_temp;
  cudaError_t e;
  if ((e = work.alloc(4, s)) || (e = cudaMemsetAsync(work.ptr, 0, 4 * sizeof(unsigned int), s))) return e;
  if (MBVH && a.order == nullptr && a.reorder && a.ray_count < (1u << 30)) {
    const size_t n = a.ray_count;
    const size_t tb = radix_sort_temp_bytes(n);
    if ((e = keys.alloc(n, s)) || (e = order.alloc(n, s)) || (e = acc.alloc(8, s)) || (e = sort_temp.alloc(tb, s)))
      return e;
    const uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    if ((e = cudaMemcpyAsync(acc.ptr, init, sizeof(init), cudaMemcpyHostToDevice, s))) return e;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const unsigned cap = (unsigned)sm_count() * 8u;
    k_ray_origin_bounds<<<blocks < cap ? blocks : cap, 256, 0, s>>>(a.rays, n, acc.ptr);
    k_ray_keys<<<blocks, 256, 0, s>>>(a.rays, n, acc.ptr, keys.ptr, order.ptr);
    if ((e = radix_sort_pairs(keys.ptr, order.ptr, n, 30, sort_temp.ptr, tb, a.status, s))) return e;
    a.order = order.ptr;
  }
  const bool st = a.stats != nullptr;
  if (a.any_hit) e = st ? launch3<MBVH, true, true>(a, s, work.ptr) : launch3<MBVH, true, false>(a, s, work.ptr);
  else if (st) e = launch3<MBVH, false, true>(a, s, work.ptr);
  else if (MBVH && a.qnodes && a.q_count > 0) {
    if ((e = deferred.alloc(a.ray_count, s))) return e;
    e = launch_compact(a, s, work.ptr, deferred.ptr);
  } else e = launch3<MBVH, false, false>(a, s, work.ptr);
  return e;
}

}  // namespace

cudaError_t launch_trace_mbvh(const TraceArgs& a, cudaStream_t s) { return launch_any<true>(a, s); }
cudaError_t launch_trace_bvh(const TraceArgs& a, cudaStream_t s) { return launch_any<false>(a, s); }

cudaError_t launch_candidates(const CandArgs& a, bool mbvh, cudaStream_t s) {
  if (a.ray_count == 0) return cudaSuccess;
  auto kern = mbvh ? k_candidates<true> : k_candidates<false>;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  size_t grid = (size_t)sm_count() * per_sm;
  const size_t need = (a.ray_count + kBlock - 1) / kBlock;
  if (grid > need) grid = need;
  kern<<<(unsigned)grid, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace rtbvh
