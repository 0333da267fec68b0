// Packet traversal: four rays share one walk of the tree, as with the
// reference's RayPacket4 iterators (src/iter_indices.rs:110-200 for the Bvh,
// :316-414 for the Mbvh; src/iter.rs:130-243 and :357-460 are the same walks
// over primitives).
//
// A packet is four consecutive lanes of a warp, one ray per lane; a warp
// carries eight packets. Each lane evaluates the node test for its own ray
// and the packet's decision is the OR over its four lanes (redux.sync over
// the lanes' 4-bit group mask), so the four lanes take every branch together
// and hold identical copies of the stack. All four lanes load the same node,
// which the L1 serves as one request per packet. Leaf primitives are tested
// by every lane against its own ray with SpatialTriangle::intersect4
// (src/builders/spatial_sah.rs:165-244) at t_min = 1e-4, the test the
// reference's packet benchmark runs (examples/benchmark.rs:43-68).
//
// Quad nodes: MbvhNode::intersect4 (src/mbvh_node.rs:242-295) -- slot i is
// hit when any lane has t_max > t_min and t_min < t; slots are walked 3..0
// without sorting; a hit leaf's primitives are tested at once, hit interior
// slots are pushed, and a popped node's mask uses the lanes' t of that
// moment. BVH2 nodes: Aabb::intersect4 (src/aabb.rs:217-246) on both
// children with BvhNode::sort_nodes4 (src/bvh_node.rs:180-213); a packet
// with a NaN origin or direction component walks nothing
// (src/iter_indices.rs:122-143).
//
// With the same arithmetic (no FMA, IEEE division, SSE min/max select rules)
// every lane's t, u, v and primitive and every packet's node/triangle counts
// equal the reference iterators'. Persistent kernel: a packet group takes
// kGroupBatch packets from a global counter at a time. The stack is bounded
// (kStack); a packet that would exceed it stops, reports prim -2 on its
// lanes and sets kStatusStackOverflow.
#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 128;
constexpr int kStack = 64;
constexpr uint32_t kGroupBatch = 4;

struct LaneRay {
  float ox, oy, oz, dx, dy, dz, ix, iy, iz, t;
};

__device__ __forceinline__ void ld8_nc(const void* p, float (&v)[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}

// SpatialTriangle::intersect4 for this lane's ray, on a leaf-ordered
// triangle {v0, prim}, {v1 - v0}, {v2 - v0} (the edges are the same IEEE
// subtractions the reference performs).
__device__ __forceinline__ bool tri_test4(const float4* tri, LaneRay& r, float& hu, float& hv, int32_t& prim) {
  float a0[8], a1[8];
  ld8_nc(tri, a0);
  ld8_nc(reinterpret_cast<const float*>(tri) + 8, a1);
  const float e1x = a0[4], e1y = a0[5], e1z = a0[6];
  const float e2x = a1[0], e2y = a1[1], e2z = a1[2];
  const float hx = (r.dy * e2z) - (r.dz * e2y);
  const float hy = (r.dz * e2x) - (r.dx * e2z);
  const float hz = (r.dx * e2y) - (r.dy * e2x);
  const float det = ((e1x * hx) + (e1y * hy)) + (e1z * hz);
  if (!(det <= -1e-6f || det >= 1e-6f)) return false;
  const float f = 1.0f / det;
  const float sx = r.ox - a0[0], sy = r.oy - a0[1], sz = r.oz - a0[2];
  const float u = f * (((sx * hx) + (sy * hy)) + (sz * hz));
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  const float qx = sy * e1z - sz * e1y;
  const float qy = sz * e1x - sx * e1z;
  const float qz = sx * e1y - sy * e1x;
  const float v = f * (((r.dx * qx) + (r.dy * qy)) + (r.dz * qz));
  if (!(v >= 0.0f && (u + v) <= 1.0f)) return false;
  const float t = f * (((e2x * qx) + (e2y * qy)) + (e2z * qz));
  if (!(t >= 1e-4f && t < r.t)) return false;
  r.t = t;
  hu = u;
  hv = v;
  prim = __float_as_int(a0[3]);
  return true;
}

// MbvhNode::intersect4 for this lane's ray: bit i set when slot i passes
// t_max > t_min && t_min < t. Axes folded x, then y, then z.
__device__ __forceinline__ uint32_t quad_test4(const DMNode* node, const LaneRay& r, int4& children, int4& counts) {
  float vx[8], vy[8], vz[8], vc[8];
  ld8_nc(node, vx);
  ld8_nc(reinterpret_cast<const float*>(node) + 8, vy);
  ld8_nc(reinterpret_cast<const float*>(node) + 16, vz);
  ld8_nc(reinterpret_cast<const float*>(node) + 24, vc);
  children = make_int4(__float_as_int(vc[0]), __float_as_int(vc[1]), __float_as_int(vc[2]), __float_as_int(vc[3]));
  counts = make_int4(__float_as_int(vc[4]), __float_as_int(vc[5]), __float_as_int(vc[6]), __float_as_int(vc[7]));
  uint32_t m = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float x1 = (vx[i] - r.ox) * r.ix, x2 = (vx[4 + i] - r.ox) * r.ix;
    float tmin = sse_min(x1, x2), tmax = sse_max(x1, x2);
    const float y1 = (vy[i] - r.oy) * r.iy, y2 = (vy[4 + i] - r.oy) * r.iy;
    tmin = sse_max(tmin, sse_min(y1, y2));
    tmax = sse_min(tmax, sse_max(y1, y2));
    const float z1 = (vz[i] - r.oz) * r.iz, z2 = (vz[4 + i] - r.oz) * r.iz;
    tmin = sse_max(tmin, sse_min(z1, z2));
    tmax = sse_min(tmax, sse_max(z1, z2));
    if (tmax > tmin && tmin < r.t) m |= 1u << i;
  }
  return m;
}

// Aabb::intersect4 for this lane's ray: tnear = t_min; hit when t_max > 0,
// t_max > t_min and t_min < t.
__device__ __forceinline__ bool box_test4(const DAabb& b, const LaneRay& r, float& tnear) {
  const float x1 = (b.min[0] - r.ox) * r.ix, y1 = (b.min[1] - r.oy) * r.iy, z1 = (b.min[2] - r.oz) * r.iz;
  const float x2 = (b.max[0] - r.ox) * r.ix, y2 = (b.max[1] - r.oy) * r.iy, z2 = (b.max[2] - r.oz) * r.iz;
  const float tmin = sse_max(sse_min(x1, x2), sse_max(sse_min(y1, y2), sse_min(z1, z2)));
  const float tmax = sse_min(sse_max(x1, x2), sse_min(sse_max(y1, y2), sse_max(z1, z2)));
  tnear = tmin;
  return tmax > 0.0f && tmax > tmin && tmin < r.t;
}

__device__ __forceinline__ int sel4i(const int4& v, uint32_t i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

template <bool MBVH, bool STATS>
__global__ void __launch_bounds__(kBlock) k_trace_packets(PacketArgs a, unsigned int* work) {
  const int lane = threadIdx.x & 31;
  const int sub = lane & 3;
  const int leader = lane & ~3;
  const unsigned gmask = 0xfu << leader;
  int32_t stack[kStack];
  for (;;) {
    unsigned int base = 0;
    if (sub == 0) base = atomicAdd(work, kGroupBatch);
    base = __shfl_sync(gmask, base, leader);
    if ((size_t)base >= a.packet_count) break;
    const size_t end = ((size_t)base + kGroupBatch < a.packet_count) ? (size_t)base + kGroupBatch : a.packet_count;
    for (size_t p = base; p < end; ++p) {
      const size_t r = 4 * p + (size_t)sub;
      LaneRay ray;
      ray.ox = __ldg(a.origin[0] + r);
      ray.oy = __ldg(a.origin[1] + r);
      ray.oz = __ldg(a.origin[2] + r);
      ray.dx = __ldg(a.direction[0] + r);
      ray.dy = __ldg(a.direction[1] + r);
      ray.dz = __ldg(a.direction[2] + r);
      ray.ix = 1.0f / ray.dx;
      ray.iy = 1.0f / ray.dy;
      ray.iz = 1.0f / ray.dz;
      ray.t = a.t[r];
      float hu = 0.0f, hv = 0.0f;
      int32_t prim = -1;
      uint32_t visits = 0, tests = 0, max_depth = 0;
      int sp = -1;
      if (MBVH) {
        if (a.node_count > 0) {
          int4 children, counts;
          uint32_t res = __reduce_or_sync(gmask, quad_test4(a.mnodes, ray, children, counts));
          if (STATS) ++visits;
          for (;;) {
            bool stop = false;
#pragma unroll 1
            for (int i = 0; i < 4; ++i) {
              const uint32_t id = 3u - (uint32_t)i;
              if (!((res >> id) & 1u)) continue;
              const int32_t count = sel4i(counts, id), lf = sel4i(children, id);
              if (count > -1) {
                if (lf < 0 || (uint32_t)lf + (uint32_t)count > a.prim_count) {
                  if (sub == 0) atomicOr(a.status, kStatusBadIndex);
                  stop = true;
                  break;
                }
                for (int32_t j = 0; j < count; ++j) {
                  if (STATS) ++tests;
                  tri_test4(a.tris + kTriFloat4 * (size_t)(lf + j), ray, hu, hv, prim);
                }
              } else if (lf > -1) {
                if (sp + 1 >= kStack) {
                  if (sub == 0) atomicOr(a.status, kStatusStackOverflow);
                  prim = -2;
                  stop = true;
                  break;
                }
                stack[++sp] = lf;
                if (STATS && (uint32_t)(sp + 1) > max_depth) max_depth = (uint32_t)(sp + 1);
              }
            }
            if (stop || sp < 0) break;
            const int32_t current = stack[sp--];
            if ((uint32_t)current >= a.node_count) {
              if (sub == 0) atomicOr(a.status, kStatusBadIndex);
              break;
            }
            res = __reduce_or_sync(gmask, quad_test4(a.mnodes + current, ray, children, counts));
            if (STATS) ++visits;
          }
        }
      } else {
        const bool nan = (ray.ox != ray.ox) || (ray.oy != ray.oy) || (ray.oz != ray.oz) || (ray.dx != ray.dx) ||
                         (ray.dy != ray.dy) || (ray.dz != ray.dz);
        const bool any_nan = __reduce_or_sync(gmask, nan ? 1u : 0u) != 0;
        sp = (a.node_count == 0 || any_nan) ? -1 : 0;
        stack[0] = 0;
        while (sp >= 0) {
          const int32_t ni = stack[sp--];
          if ((uint32_t)ni >= a.node_count) {
            if (sub == 0) atomicOr(a.status, kStatusBadIndex);
            break;
          }
          const DAabb node = load_aabb(a.nodes + ni);
          if (node.count > -1) {
            if (node.left_first < 0 || (uint32_t)node.left_first + (uint32_t)node.count > a.prim_count) {
              if (sub == 0) atomicOr(a.status, kStatusBadIndex);
              break;
            }
            for (int32_t j = 0; j < node.count; ++j) {
              if (STATS) ++tests;
              tri_test4(a.tris + kTriFloat4 * (size_t)(node.left_first + j), ray, hu, hv, prim);
            }
          } else if (node.left_first > -1) {
            if (STATS) ++visits;
            const int32_t lf = node.left_first;
            if ((uint32_t)lf + 1u >= a.node_count) {
              if (sub == 0) atomicOr(a.status, kStatusBadIndex);
              break;
            }
            float lt = 0.0f, rt = 0.0f;
            const bool lh = __reduce_or_sync(gmask, box_test4(load_aabb(a.nodes + lf), ray, lt) ? 1u : 0u) != 0;
            const bool rh = __reduce_or_sync(gmask, box_test4(load_aabb(a.nodes + lf + 1), ray, rt) ? 1u : 0u) != 0;
            if (sp + 2 >= kStack) {
              if (sub == 0) atomicOr(a.status, kStatusStackOverflow);
              prim = -2;
              break;
            }
            if (lh && rh) {
              const bool any_less = __reduce_or_sync(gmask, lt < rt ? 1u : 0u) != 0;
              if (any_less) { stack[++sp] = lf; stack[++sp] = lf + 1; }
              else { stack[++sp] = lf + 1; stack[++sp] = lf; }
            } else if (lh) {
              stack[++sp] = lf;
            } else if (rh) {
              stack[++sp] = lf + 1;
            }
            if (STATS && (uint32_t)(sp + 1) > max_depth) max_depth = (uint32_t)(sp + 1);
          }
        }
      }
      a.t[r] = ray.t;
      if (a.hits) a.hits[r] = make_float4(ray.t, hu, hv, __int_as_float(prim));
      if (STATS && sub == 0) {
        a.stats[3 * p + 0] = visits;
        a.stats[3 * p + 1] = tests;
        a.stats[3 * p + 2] = max_depth;
      }
    }
  }
}

template <bool MBVH, bool STATS>
cudaError_t launch2(const PacketArgs& a, cudaStream_t s, unsigned int* work) {
  auto kern = k_trace_packets<MBVH, STATS>;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  size_t grid = (size_t)sm_count() * per_sm;
  const size_t need = (a.packet_count + (kBlock / 4) - 1) / (kBlock / 4);
  if (grid > need) grid = need;
  kern<<<(unsigned)grid, kBlock, 0, s>>>(a, work);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace_packets(const PacketArgs& a, bool mbvh, cudaStream_t s) {
  if (a.packet_count == 0) return cudaSuccess;
  // 32-bit packet counter: after the last batch every group adds kGroupBatch
  // once more, which must not wrap
  if (a.packet_count > (1ull << 30)) return cudaErrorInvalidValue;
  Scratch<unsigned int> work;
  cudaError_t e;
  if ((e = work.alloc(1, s)) || (e = cudaMemsetAsync(work.ptr, 0, sizeof(unsigned int), s))) return e;
  const bool st = a.stats != nullptr;
  if (mbvh) e = st ? launch2<true, true>(a, s, work.ptr) : launch2<true, false>(a, s, work.ptr);
  else e = st ? launch2<false, true>(a, s, work.ptr) : launch2<false, false>(a, s, work.ptr);
  return e;
}

}  // namespace rtbvh
