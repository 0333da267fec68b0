// BVH2 -> 4-wide MBVH collapse (Mbvh::construct, src/bvh.rs:381-404, and
// MbvhNode::merge_nodes, src/mbvh_node.rs:297-411) on the GPU.
//
// The reference numbers quad nodes by a recursive walk that hands out
// `pool_ptr++` in slot order (a pre-order over quad nodes). Quad nodes are
// exactly the interior BVH2 nodes at even depth, and the quad subtree rooted
// at such a node g holds cntE(g) quad nodes, where
//   cntE(c) = 1 + cntO(left) + cntO(right),  cntO(c) = cntE(left) + cntE(right)
// for interior c and 0 for leaves. So:
//   1. parent pointers;
//   2. cntE/cntO bottom-up (the second child to arrive at a parent computes it);
//   3. top-down, one quad level per step of a cooperative launch: a quad node
//      with index mi gives its k-th interior slot the index
//      mi + 1 + sum of cntE over the interior slots before it.
// The slot contents reproduce merge_nodes line by line, including its quirks
// (a leaf child keeps the parent's box in its slot; the second slot of that
// side stays empty with the parent's box).
#include <mutex>

#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kNone = 0xffffffffu;

// Arrival at a parent in the bottom-up walks: atomic add with acquire and
// release semantics at device scope. The release publishes this thread's
// writes for its child; the second arrival's acquire makes the sibling's
// writes visible to it (one instruction where fence + add + fence were).
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t* p) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

__device__ __forceinline__ bool box_contains(const DAabb& outer, const DAabb& inner) {
  // false on NaN: such a box counts as not containing
  return outer.min[0] <= inner.min[0] && outer.min[1] <= inner.min[1] && outer.min[2] <= inner.min[2] &&
         outer.max[0] >= inner.max[0] && outer.max[1] >= inner.max[1] && outer.max[2] >= inner.max[2];
}

// Vertex box of triangle p (9 floats), grown by 1e-4: what Bvh::refit
// (src/bvh.rs:176-205) gives a leaf of that one triangle.
__device__ __forceinline__ DAabb grown_triangle_box(const float* __restrict__ vertices, uint32_t p) {
  const float* v = vertices + 9 * (size_t)p;
  DAabb b;
  for (int a = 0; a < 3; ++a) { b.min[a] = 1e34f; b.max[a] = -1e34f; }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float x = __ldg(v + 3 * j + a);
      b.min[a] = rs_min(b.min[a], x);
      b.max[a] = rs_max(b.max[a], x);
    }
  for (int a = 0; a < 3; ++a) { b.min[a] = b.min[a] - 0.0001f; b.max[a] = b.max[a] + 0.0001f; }
  b.count = 0;
  b.left_first = 0;
  return b;
}

__global__ void __launch_bounds__(kBlock)
    k_parents(const DAabb* __restrict__ nodes, uint32_t node_count, uint32_t* __restrict__ parent,
              uint32_t* __restrict__ arrive, uint32_t* __restrict__ status) {
  uint32_t c = blockIdx.x * kBlock + threadIdx.x;
  if (c >= node_count) return;
  arrive[c] = 0;
  DAabb nd = load_aabb(nodes + c);
  if (nd.count < 0 && nd.left_first >= 0) {
    uint32_t lf = (uint32_t)nd.left_first;
    if (lf + 1 < node_count) {
      parent[lf] = c;
      parent[lf + 1] = c;
    } else {
      atomicOr(status, kStatusBadIndex);
    }
  }
}

// With TRIS, the same walk also computes every node's traversal box `tb`
// from the triangles: a leaf's is the union of its triangles' vertex boxes
// grown by 1e-4, an interior node's the union of its children's (the union
// of boxes grown by 1e-4 is the union grown by 1e-4); count/left_first are
// copied from `nodes`.
template <bool TRIS>
__global__ void __launch_bounds__(kBlock)
    k_counts_bottom_up(const DAabb* __restrict__ nodes, uint32_t node_count, const uint32_t* __restrict__ parent,
                       uint32_t* __restrict__ arrive, uint32_t* __restrict__ cnt_e, uint32_t* __restrict__ cnt_o,
                       MbvhTriangles tri, uint32_t* __restrict__ status) {
  uint32_t c = blockIdx.x * kBlock + threadIdx.x;
  if (c >= node_count) return;
  DAabb nd = load_aabb(nodes + c);
  if (nd.count < 0) return;  // walks start at leaves
  cnt_e[c] = 0;
  cnt_o[c] = 0;
  if (TRIS) {
    DAabb box = nd;
    for (int a = 0; a < 3; ++a) { box.min[a] = 1e34f; box.max[a] = -1e34f; }
    if (nd.left_first >= 0) {
      for (int a = 0; a < 3; ++a) { box.min[a] = 1e34f - 0.0001f; box.max[a] = -1e34f + 0.0001f; }
      for (int32_t i = 0; i < nd.count; ++i) {
        const uint32_t slot = (uint32_t)nd.left_first + (uint32_t)i;
        const uint32_t p = slot < tri.index_count ? __ldg(tri.indices + slot) : kNone;
        if (p >= tri.vertex_count) {
          atomicOr(status, kStatusBadIndex);
          break;
        }
        const DAabb t = grown_triangle_box(tri.vertices, p);
        for (int a = 0; a < 3; ++a) { box.min[a] = rs_min(box.min[a], t.min[a]); box.max[a] = rs_max(box.max[a], t.max[a]); }
      }
    }
    store_aabb(tri.tb + c, box);
  }
  uint32_t x = c;
  for (uint32_t steps = 0; steps < node_count; ++steps) {
    uint32_t p = __ldcg(parent + x);
    if (p == kNone) break;
    if (arrive_acq_rel(arrive + p) == 0u) break;  // first arrival: the sibling finishes p
    DAabb pn = load_aabb(nodes + p);
    uint32_t lf = (uint32_t)pn.left_first;
    uint32_t e = 1u + __ldcg(cnt_o + lf) + __ldcg(cnt_o + lf + 1);
    uint32_t o = __ldcg(cnt_e + lf) + __ldcg(cnt_e + lf + 1);
    cnt_e[p] = e;
    cnt_o[p] = o;
    if (TRIS) {
      const DAabb l = load_aabb_cg(tri.tb + lf), r = load_aabb_cg(tri.tb + lf + 1);
      for (int a = 0; a < 3; ++a) {
        pn.min[a] = rs_min(l.min[a], r.min[a]);
        pn.max[a] = rs_max(l.max[a], r.max[a]);
      }
      store_aabb(tri.tb + p, pn);
    }
    x = p;
  }
}

struct CollapseParams {
  const DAabb* nodes;
  uint32_t node_count;
  const uint32_t* cnt_e;
  DMNode* mnodes;
  uint32_t m_total;
  uint2* queue[2];
  uint32_t* qcount;  // 3 rotating counters
  GridBarrier* bar;
  uint32_t* status;
  // escape flags only: triangles, per quad node the intersection of the
  // slot boxes on the way to it, the count of escaped triangles
  MbvhTriangles tri;
  DAabb* ibox;
  uint32_t* escaped;
  DTBox* tboxes;  // optional (TRIS): subtree boxes of every quad node's slots
  // optional: the quad count, read on the device; m_total then holds the
  // capacity of mnodes / ibox / tboxes
  const uint32_t* m_total_dev;
};

// Warp-aggregated reservation of n consecutive entries from *counter: every
// lane of the warp calls it (n = 0 for nothing), one atomic per warp; the
// lane's first entry is returned. The top-down passes append to one queue
// counter per level, whose atomics would otherwise serialise.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counter, uint32_t n) {
  const int lane = threadIdx.x & 31;
  uint32_t incl = n;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + incl - n;
}

__device__ __forceinline__ void set_slot_box(DMNode& m, int i, const DAabb& b) {
  m.min_x[i] = b.min[0]; m.min_y[i] = b.min[1]; m.min_z[i] = b.min[2];
  m.max_x[i] = b.max[0]; m.max_y[i] = b.max[1]; m.max_z[i] = b.max[2];
}

// Escape flags of quad node mi's slots (TRIS): an interior slot hands its
// child quad the intersection of the slot boxes on the way to it; a leaf
// slot's triangles are escaped when their vertex box grown by 1e-4 is not
// inside that intersection -- the reference's walk tests these boxes
// before it yields the triangle (src/iter_indices.rs:264-313), so it can
// miss the triangle's hits. Flags go to the flags word of each leaf-ordered
// triangle record (kTriEscape).
__device__ void mark_escapes(const CollapseParams& p, uint32_t mi, const DMNode& m) {
  const DAabb in = load_aabb_cg(p.ibox + mi);
  uint32_t n_esc = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int32_t ch = m.children[i], cnt = m.counts[i];
    if (cnt < 0 && ch < 0) continue;  // empty slot
    const float smin[3] = {m.min_x[i], m.min_y[i], m.min_z[i]}, smax[3] = {m.max_x[i], m.max_y[i], m.max_z[i]};
    DAabb box;
    bool nan = false;
    for (int a = 0; a < 3; ++a) {
      nan = nan || !(smin[a] == smin[a]) || !(smax[a] == smax[a]);
      box.min[a] = fmaxf(in.min[a], smin[a]);
      box.max[a] = fminf(in.max[a], smax[a]);
    }
    if (nan)  // a NaN bound: nothing below counts as inside
      for (int a = 0; a < 3; ++a) { box.min[a] = 3.0e38f; box.max[a] = -3.0e38f; }
    box.count = 0;
    box.left_first = 0;
    if (cnt < 0) {
      if ((uint32_t)ch < p.m_total) store_aabb(p.ibox + ch, box);
      continue;
    }
    for (int32_t j = 0; j < cnt; ++j) {
      const uint32_t slot = (uint32_t)ch + (uint32_t)j;
      const uint32_t prim = slot < p.tri.index_count ? __ldg(p.tri.indices + slot) : kNone;
      if (prim >= p.tri.vertex_count) {
        atomicOr(p.status, kStatusBadIndex);
        break;
      }
      const bool esc = !box_contains(box, grown_triangle_box(p.tri.vertices, prim));
      reinterpret_cast<float*>(p.tri.tris + (size_t)kTriFloat4 * slot + 1)[3] = __uint_as_float(esc ? kTriEscape : 0u);
      n_esc += esc ? 1u : 0u;
    }
  }
  if (n_esc) atomicAdd(p.escaped, n_esc);
}

// merge_nodes(mi, c) without the recursion: fills quad node mi and appends
// its interior slots (bvh node, quad index) to `next`. AGG: called by all
// lanes of a warp (`valid` false for lanes without an item), the queue
// entries reserved once per warp.
template <bool TRIS, bool AGG>
__device__ void emit_quad(const CollapseParams& p, uint32_t c, uint32_t mi, uint2* next, uint32_t* next_count,
                          bool valid = true) {
  const DAabb cur = load_aabb(p.nodes + c);
  DMNode m;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    set_slot_box(m, i, cur);
    m.children[i] = -1;
    m.counts[i] = -1;
  }
  int32_t nodes_[4] = {-1, -1, -1, -1};
  int32_t leafs[4] = {-1, -1, -1, -1};
  int32_t sub[4] = {-1, -1, -1, -1};  // BVH2 node under each slot (TRIS: its box from the triangles)
  if (cur.left_first >= 0) {
    const uint32_t lf = (uint32_t)cur.left_first;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int s0 = 2 * side;
      const uint32_t child = lf + side;
      if (child < p.node_count) {
        const DAabb cn = load_aabb(p.nodes + child);
        if (cn.left_first >= 0) {
          const uint32_t clf = (uint32_t)cn.left_first;
          if (cn.count >= 0) {
            nodes_[s0] = (int32_t)clf;
            leafs[s0] = cn.count;
            sub[s0] = (int32_t)child;
          } else if (clf + 1 < p.node_count) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              const DAabb g = load_aabb(p.nodes + clf + k);
              if (g.count >= 0) {
                nodes_[s0 + k] = g.left_first;
                leafs[s0 + k] = g.count;
              } else {
                nodes_[s0 + k] = (int32_t)(clf + k);
              }
              set_slot_box(m, s0 + k, g);
              sub[s0 + k] = (int32_t)(clf + k);
            }
          } else {
            atomicOr(p.status, kStatusBadIndex);
          }
        }
      }
    }
  }
  uint32_t n_int = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) n_int += (nodes_[i] >= 0 && leafs[i] < 0) ? 1u : 0u;
  if (!valid) n_int = 0;
  uint32_t qslot = 0;
  if (AGG) qslot = warp_reserve(next_count, n_int);
  else if (n_int) qslot = atomicAdd(next_count, n_int);
  if (!valid) return;
  uint32_t next_index = mi + 1u;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int32_t node = nodes_[i];
    const int32_t count = leafs[i];
    if (node >= 0 && count >= 0) {
      m.children[i] = node;
      m.counts[i] = count;
      continue;
    } else if (node < 0) {
      if (node != -1) atomicOr(p.status, kStatusBadIndex);
      continue;
    }
    const uint32_t g = (uint32_t)node;
    const uint32_t idx = next_index;
    next_index += __ldg(p.cnt_e + g);
    const uint32_t slot = qslot++;
    if (idx < p.m_total) {
      m.children[i] = (int32_t)idx;
      if (slot < p.m_total) next[slot] = make_uint2(g, idx);
      else atomicOr(p.status, kStatusBadIndex);
    } else {
      atomicOr(p.status, kStatusBadIndex);
    }
  }
  if (mi < p.m_total) {
    float4* dst = reinterpret_cast<float4*>(p.mnodes + mi);
    const float4* src = reinterpret_cast<const float4*>(&m);
#pragma unroll
    for (int k = 0; k < 8; ++k) dst[k] = src[k];
    if (TRIS) mark_escapes(p, mi, m);
    if (TRIS && p.tboxes) {
      DTBox t;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        bool ok = sub[i] >= 0 && (uint32_t)sub[i] < p.node_count;
        DAabb b = cur;
        if (ok) b = load_aabb_cg(p.tri.tb + sub[i]);
        for (int a = 0; a < 3; ++a)  // false for NaN
          ok = ok && fabsf(b.min[a]) <= kCompactRange && fabsf(b.max[a]) <= kCompactRange;
        const float inf = __int_as_float(0x7f800000);
        t.min_x[i] = ok ? b.min[0] : -inf; t.max_x[i] = ok ? b.max[0] : inf;
        t.min_y[i] = ok ? b.min[1] : -inf; t.max_y[i] = ok ? b.max[1] : inf;
        t.min_z[i] = ok ? b.min[2] : -inf; t.max_z[i] = ok ? b.max[2] : inf;
      }
      float4* td = reinterpret_cast<float4*>(p.tboxes + mi);
      const float4* ts = reinterpret_cast<const float4*>(&t);
#pragma unroll
      for (int k = 0; k < 6; ++k) td[k] = ts[k];
    }
  } else {
    atomicOr(p.status, kStatusBadIndex);
  }
}

template <bool TRIS>
__global__ void __launch_bounds__(kBlock) k_collapse(CollapseParams p) {
  if (p.m_total_dev) {
    // every block reads the same word (written before the launch), so all
    // of them return here together or none does
    const uint32_t mt = __ldcg(p.m_total_dev);
    if (mt == 0 || mt > p.m_total) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(p.status, kStatusBadIndex);
      return;
    }
    p.m_total = mt;
  }
  const uint32_t G = gridDim.x;
  const uint32_t tid = blockIdx.x * kBlock + threadIdx.x, nthreads = G * kBlock;
  for (uint32_t level = 0; level < p.m_total + 1; ++level) {
    uint32_t size = __ldcg(p.qcount + (level % 3));
    if (size == 0) break;
    if (size > p.m_total) size = p.m_total;  // only after a kStatusBadIndex
    const uint2* q = p.queue[level & 1];
    uint2* next = p.queue[(level + 1) & 1];
    uint32_t* next_count = p.qcount + ((level + 1) % 3);
    // warp-uniform loop: every lane takes part in the queue reservation
    for (uint32_t k0 = tid - (threadIdx.x & 31u); k0 < size; k0 += nthreads) {
      const uint32_t k = k0 + (threadIdx.x & 31u);
      const bool valid = k < size;
      const uint2 item = valid ? __ldcg(q + k) : make_uint2(0u, 0u);
      emit_quad<TRIS, true>(p, item.x, item.y, next, next_count, valid);
    }
    if (tid == 0) p.qcount[(level + 2) % 3] = 0;
    if (!grid_sync(p.bar, G, p.status)) return;
  }
}

__global__ void k_collapse_init(const uint32_t* cnt_e, const DAabb* nodes, uint2* queue0, uint32_t* qcount,
                                uint32_t* m_total_out) {
  if (threadIdx.x == 0) {
    queue0[0] = make_uint2(0u, 0u);
    qcount[0] = 1;
    qcount[1] = 0;
    qcount[2] = 0;
    DAabb r = *nodes;
    uint32_t t = r.count < 0 ? cnt_e[0] : 1u;
    *m_total_out = t;
  }
}

// The root quad's slots are the first boxes on every way down.
__global__ void k_ibox_init(DAabb* ibox) {
  if (threadIdx.x == 0) {
    DAabb b;
    for (int a = 0; a < 3; ++a) { b.min[a] = -3.0e38f; b.max[a] = 3.0e38f; }
    b.count = 0;
    b.left_first = 0;
    store_aabb(ibox, b);
  }
}


// ---------------------------------------------------------------- many meshes
// A concatenated forest: mesh m's root is BVH2 node 2 off_m - m. Its quad
// nodes get the contiguous index range [mbase[m], mbase[m+1]) (the
// single-mesh numbering shifted by mbase[m]), and one block per mesh runs
// the top-down frontier of k_collapse with block barriers.
__global__ void __launch_bounds__(1024) k_seg_mbase(const DAabb* __restrict__ nodes, const uint32_t* __restrict__ cnt_e,
                                                    const uint32_t* __restrict__ prim_off, uint32_t mesh_count,
                                                    uint32_t* __restrict__ mbase) {
  __shared__ uint32_t s_warp[32];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < mesh_count; base += 1024) {
    const uint32_t m = base + threadIdx.x;
    uint32_t q = 0;
    if (m < mesh_count) {
      const uint32_t off = prim_off[m], n = prim_off[m + 1] - off;
      if (n > 0) {
        const uint32_t root = 2u * off - m;
        q = load_aabb(nodes + root).count < 0 ? cnt_e[root] : 1u;
      }
    }
    uint32_t total;
    const uint32_t incl = block_inclusive_scan<1024>(q, s_warp, &total);
    if (m < mesh_count) mbase[m] = carry + incl - q;
    carry += total;
  }
  if (threadIdx.x == 0) mbase[mesh_count] = carry;
}

struct SegCollapseParams {
  CollapseParams c;
  const uint32_t* prim_off;
  const uint32_t* order;
  const uint32_t* mbase;
  uint2* queue[2];
  uint32_t mesh_count;
};

__global__ void __launch_bounds__(kBlock) k_collapse_segments(SegCollapseParams p) {
  __shared__ uint32_t s_count[2];
  for (uint32_t q = blockIdx.x; q < p.mesh_count; q += gridDim.x) {
    const uint32_t m = p.order[q];
    const uint32_t off = p.prim_off[m], n = p.prim_off[m + 1] - off;
    if (n == 0) continue;
    const uint32_t base = p.mbase[m];
    const uint32_t quads = p.mbase[m + 1] - base;
    const uint32_t root = 2u * off - m;
    const DAabb rb = load_aabb(p.c.nodes + root);
    if (rb.count >= 0) {
      // Root leaf (n <= 2): the single-mesh tree has this one node, so
      // merge_nodes finds only the root itself in slot 0. emit_quad would
      // read the next mesh's nodes as the root's second child here.
      if (threadIdx.x == 0 && quads >= 1) {
        DMNode q;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          set_slot_box(q, i, rb);
          q.children[i] = -1;
          q.counts[i] = -1;
        }
        q.children[0] = rb.left_first;
        q.counts[0] = rb.count;
        float4* dst = reinterpret_cast<float4*>(p.c.mnodes + base);
        const float4* src = reinterpret_cast<const float4*>(&q);
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = src[k];
      }
      continue;
    }
    if (threadIdx.x == 0) {
      p.queue[0][base] = make_uint2(root, base);
      s_count[0] = 1;
      s_count[1] = 0;
    }
    __syncthreads();
    int cur = 0;
    for (uint32_t level = 0; level <= quads; ++level) {
      uint32_t size = s_count[cur];
      if (size == 0) break;
      if (size > quads) size = quads;
      const uint2* qin = p.queue[cur] + base;
      uint2* qout = p.queue[cur ^ 1] + base;
      for (uint32_t k = threadIdx.x; k < size; k += kBlock) {
        const uint2 item = qin[k];
        emit_quad<false, false>(p.c, item.x, item.y, qout, &s_count[cur ^ 1]);
      }
      __syncthreads();
      if (threadIdx.x == 0) s_count[cur] = 0;
      __syncthreads();
      cur ^= 1;
    }
    __syncthreads();
  }
}

// Bvh::refit (src/bvh.rs:176-205): leaf box = union of its primitives'
// boxes + 1e-4, interior box = union of the two children + 1e-4, computed
// bottom-up (the second child to arrive finishes the parent). Unions are
// exact, so the boxes equal the reference's reverse-order loop bit for bit.
// Unlike the reference, count/left_first are kept (see include/rtbvh.h).
__global__ void __launch_bounds__(kBlock)
    k_refit(DAabb* __restrict__ nodes, uint32_t node_count, const uint32_t* __restrict__ indices, uint32_t index_count,
            uint32_t prim_count,
            const DAabb* __restrict__ aabbs, const uint32_t* __restrict__ parent, uint32_t* __restrict__ arrive,
            uint32_t* __restrict__ status) {
  uint32_t c = blockIdx.x * kBlock + threadIdx.x;
  if (c >= node_count) return;
  DAabb nd = load_aabb_cg(nodes + c);
  if (nd.count < 0 && nd.left_first >= 0) return;  // interior: finished by a child walk
  DAabb box = nd;
  for (int a = 0; a < 3; ++a) { box.min[a] = 1e34f; box.max[a] = -1e34f; }
  if (nd.left_first >= 0) {
    for (int32_t i = 0; i < nd.count; ++i) {
      uint32_t slot = (uint32_t)nd.left_first + (uint32_t)i;
      if (slot >= index_count) { atomicOr(status, kStatusBadIndex); break; }
      uint32_t p = __ldg(indices + slot);
      if (p >= prim_count) { atomicOr(status, kStatusBadIndex); break; }
      DAabb b = load_aabb(aabbs + p);
      for (int a = 0; a < 3; ++a) { box.min[a] = rs_min(box.min[a], b.min[a]); box.max[a] = rs_max(box.max[a], b.max[a]); }
    }
    for (int a = 0; a < 3; ++a) { box.min[a] = box.min[a] - 0.0001f; box.max[a] = box.max[a] + 0.0001f; }
  }
  store_aabb(nodes + c, box);
  if (nd.left_first < 0) return;
  uint32_t x = c;
  for (uint32_t steps = 0; steps < node_count; ++steps) {
    uint32_t p = __ldcg(parent + x);
    if (p == kNone) break;
    if (arrive_acq_rel(arrive + p) == 0u) break;
    DAabb pn = load_aabb_cg(nodes + p);
    const uint32_t lf = (uint32_t)pn.left_first;
    DAabb l = load_aabb_cg(nodes + lf), r = load_aabb_cg(nodes + lf + 1);
    for (int a = 0; a < 3; ++a) {
      float mn = rs_min(rs_min(1e34f, l.min[a]), r.min[a]);
      float mx = rs_max(rs_max(-1e34f, l.max[a]), r.max[a]);
      pn.min[a] = mn - 0.0001f;
      pn.max[a] = mx + 0.0001f;
    }
    store_aabb(nodes + p, pn);
    x = p;
  }
}

}  // namespace

ResultCode build_mbvh(const DAabb* nodes, uint32_t node_count, cudaStream_t s, DMNode** mnodes_out,
                      uint32_t* mnode_count, const MbvhTriangles* tri, uint32_t* escaped_out) {
  *mnodes_out = nullptr;
  *mnode_count = 0;
  if (escaped_out) *escaped_out = 0;
  if (node_count == 0) return Ok;  // Mbvh::default()
  const bool with_tris = tri != nullptr;
  if (with_tris && (!tri->indices || !tri->vertices || !tri->tris || !tri->tb)) return Error;
  cudaError_t e;
  Scratch<uint32_t> parent, arrive, cnt_e, cnt_o, status, mtot;
  if ((e = parent.alloc(node_count, s)) || (e = arrive.alloc(node_count, s)) || (e = cnt_e.alloc(node_count, s)) ||
      (e = cnt_o.alloc(node_count, s)) || (e = status.alloc(4, s)) || (e = mtot.alloc(4, s)))
    return cuda_rc(e);
  if ((e = cudaMemsetAsync(parent.ptr, 0xff, (size_t)node_count * 4, s)) ||
      (e = cudaMemsetAsync(status.ptr, 0, 16, s)))
    return cuda_rc(e);
  // unreachable nodes keep an empty leaf box (never read by a collapse)
  if (with_tris && (e = cudaMemsetAsync(tri->tb, 0, (size_t)node_count * sizeof(DAabb), s))) return cuda_rc(e);
  const unsigned blocks = (node_count + kBlock - 1) / kBlock;
  k_parents<<<blocks, kBlock, 0, s>>>(nodes, node_count, parent.ptr, arrive.ptr, status.ptr);
  const MbvhTriangles none;
  if (with_tris)
    k_counts_bottom_up<true><<<blocks, kBlock, 0, s>>>(nodes, node_count, parent.ptr, arrive.ptr, cnt_e.ptr,
                                                       cnt_o.ptr, *tri, status.ptr);
  else
    k_counts_bottom_up<false><<<blocks, kBlock, 0, s>>>(nodes, node_count, parent.ptr, arrive.ptr, cnt_e.ptr,
                                                        cnt_o.ptr, none, status.ptr);
  Scratch<uint2> q0, q1;
  Scratch<uint32_t> qcount;
  Scratch<GridBarrier> bar;
  if ((e = qcount.alloc(4, s)) || (e = bar.alloc(1, s))) return cuda_rc(e);
  if ((e = q0.alloc(node_count, s)) || (e = q1.alloc(node_count, s))) return cuda_rc(e);
  k_collapse_init<<<1, 32, 0, s>>>(cnt_e.ptr, nodes, q0.ptr, qcount.ptr, mtot.ptr);
  // The quad count stays on the device (the collapse reads it); arrays are
  // sized by its bound: quad nodes are interior BVH2 nodes, at most
  // (node_count - 1) / 2 of a binary tree, or the root leaf.
  const uint32_t m_cap = (node_count + 1u) / 2u;
  Scratch<DAabb> ibox;
  if (with_tris) {
    if ((e = ibox.alloc(m_cap, s))) return cuda_rc(e);
    k_ibox_init<<<1, 32, 0, s>>>(ibox.ptr);
  }
  DMNode* mnodes = nullptr;
  DTBox* tboxes = nullptr;
  if ((e = device_alloc(&mnodes, m_cap, s))) return cuda_rc(e);
  if (with_tris && tri->tboxes_out && (e = device_alloc(&tboxes, m_cap, s))) {
    pool_free(mnodes, s);
    return cuda_rc(e);
  }
  auto drop = [&]() {
    pool_free(mnodes, s);
    pool_free(tboxes, s);
  };
  if ((e = cudaMemsetAsync(bar.ptr, 0, sizeof(GridBarrier), s))) {
    drop();
    return cuda_rc(e);
  }
  auto kern = with_tris ? k_collapse<true> : k_collapse<false>;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  unsigned grid = (unsigned)(sm_count() * per_sm);
  const unsigned useful = (m_cap + kBlock - 1) / kBlock;
  if (grid > useful) grid = useful;
  if (grid < 1) grid = 1;
  CollapseParams p;
  p.nodes = nodes;
  p.node_count = node_count;
  p.cnt_e = cnt_e.ptr;
  p.mnodes = mnodes;
  p.m_total = m_cap;
  p.m_total_dev = mtot.ptr;
  p.queue[0] = q0.ptr;
  p.queue[1] = q1.ptr;
  p.qcount = qcount.ptr;
  p.bar = bar.ptr;
  p.status = status.ptr;
  if (with_tris) p.tri = *tri;
  p.ibox = ibox.ptr;
  p.escaped = status.ptr + 2;
  p.tboxes = tboxes;
  void* args[] = {&p};
  if ((e = cudaLaunchCooperativeKernel((void*)kern, dim3(grid), dim3(kBlock), args, 0, s))) {
    drop();
    return cuda_rc(e);
  }
  uint32_t st[4] = {0, 0, 0, 0};
  if ((e = cudaMemcpyAsync(st, status.ptr, 12, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(st + 3, mtot.ptr, 4, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s))) {
    drop();
    return cuda_rc(e);
  }
  if (st[0] != 0) {
    drop();
    return (st[0] & kStatusTimeout) ? Timeout : Error;
  }
  const uint32_t m_total = st[3];  // checked on the device: 1 .. m_cap
  *mnodes_out = mnodes;
  *mnode_count = m_total;
  if (with_tris && tri->tboxes_out) *tri->tboxes_out = tboxes;
  if (escaped_out) *escaped_out = st[2];
  return Ok;
}

}  // namespace rtbvh

namespace rtbvh {

ResultCode refit_bvh(DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                     uint32_t prim_count, const DAabb* aabbs, cudaStream_t s) {
  if (node_count == 0) return Ok;
  cudaError_t e;
  Scratch<uint32_t> parent, arrive, status;
  if ((e = parent.alloc(node_count, s)) || (e = arrive.alloc(node_count, s)) || (e = status.alloc(4, s)))
    return cuda_rc(e);
  if ((e = cudaMemsetAsync(parent.ptr, 0xff, (size_t)node_count * 4, s)) ||
      (e = cudaMemsetAsync(status.ptr, 0, 16, s)))
    return cuda_rc(e);
  const unsigned blocks = (node_count + kBlock - 1) / kBlock;
  k_parents<<<blocks, kBlock, 0, s>>>(nodes, node_count, parent.ptr, arrive.ptr, status.ptr);
  k_refit<<<blocks, kBlock, 0, s>>>(nodes, node_count, indices, index_count, prim_count, aabbs, parent.ptr,
                                    arrive.ptr, status.ptr);
  uint32_t st = 0;
  if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(&st, status.ptr, 4, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_rc(e);
  return st ? Error : Ok;
}

}  // namespace rtbvh

// ---------------------------------------------------------------- refit without allocation
// Variant of refit_bvh for callers that must not allocate device memory,
// for example a renderer that refits every frame inside a region where it
// is not allowed to call cudaMalloc (an allocation can synchronise the
// device and can fail mid-frame). Its scratch (parent pointers, arrival
// counters) lives in this file-scope array instead of being allocated per
// call; errors go to the Bvh's own status word. The array is reserved on a
// GPU when this module is first used there (with lazy module loading, at
// the latest on the first call) and stays reserved until the process exits.
namespace rtbvh {

namespace {

constexpr uint32_t kNoAllocHeadWords = 64;  // 256 bytes ahead of the arrays (unused), keeps them 256-byte aligned
static __device__ __align__(256) uint32_t g_refit_scratch[kNoAllocHeadWords + 2u * RTBVH_REFIT_NOALLOC_MAX_NODES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_refit_scratch on the current device, looked up once
// per device (with that device current) on its first use.
cudaError_t noalloc_scratch(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_refit_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace

ResultCode refit_bvh_noalloc(DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                             uint32_t prim_count, const DAabb* aabbs, uint32_t* status, cudaStream_t s) {
  if (node_count == 0) return Ok;
  if (node_count > RTBVH_REFIT_NOALLOC_MAX_NODES) return InvalidArgument;
  uint32_t* base = nullptr;
  cudaError_t e = noalloc_scratch(&base);
  if (e != cudaSuccess) return cuda_rc(e);
  uint32_t* parent = base + kNoAllocHeadWords;
  uint32_t* arrive = parent + RTBVH_REFIT_NOALLOC_MAX_NODES;
  // The array keeps the previous call's contents: reset what must start
  // clean (k_parents zeroes the arrival counters itself).
  if ((e = cudaMemsetAsync(parent, 0xff, (size_t)node_count * 4, s))) return cuda_rc(e);
  const unsigned blocks = (node_count + kBlock - 1) / kBlock;
  k_parents<<<blocks, kBlock, 0, s>>>(nodes, node_count, parent, arrive, status);
  k_refit<<<blocks, kBlock, 0, s>>>(nodes, node_count, indices, index_count, prim_count, aabbs, parent, arrive,
                                    status);
  return cuda_rc(cudaGetLastError());
}

}  // namespace rtbvh

namespace rtbvh {

cudaError_t launch_collapse_segments(const DAabb* nodes, uint32_t node_count, const uint32_t* prim_off,
                                     const uint32_t* order, uint32_t mesh_count, uint32_t* parent, uint32_t* arrive,
                                     uint32_t* cnt_e, uint32_t* cnt_o, uint32_t* mbase, uint2* q0, uint2* q1,
                                     DMNode* mnodes, uint32_t m_capacity, uint32_t* status, unsigned blocks,
                                     cudaStream_t s) {
  if (node_count == 0 || mesh_count == 0) return cudaSuccess;
  cudaError_t e;
  if ((e = cudaMemsetAsync(parent, 0xff, (size_t)node_count * 4, s))) return e;
  const unsigned nb = (node_count + kBlock - 1) / kBlock;
  k_parents<<<nb, kBlock, 0, s>>>(nodes, node_count, parent, arrive, status);
  k_counts_bottom_up<false><<<nb, kBlock, 0, s>>>(nodes, node_count, parent, arrive, cnt_e, cnt_o, MbvhTriangles(),
                                                  status);
  k_seg_mbase<<<1, 1024, 0, s>>>(nodes, cnt_e, prim_off, mesh_count, mbase);
  SegCollapseParams p;
  p.c.nodes = nodes;
  p.c.node_count = node_count;
  p.c.cnt_e = cnt_e;
  p.c.mnodes = mnodes;
  p.c.m_total = m_capacity;
  p.c.queue[0] = q0;
  p.c.queue[1] = q1;
  p.c.qcount = nullptr;
  p.c.bar = nullptr;
  p.c.status = status;
  p.c.ibox = nullptr;
  p.c.escaped = nullptr;
  p.c.tboxes = nullptr;
  p.c.m_total_dev = nullptr;
  p.prim_off = prim_off;
  p.order = order;
  p.mbase = mbase;
  p.queue[0] = q0;
  p.queue[1] = q1;
  p.mesh_count = mesh_count;
  k_collapse_segments<<<blocks, kBlock, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace rtbvh

// ---------------------------------------------------------------- compact quad nodes
namespace rtbvh {

namespace {

// One axis of a DQNode: grid start lo = the smallest bound of the four
// slots, step 2^k with 255 * 2^k covering the axis extent, lower bounds
// rounded down and upper bounds rounded up. The checks are exact: x - lo is
// split into hi + lo parts (two-sum, this file is compiled without
// contraction) and compared with q * 2^k, which is exact in float. False if a
// value is out of range or does not fit.
__device__ __forceinline__ void two_diff(float a, float b, float& hi, float& lo) {
  hi = a - b;
  const float bb = hi - a;
  lo = (a - (hi - bb)) + (-b - bb);
}

__device__ bool quantize_axis(const float* mn, const float* mx, float* lo_out, uint32_t* e_out, uint32_t* qlo,
                              uint32_t* qhi) {
  float lo = mn[0], hi = mn[0];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (!(fabsf(mn[i]) <= kQuantRange) || !(fabsf(mx[i]) <= kQuantRange)) return false;
    lo = fminf(lo, fminf(mn[i], mx[i]));
    hi = fmaxf(hi, fmaxf(mn[i], mx[i]));
  }
  int k = -126;
  const float ext = hi - lo;
  if (ext > 0.0f) {
    int ex;
    const float m = frexpf(ext / 255.0f, &ex);  // ext / 255 = m 2^ex, m in [0.5, 1)
    k = (m == 0.5f) ? ex - 1 : ex;
    if (k < -126) k = -126;
  }
  for (int attempt = 0; attempt < 3; ++attempt, ++k) {
    if (k > 127) return false;
    const float step = __uint_as_float((uint32_t)(k + 127) << 23);
    const float inv_step = (k <= 126) ? __uint_as_float((uint32_t)(127 - k) << 23) : 0.0f;
    if (k > 126 || k < -126) return false;
    uint32_t L = 0, H = 0;
    bool ok = true;
    for (int i = 0; i < 4 && ok; ++i) {
      float dh, dl;
      two_diff(mn[i], lo, dh, dl);  // mn - lo == dh + dl exactly
      float q = floorf(dh * inv_step);
      if (q < 0.0f) q = 0.0f;
      if (q > 255.0f) q = 255.0f;
      // need q * step <= dh + dl
      for (int g = 0; g < 4 && q > 0.0f; ++g) {
        const float v = q * step;
        if (v < dh || (v == dh && dl >= 0.0f)) break;
        q -= 1.0f;
      }
      {
        const float v = q * step;
        if (!(v < dh || (v == dh && dl >= 0.0f))) q = 0.0f;  // 0 is always below: lo is the minimum
      }
      const uint32_t ql = (uint32_t)q;
      two_diff(mx[i], lo, dh, dl);
      q = ceilf(dh * inv_step);
      if (q < 0.0f) q = 0.0f;
      // need q * step >= dh + dl
      for (int g = 0; g < 4; ++g) {
        const float v = q * step;
        if (v > dh || (v == dh && dl <= 0.0f)) break;
        q += 1.0f;
      }
      const float v = q * step;
      if (q > 255.0f || !(v > dh || (v == dh && dl <= 0.0f))) {
        ok = false;
      } else {
        L |= ql << (8 * i);
        H |= (uint32_t)q << (8 * i);
      }
    }
    if (ok) {
      *lo_out = lo;
      *e_out = (uint32_t)(k + 127);
      *qlo = L;
      *qhi = H;
      return true;
    }
  }
  return false;
}

__global__ void __launch_bounds__(kBlock) k_quantize(const DMNode* __restrict__ in, uint32_t count,
                                                      const uint32_t* __restrict__ live_count,
                                                      DQNode* __restrict__ out) {
  const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= count || (live_count && i >= __ldg(live_count))) return;
  const DMNode m = in[i];
  DQNode q;
  uint32_t ex = 0, ey = 0, ez = 0;
  bool ok = quantize_axis(m.min_x, m.max_x, &q.lo[0], &ex, &q.qx[0], &q.qx[1]) &&
            quantize_axis(m.min_y, m.max_y, &q.lo[1], &ey, &q.qy[0], &q.qy[1]) &&
            quantize_axis(m.min_z, m.max_z, &q.lo[2], &ez, &q.qz[0], &q.qz[1]);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    q.children[k] = m.children[k];
    ok = ok && m.counts[k] >= -32768 && m.counts[k] <= 32767;
    q.counts[k] = (int16_t)m.counts[k];
  }
  if (!ok) {
    q.lo[0] = q.lo[1] = q.lo[2] = 0.0f;
    q.qx[0] = q.qx[1] = q.qy[0] = q.qy[1] = q.qz[0] = q.qz[1] = 0u;
    ex = ey = ez = 0;
  }
  bool in_range = true;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    in_range = in_range && fabsf(m.min_x[k]) <= kCompactRange && fabsf(m.max_x[k]) <= kCompactRange &&
               fabsf(m.min_y[k]) <= kCompactRange && fabsf(m.max_y[k]) <= kCompactRange &&
               fabsf(m.min_z[k]) <= kCompactRange && fabsf(m.max_z[k]) <= kCompactRange;
  const uint32_t flags = (ok ? 0u : kQFlagExact) | (in_range ? 0u : kQFlagOutOfRange);
  q.exps = ex | (ey << 8) | (ez << 16) | (flags << 24);
  const float4* src = reinterpret_cast<const float4*>(&q);
  float4* dst = reinterpret_cast<float4*>(out + i);
#pragma unroll
  for (int k = 0; k < 4; ++k) dst[k] = src[k];
}

}  // namespace

cudaError_t launch_quantize_mbvh(const DMNode* mnodes, uint32_t count, DQNode* qnodes, cudaStream_t s,
                                 const uint32_t* live_count) {
  if (count == 0) return cudaSuccess;
  k_quantize<<<(count + kBlock - 1) / kBlock, kBlock, 0, s>>>(mnodes, count, live_count, qnodes);
  return cudaGetLastError();
}

}  // namespace rtbvh

// ---------------------------------------------------------------- traversal tree (4-wide, tight boxes)
// A second 4-wide collapse of the BVH2 for the closest-hit traversal: each
// node takes the two children of its BVH2 node and keeps opening the
// interior child of largest half area until it has four slots (every slot
// keeps its own BVH2 box; the reference Mbvh instead gives a leaf slot its
// parent's box and opens strictly by depth). The tree is an internal
// acceleration structure: its boxes contain every triangle of their
// subtrees, so a traversal over it finds the same nearest hit.
//
// BVH2s whose boxes need not contain their triangles (a binned-SAH build;
// triangles attached after the build) get the same collapse over boxes
// recomputed from the triangles (build_mbvh with MbvhTriangles computes
// them), and their escaped triangles -- those that lie outside a box the
// reference's Mbvh tests on the way to them -- are flagged (mark_escapes).
// A ray that hits an escaped triangle (t below its current nearest) leaves
// the walk and is traced again over the exact Mbvh. For every other ray the
// nearest hit equals the reference's: (1) the walk's nearest triangle T is
// not escaped, so every box the reference tests on the way to T contains
// T, and the reference reaches T unless it already holds a nearer hit; (2)
// a triangle T' nearer than T that the reference reaches lies inside the
// walk's boxes, so the walk reaches and hits T' too -- it would have kept
// T' (not escaped) or handed the ray on.
namespace rtbvh {

namespace {

struct WideParams {
  const DAabb* nodes;
  uint32_t node_count;
  DMNode* wnodes;
  uint32_t capacity;
  uint32_t* walloc;   // next free traversal-node index
  uint2* queue[2];
  uint32_t* qcount;   // 3 rotating counters
  GridBarrier* bar;
  uint32_t* status;
  // optional checks run before the launch: the tree is not collapsed when
  // check[0] != 0 (boxes that do not nest, or duplicate leaf slots) or,
  // with expect_seen != UINT32_MAX, when check[1] (primitives seen in
  // leaves) differs from it
  const uint32_t* check;
  uint32_t expect_seen;
};

// Traversal node wi from BVH2 node c. Interior slots get indices from
// *alloc (below alloc_end) and are appended to `next` (next_cap entries).
struct WideCtx {
  const DAabb* nodes;
  uint32_t node_count;
  DMNode* wnodes;
  uint32_t* alloc;
  uint32_t alloc_end;
  uint32_t next_cap;
  uint32_t* status;
};

// AGG: called by all lanes of a warp (`valid` false for lanes without an
// item), node indices and queue entries reserved once per warp.
template <bool AGG>
__device__ void emit_wide(const WideCtx& p, uint32_t c, uint32_t wi, uint2* next, uint32_t* next_count,
                          bool valid = true) {
  uint32_t slot[4];
  DAabb box[4];
  int ns = 0;
  bool ok = valid;
  const DAabb cur = load_aabb(p.nodes + c);
  if (!ok) {
  } else if (cur.count >= 0 || cur.left_first < 0) {
    slot[0] = c;
    box[0] = cur;
    ns = 1;
  } else if ((uint32_t)cur.left_first + 1u < p.node_count) {
    slot[0] = (uint32_t)cur.left_first;
    slot[1] = slot[0] + 1u;
    box[0] = load_aabb(p.nodes + slot[0]);
    box[1] = load_aabb(p.nodes + slot[1]);
    ns = 2;
    while (ns < 4) {
      int best = -1;
      float best_area = -1.0f;
      for (int i = 0; i < ns; ++i) {
        if (box[i].count >= 0 || box[i].left_first < 0) continue;
        const float a = half_area(box[i].min[0], box[i].min[1], box[i].min[2], box[i].max[0], box[i].max[1],
                                  box[i].max[2]);
        if (a > best_area) {
          best_area = a;
          best = i;
        }
      }
      if (best < 0) break;
      const uint32_t lf = (uint32_t)box[best].left_first;
      if (lf + 1u >= p.node_count) {
        atomicOr(p.status, kStatusBadIndex);
        break;
      }
      slot[best] = lf;
      box[best] = load_aabb(p.nodes + lf);
      slot[ns] = lf + 1u;
      box[ns] = load_aabb(p.nodes + lf + 1u);
      ++ns;
    }
  } else {
    atomicOr(p.status, kStatusBadIndex);
    ok = false;
  }
  uint32_t n_int = 0;
  if (ok)
    for (int i = 0; i < ns; ++i) n_int += (box[i].count < 0 && box[i].left_first >= 0) ? 1u : 0u;
  uint32_t base = 0, qbase = 0;
  if (AGG) {
    base = warp_reserve(p.alloc, n_int);
    qbase = warp_reserve(next_count, n_int);
  } else if (n_int) {
    base = atomicAdd(p.alloc, n_int);
    qbase = atomicAdd(next_count, n_int);
  }
  if (!ok) return;
  if (n_int && base + n_int > p.alloc_end) {
    atomicOr(p.status, kStatusBadIndex);
    return;
  }
  DMNode m;
  uint32_t k = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const DAabb& b = box[i < ns ? i : 0];
    m.min_x[i] = b.min[0]; m.min_y[i] = b.min[1]; m.min_z[i] = b.min[2];
    m.max_x[i] = b.max[0]; m.max_y[i] = b.max[1]; m.max_z[i] = b.max[2];
    if (i >= ns) {
      m.children[i] = -1;
      m.counts[i] = -1;
    } else if (b.count >= 0 || b.left_first < 0) {
      m.children[i] = b.left_first;
      m.counts[i] = b.count;
    } else {
      const uint32_t q = qbase + k;
      const uint32_t child = base + k++;
      m.children[i] = (int32_t)child;
      m.counts[i] = -1;
      if (q < p.next_cap) next[q] = make_uint2(slot[i], child);
      else atomicOr(p.status, kStatusBadIndex);
    }
  }
  float4* dst = reinterpret_cast<float4*>(p.wnodes + wi);
  const float4* src = reinterpret_cast<const float4*>(&m);
#pragma unroll
  for (int j = 0; j < 8; ++j) dst[j] = src[j];
}

__global__ void __launch_bounds__(kBlock) k_wide_collapse(WideParams p) {
  if (p.check) {  // the same words for every block: all return or none
    const uint32_t bad = __ldcg(p.check), seen = __ldcg(p.check + 1);
    if (bad || (p.expect_seen != kNone && seen != p.expect_seen)) return;
  }
  const uint32_t G = gridDim.x;
  const uint32_t tid = blockIdx.x * kBlock + threadIdx.x, nthreads = G * kBlock;
  WideCtx ctx;
  ctx.nodes = p.nodes;
  ctx.node_count = p.node_count;
  ctx.wnodes = p.wnodes;
  ctx.alloc = p.walloc;
  ctx.alloc_end = p.capacity;
  ctx.next_cap = p.capacity;
  ctx.status = p.status;
  for (uint32_t level = 0; level < p.capacity + 1; ++level) {
    uint32_t size = __ldcg(p.qcount + (level % 3));
    if (size == 0) break;
    if (size > p.capacity) size = p.capacity;  // only after a kStatusBadIndex
    const uint2* q = p.queue[level & 1];
    uint2* next = p.queue[(level + 1) & 1];
    uint32_t* next_count = p.qcount + ((level + 1) % 3);
    // warp-uniform loop: every lane takes part in the reservations
    for (uint32_t k0 = tid - (threadIdx.x & 31u); k0 < size; k0 += nthreads) {
      const uint32_t k = k0 + (threadIdx.x & 31u);
      const bool valid = k < size;
      const uint2 item = valid ? __ldcg(q + k) : make_uint2(0u, 0u);
      emit_wide<true>(ctx, item.x, item.y, next, next_count, valid);
    }
    if (tid == 0) p.qcount[(level + 2) % 3] = 0;
    if (!grid_sync(p.bar, G, p.status)) return;
  }
}

// Nesting check: every interior node's box contains both children's boxes.
// The traversal tree finds the nearest hit only if the boxes it reads
// contain their triangles, which holds for nested trees (leaf boxes are
// always built from their primitives). A binned-SAH tree can violate it:
// the reference sizes a left child's box from the bins before
// best_splits[axis].count, a primitive count, instead of the split bin
// (src/builders/binned_sah.rs), so the reference's own traversal can miss
// hits there, and only its exact node order reproduces them.
__global__ void __launch_bounds__(kBlock) k_check_nested(const DAabb* __restrict__ nodes, uint32_t node_count,
                                                          uint32_t* __restrict__ not_nested) {
  const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
  if (c >= node_count) return;
  const DAabb n = load_aabb(nodes + c);
  if (n.count >= 0 || n.left_first < 0) return;
  const uint32_t lf = (uint32_t)n.left_first;
  if (lf + 1u >= node_count) {
    atomicOr(not_nested, 1u);
    return;
  }
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const DAabb ch = load_aabb(nodes + lf + k);
#pragma unroll
    for (int a = 0; a < 3; ++a) ok = ok && ch.min[a] >= n.min[a] && ch.max[a] <= n.max[a];
  }
  if (!ok) atomicOr(not_nested, 1u);
}

// The leaves of the object-split builders hold every index slot once and
// every primitive once, so their boxes cover whole primitives. Spatial-split
// trees (several fragments of a triangle, fragment boxes, unused slots) do
// not: any of those sets *bad.
__global__ void __launch_bounds__(kBlock) k_check_leaves(const DAabb* __restrict__ nodes, uint32_t node_count,
                                                         const uint32_t* __restrict__ indices, uint32_t index_count,
                                                         uint32_t* __restrict__ seen, uint32_t* __restrict__ total,
                                                         uint32_t* __restrict__ bad) {
  const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
  if (c >= node_count) return;
  const DAabb n = load_aabb(nodes + c);
  if (n.count < 0 || n.left_first < 0) return;
  atomicAdd(total, (uint32_t)n.count);
  for (int32_t k = 0; k < n.count; ++k) {
    const uint32_t slot = (uint32_t)n.left_first + (uint32_t)k;
    if (slot >= index_count) {
      atomicOr(bad, 1u);
      return;
    }
    const uint32_t p = __ldg(indices + slot);
    if (p >= index_count || atomicAdd(seen + p, 1u) != 0u) {
      atomicOr(bad, 1u);
      return;
    }
  }
}

__global__ void k_wide_init(uint2* queue0, uint32_t* qcount, uint32_t* walloc) {
  if (threadIdx.x == 0) {
    queue0[0] = make_uint2(0u, 0u);
    qcount[0] = 1;
    qcount[1] = 0;
    qcount[2] = 0;
    *walloc = 1;
  }
}

// Many meshes: one block per mesh builds the mesh's traversal tree in the
// node range [off_m, off_m + n_m) (a mesh of n primitives has at most n - 1
// interior BVH2 nodes), root at off_m, with the frontier in the same range
// of the two queues.
__global__ void __launch_bounds__(kBlock)
    k_wide_segments(const DAabb* __restrict__ nodes, uint32_t node_count, const uint32_t* __restrict__ prim_off,
                    const uint32_t* __restrict__ order, uint32_t mesh_count, DMNode* wnodes, uint2* q0, uint2* q1,
                    uint32_t* status) {
  __shared__ uint32_t s_count[2];
  __shared__ uint32_t s_alloc;
  for (uint32_t q = blockIdx.x; q < mesh_count; q += gridDim.x) {
    const uint32_t m = order[q];
    const uint32_t off = prim_off[m], n = prim_off[m + 1] - off;
    if (n == 0) continue;
    WideCtx ctx;
    ctx.nodes = nodes;
    ctx.node_count = node_count;
    ctx.wnodes = wnodes;
    ctx.alloc = &s_alloc;
    ctx.alloc_end = off + n;
    ctx.next_cap = n;
    ctx.status = status;
    if (threadIdx.x == 0) {
      q0[off] = make_uint2(2u * off - m, off);
      s_count[0] = 1;
      s_count[1] = 0;
      s_alloc = off + 1u;
    }
    __syncthreads();
    int cur = 0;
    for (uint32_t level = 0; level <= n; ++level) {
      uint32_t size = s_count[cur];
      if (size == 0) break;
      if (size > n) size = n;
      const uint2* qin = (cur ? q1 : q0) + off;
      uint2* qout = (cur ? q0 : q1) + off;
      for (uint32_t k = threadIdx.x; k < size; k += kBlock) {
        const uint2 item = qin[k];
        emit_wide<false>(ctx, item.x, item.y, qout, &s_count[cur ^ 1]);
      }
      __syncthreads();
      if (threadIdx.x == 0) s_count[cur] = 0;
      __syncthreads();
      cur ^= 1;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_wide_segments(const DAabb* nodes, uint32_t node_count, const uint32_t* prim_off,
                                 const uint32_t* order, uint32_t mesh_count, uint32_t total_prims, DMNode* wnodes,
                                 DQNode* wq, uint2* q0, uint2* q1, uint32_t* status, unsigned blocks, cudaStream_t s) {
  if (mesh_count == 0 || total_prims == 0) return cudaSuccess;
  k_wide_segments<<<blocks, kBlock, 0, s>>>(nodes, node_count, prim_off, order, mesh_count, wnodes, q0, q1, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // slots of a mesh's range past its own tree are converted too and never read
  return launch_quantize_mbvh(wnodes, total_prims, wq, s);
}

ResultCode build_wide(const DAabb* nodes, uint32_t node_count, const uint32_t* indices, uint32_t index_count,
                      cudaStream_t s, DMNode** wnodes_out, DQNode** wq_out, uint32_t* wcount, bool nested) {
  *wnodes_out = nullptr;
  *wq_out = nullptr;
  *wcount = 0;
  if (node_count == 0) return Ok;
  // one traversal node per BVH2 interior node at most, or the root leaf
  const uint32_t capacity = node_count < 3u ? 1u : (node_count + 1u) / 2u;
  cudaError_t e;
  Scratch<uint32_t> status, qcount, walloc;
  Scratch<uint2> q0, q1;
  Scratch<GridBarrier> bar;
  if ((e = status.alloc(4, s)) || (e = qcount.alloc(4, s)) || (e = walloc.alloc(1, s)) || (e = q0.alloc(capacity, s)) ||
      (e = q1.alloc(capacity, s)) || (e = bar.alloc(1, s)))
    return cuda_rc(e);
  DMNode* wn = nullptr;
  DQNode* wq = nullptr;
  auto fail = [&](ResultCode rc) {
    pool_free(wn, s);
    pool_free(wq, s);
    return rc;
  };
  if ((e = device_alloc(&wn, capacity, s))) return fail(cuda_rc(e));
  if ((e = cudaMemsetAsync(status.ptr, 0, 16, s)) || (e = cudaMemsetAsync(bar.ptr, 0, sizeof(GridBarrier), s)))
    return fail(cuda_rc(e));
  const unsigned node_blocks = (node_count + kBlock - 1) / kBlock;
  // status[1]: not nested, or leaves that are not whole primitives once
  // each -> no traversal tree (closest hit uses the exact nodes); the
  // collapse reads the result on the device and does nothing then
  const bool checked = !nested || indices;
  Scratch<uint32_t> seen;
  if (checked) {
    if (!nested) k_check_nested<<<node_blocks, kBlock, 0, s>>>(nodes, node_count, status.ptr + 1);
    if (indices) {
      if ((e = seen.alloc(index_count, s)) || (e = cudaMemsetAsync(seen.ptr, 0, (size_t)index_count * 4, s)))
        return fail(cuda_rc(e));
      k_check_leaves<<<node_blocks, kBlock, 0, s>>>(nodes, node_count, indices, index_count, seen.ptr, status.ptr + 2,
                                                    status.ptr + 1);
    }
  }
  k_wide_init<<<1, 32, 0, s>>>(q0.ptr, qcount.ptr, walloc.ptr);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wide_collapse, kBlock, 0);
  if (per_sm < 1) per_sm = 1;
  unsigned grid = (unsigned)(sm_count() * per_sm);
  const unsigned useful = (capacity + kBlock - 1) / kBlock;
  if (grid > useful) grid = useful;
  if (grid < 1) grid = 1;
  WideParams p;
  p.nodes = nodes;
  p.node_count = node_count;
  p.wnodes = wn;
  p.capacity = capacity;
  p.walloc = walloc.ptr;
  p.queue[0] = q0.ptr;
  p.queue[1] = q1.ptr;
  p.qcount = qcount.ptr;
  p.bar = bar.ptr;
  p.status = status.ptr;
  p.check = checked ? status.ptr + 1 : nullptr;
  p.expect_seen = indices ? index_count : kNone;
  void* args[] = {&p};
  if ((e = cudaLaunchCooperativeKernel((void*)k_wide_collapse, dim3(grid), dim3(kBlock), args, 0, s)))
    return fail(cuda_rc(e));
  // compact nodes for the live part of the tree (the node count is read on
  // the device), then one readback for everything
  if ((e = device_alloc(&wq, capacity, s))) return fail(cuda_rc(e));
  if ((e = launch_quantize_mbvh(wn, capacity, wq, s, walloc.ptr))) return fail(cuda_rc(e));
  uint32_t h[4] = {0, 0, 0, 0};
  if ((e = cudaMemcpyAsync(h, walloc.ptr, 4, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaMemcpyAsync(h + 1, status.ptr, 12, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
    return fail(cuda_rc(e));
  if (checked && (h[2] || (indices && h[3] != index_count))) return fail(Ok);
  if (h[1] != 0) return fail((h[1] & kStatusTimeout) ? Timeout : Error);
  if (h[0] == 0 || h[0] > capacity) return fail(Error);
  *wnodes_out = wn;
  *wq_out = wq;
  *wcount = h[0];
  return Ok;
}

}  // namespace rtbvh
