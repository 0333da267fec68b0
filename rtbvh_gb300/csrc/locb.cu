// Locally-ordered clustering build (src/builders/locb.rs) on the GPU.
//
// Pipeline: primitive boxes -> world box (Aabb::union_of_list) -> 30-bit
// Morton codes of the centres -> stable radix sort -> leaves (sorted boxes
// + 1e-4) -> clustering levels until one node is left.
//
// The clustering levels above kTailNodes nodes run in ONE cooperative
// launch. A level of m nodes [begin, end) does, with a grid barrier after
// each phase:
//   A. for a contiguous chunk per block: the nearest neighbour of every
//      node inside the window [max(begin, i-14), min(end, i+15)) by the
//      half area of the union, first (lowest index) minimum wins -- boxes
//      staged in shared memory, the neighbours of a 14-node halo on either
//      side recomputed -- so the block knows its nodes' merge flags
//      (i < j, nb[j] == i) and counts them at once;
//   B. the prefix of the blocks' counts and the scatter of parents,
//      unmerged nodes (next level) and children (final node array).
// (The segmented builds of many meshes use the three-phase form of the
// same level: nn_tile, the flag count, scatter_tile.)
// Node positions follow the reference exactly (locb.rs:178-215), so the
// output is bit-identical to the reference's node array. Levels of at most
// kTailNodes nodes are finished by k_locb_tail: one block of 1024 threads
// with the whole level in shared memory and block barriers only.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 256;
constexpr int kRadius = 14;       // LocallyOrderedClusteringBuilder::search_radius
constexpr uint32_t kTailNodes = 2048;

struct LocbParams {
  DAabb* lvl[2];
  DAabb* final_nodes;
  uint32_t* nb;
  uint32_t* blocksum;
  GridBarrier* bar;
  uint32_t* status;
  uint32_t* info;  // levels run, then begin, end and level buffer of the first tail level
  uint32_t n;
};

struct SBox {
  float mn[3], mx[3];
};

__device__ __forceinline__ SBox to_sbox(const DAabb& a) {
  SBox b;
  b.mn[0] = a.min[0]; b.mn[1] = a.min[1]; b.mn[2] = a.min[2];
  b.mx[0] = a.max[0]; b.mx[1] = a.max[1]; b.mx[2] = a.max[2];
  return b;
}

// half_area(union(a, b)); only the comparison of these values matters, so
// native min/max are fine here (a -0/+0 difference cannot change an order).
__device__ __forceinline__ float union_half_area(const SBox& a, const SBox& b) {
  return half_area(fminf(a.mn[0], b.mn[0]), fminf(a.mn[1], b.mn[1]), fminf(a.mn[2], b.mn[2]),
                   fmaxf(a.mx[0], b.mx[0]), fmaxf(a.mx[1], b.mx[1]), fmaxf(a.mx[2], b.mx[2]));
}

// Merge flag of node i (locb.rs:159-167).
__device__ __forceinline__ uint32_t merge_flag(const uint32_t* nb, uint32_t i) {
  uint32_t j = __ldcg(nb + i);
  return (i < j && __ldcg(nb + j) == i) ? 1u : 0u;
}

// Phase 1 for the tile [t0, t0 + kBlock) of the level [begin, end).
__device__ void nn_tile(const DAabb* in, uint32_t* nb, uint32_t begin, uint32_t end, uint32_t t0, SBox* s_box,
                        uint32_t* status) {
  const int span = kBlock + 2 * kRadius;
  for (int k = threadIdx.x; k < span; k += kBlock) {
    int64_t idx = (int64_t)t0 - kRadius + k;
    if (idx >= (int64_t)begin && idx < (int64_t)end) s_box[k] = to_sbox(load_aabb_cg(in + idx));
  }
  __syncthreads();
  const uint32_t i = t0 + threadIdx.x;
  if (i < end) {
    const uint32_t sb = (i > begin + kRadius) ? i - kRadius : begin;
    const uint32_t se = min(i + kRadius + 1, end);
    const SBox bi = s_box[i - t0 + kRadius];
    float best = 3.40282347e+38f;
    int64_t best_j = -1;
    for (uint32_t j = sb; j < i; ++j) {
      float d = union_half_area(s_box[j - t0 + kRadius], bi);
      if (d < best) { best = d; best_j = j; }
    }
    for (uint32_t j = i + 1; j < se; ++j) {
      float d = union_half_area(bi, s_box[j - t0 + kRadius]);
      if (d < best) { best = d; best_j = j; }
    }
    if (best_j < 0) {
      atomicOr(status, kStatusNoNeighbour);
      best_j = i;
    }
    nb[i] = (uint32_t)best_j;
  }
  __syncthreads();
}

// Phase 3 for the sub-tile [s0, min(s0 + kBlock, c1)); `carry` is the number
// of merge flags before s0 in the level. Returns the carry for the next sub-tile.
__device__ uint32_t scatter_tile(const DAabb* in, DAabb* out, DAabb* final_nodes, const uint32_t* nb, uint32_t begin,
                                 uint32_t end, uint32_t s0, uint32_t c1, uint32_t carry, uint32_t mc,
                                 uint32_t* s_flag, uint32_t* s_warp, uint32_t* status) {
  for (int k = threadIdx.x; k < kBlock + kRadius; k += kBlock) {
    uint32_t idx = s0 + k;
    s_flag[k] = idx < end ? merge_flag(nb, idx) : 0u;
  }
  __syncthreads();
  const uint32_t i = s0 + threadIdx.x;
  uint32_t f = (i < c1) ? s_flag[threadIdx.x] : 0u;
  uint32_t tile_total;
  uint32_t incl = block_inclusive_scan<kBlock>(f, s_warp, &tile_total) + carry;
  const uint32_t unmerged_begin = begin - mc;
  const uint32_t children_begin = end - 2u * mc;
  if (i < c1) {
    const uint32_t j = __ldcg(nb + i);
    const uint32_t merged_i = incl;
    if (__ldcg(nb + j) == i) {
      if (i < j) {
        uint32_t merged_j = merged_i;
        for (uint32_t k = i + 1; k <= j; ++k) merged_j += s_flag[k - s0];
        const uint32_t pos = unmerged_begin + j - begin - merged_j;
        const uint32_t fc = children_begin + (merged_i - 1u) * 2u;
        DAabb a = load_aabb_cg(in + i), b = load_aabb_cg(in + j);
        DAabb p;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          p.min[ax] = rs_min(b.min[ax], a.min[ax]);
          p.max[ax] = rs_max(b.max[ax], a.max[ax]);
        }
        p.count = -1;
        p.left_first = (int32_t)fc;
        if (pos < end && fc + 1 < end) {
          store_aabb(out + pos, p);
          store_aabb(final_nodes + fc, a);
          store_aabb(final_nodes + fc + 1, b);
        } else {
          atomicOr(status, kStatusBadIndex);
        }
      }
    } else {
      const uint32_t pos = unmerged_begin + i - begin - merged_i;
      if (pos < end) store_aabb(out + pos, load_aabb_cg(in + i));
      else atomicOr(status, kStatusBadIndex);
    }
  }
  __syncthreads();
  return carry + tile_total;
}

// Clustering levels of the range [begin, end) run by one block (block
// barriers only) until one node is left, which is stored at final[begin].
// Returns false (status set) on a level without a merge.
__device__ bool locb_block_finish(DAabb* const lvl[2], DAabb* final_nodes, uint32_t* nb, uint32_t& begin,
                                  uint32_t& end, int& cur, uint32_t& levels, SBox* s_box, uint32_t* s_flag,
                                  uint32_t* s_warp, uint32_t* status) {
  while (end - begin > 1) {
    const DAabb* in = lvl[cur];
    DAabb* out = lvl[cur ^ 1];
    for (uint32_t t0 = begin; t0 < end; t0 += kBlock) nn_tile(in, nb, begin, end, t0, s_box, status);
    __threadfence_block();
    __syncthreads();
    uint32_t local = 0;
    for (uint32_t i = begin + threadIdx.x; i < end; i += kBlock) local += merge_flag(nb, i);
    uint32_t mc;
    block_inclusive_scan<kBlock>(local, s_warp, &mc);
    if (mc == 0) {
      if (threadIdx.x == 0) atomicOr(status, kStatusNoMerge);
      return false;
    }
    uint32_t carry = 0;
    for (uint32_t s0 = begin; s0 < end; s0 += kBlock)
      carry = scatter_tile(in, out, final_nodes, nb, begin, end, s0, end, carry, mc, s_flag, s_warp, status);
    __threadfence_block();
    __syncthreads();
    begin -= mc;
    end -= 2u * mc;
    cur ^= 1;
    ++levels;
  }
  if (threadIdx.x == 0) store_aabb(final_nodes + begin, load_aabb_cg(lvl[cur] + begin));
  __syncthreads();
  return true;
}

// Merge state of node i of a wide level, kept in the top bits of its nb word
// (neighbour indices are below 2^30): kPairHead when i < nb[i] and
// nb[nb[i]] == i (i heads a merged pair: the merge flag of locb.rs:159-167),
// kPairTail when nb[i] < i and nb[nb[i]] == i.
constexpr uint32_t kPairHead = 1u << 30;
constexpr uint32_t kPairTail = 2u << 30;
constexpr uint32_t kNbMask = (1u << 30) - 1u;
constexpr int kHalo = 2 * kRadius;  // boxes a sub-tile stages on each side

// Phase A for the sub-tile [s0, s1) of a block's chunk of the level
// [begin, end): the nearest neighbours of the nodes [s0 - 14, s1 + 14) --
// the sub-tile and the halo its merge states depend on, with nn_tile's
// window and tie rule; the boxes [s0 - 28, s1 + 28) staged in shared
// memory -- then each sub-tile node's neighbour and merge state go to nb.
// Returns the thread's count of pair heads.
__device__ uint32_t nn_state_tile(const DAabb* in, uint32_t* nb, uint32_t begin, uint32_t end, uint32_t s0,
                                  uint32_t s1, SBox* s_box, uint16_t* s_nb, uint32_t* status) {
  const int64_t base = (int64_t)s0 - kHalo;  // s_box[k] holds node base + k
  const int span = kBlock + 2 * kHalo;
  for (int k = threadIdx.x; k < span; k += kBlock) {
    const int64_t idx = base + k;
    if (idx >= (int64_t)begin && idx < (int64_t)end) s_box[k] = to_sbox(load_aabb_cg(in + idx));
  }
  __syncthreads();
  // nodes [n0, n1): s_nb[x - (s0 - 14)] = neighbour of x, as an index into s_box
  const uint32_t n0 = s0 > begin + kRadius ? s0 - kRadius : begin;
  const uint32_t n1 = min(s1 + kRadius, end);
  for (uint32_t x = n0 + threadIdx.x; x < n1; x += kBlock) {
    const uint32_t sb = (x > begin + kRadius) ? x - kRadius : begin;
    const uint32_t se = min(x + kRadius + 1, end);
    const SBox bx = s_box[x - base];
    float best = 3.40282347e+38f;
    int64_t best_j = -1;
    for (uint32_t j = sb; j < x; ++j) {
      const float d = union_half_area(s_box[j - base], bx);
      if (d < best) { best = d; best_j = j; }
    }
    for (uint32_t j = x + 1; j < se; ++j) {
      const float d = union_half_area(bx, s_box[j - base]);
      if (d < best) { best = d; best_j = j; }
    }
    if (best_j < 0) {
      atomicOr(status, kStatusNoNeighbour);
      best_j = x;
    }
    s_nb[x - (s0 - kRadius)] = (uint16_t)(best_j - base);
  }
  __syncthreads();
  uint32_t heads = 0;
  const uint32_t i = s0 + threadIdx.x;
  if (i < s1) {
    const int64_t rel = (int64_t)s0 - kRadius - base;  // s_nb index of node v: v - base - rel
    const uint32_t j = (uint32_t)(base + s_nb[i - base - rel]);
    const uint32_t jj = (uint32_t)(base + s_nb[j - base - rel]);
    uint32_t state = 0;
    if (jj == i && i < j) state = kPairHead;
    else if (jj == i && j < i) state = kPairTail;
    nb[i] = j | state;
    heads = state == kPairHead ? 1u : 0u;
  }
  __syncthreads();
  return heads;
}

// Phase B for the sub-tile [s0, s1): the prefix of the pair heads (carry:
// heads before s0 in the level) and the placement of scatter_tile, from the
// nb words phase A left (heads up to 14 nodes past s1 may belong to the next
// block's chunk). Returns the carry for the next sub-tile.
__device__ uint32_t place_tile(const DAabb* in, DAabb* out, DAabb* final_nodes, const uint32_t* nb, uint32_t begin,
                               uint32_t end, uint32_t s0, uint32_t s1, uint32_t carry, uint32_t mc, uint32_t* s_word,
                               uint32_t* s_warp, uint32_t* status) {
  for (int k = threadIdx.x; k < kBlock + kRadius; k += kBlock) {
    const uint32_t idx = s0 + k;
    s_word[k] = idx < end ? __ldcg(nb + idx) : 0u;
  }
  __syncthreads();
  const uint32_t i = s0 + threadIdx.x;
  const uint32_t w = i < s1 ? s_word[threadIdx.x] : 0u;
  uint32_t tile_total;
  const uint32_t incl = block_inclusive_scan<kBlock>((w & kPairHead) ? 1u : 0u, s_warp, &tile_total) + carry;
  const uint32_t unmerged_begin = begin - mc;
  const uint32_t children_begin = end - 2u * mc;
  if (i < s1) {
    const uint32_t merged_i = incl;
    if (w & kPairHead) {
      const uint32_t j = w & kNbMask;
      uint32_t merged_j = merged_i;
      for (uint32_t k = i + 1; k <= j; ++k) merged_j += (s_word[k - s0] & kPairHead) ? 1u : 0u;
      const uint32_t pos = unmerged_begin + j - begin - merged_j;
      const uint32_t fc = children_begin + (merged_i - 1u) * 2u;
      const DAabb a = load_aabb_cg(in + i), b = load_aabb_cg(in + j);
      DAabb par;
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        par.min[ax] = rs_min(b.min[ax], a.min[ax]);
        par.max[ax] = rs_max(b.max[ax], a.max[ax]);
      }
      par.count = -1;
      par.left_first = (int32_t)fc;
      if (j < end && pos < end && fc + 1 < end) {
        store_aabb(out + pos, par);
        store_aabb(final_nodes + fc, a);
        store_aabb(final_nodes + fc + 1, b);
      } else {
        atomicOr(status, kStatusBadIndex);
      }
    } else if (!(w & kPairTail)) {
      const uint32_t pos = unmerged_begin + i - begin - merged_i;
      if (pos < end) store_aabb(out + pos, load_aabb_cg(in + i));
      else atomicOr(status, kStatusBadIndex);
    }
  }
  __syncthreads();
  return carry + tile_total;
}

// The clustering levels above kTailNodes nodes. Per level, two phases with
// a grid barrier after each: (A) every block takes a contiguous chunk of
// the level and computes the nearest neighbours of its nodes and of a
// 14-node halo on either side (the halo is recomputed, not waited for), so
// it knows its nodes' merge states and counts its pair heads at once; (B)
// the prefix of the blocks' counts and the placement of parents, unmerged
// nodes and children (locb.rs:178-215).
__global__ void __launch_bounds__(kBlock) k_locb_levels(LocbParams p) {
  __shared__ SBox s_box[kBlock + 2 * kHalo];
  __shared__ uint16_t s_nb[kBlock + 2 * kRadius];
  __shared__ uint32_t s_word[kBlock + kRadius];
  __shared__ uint32_t s_warp[kBlock / 32];
  const uint32_t node_count = 2u * p.n - 1u;
  uint32_t begin = p.n - 1u, end = node_count;
  int cur = 0;
  const uint32_t G = gridDim.x;
  uint32_t levels = 0;

  // ---------------------------------------------------------------- wide levels
  while (end - begin > kTailNodes) {
    const uint32_t m = end - begin;
    const DAabb* in = p.lvl[cur];
    DAabb* out = p.lvl[cur ^ 1];
    const uint32_t chunk = (m + G - 1) / G;
    const uint32_t c0 = min(begin + blockIdx.x * chunk, end);
    const uint32_t c1 = min(c0 + chunk, end);
    uint32_t local = 0;
    for (uint32_t s0 = c0; s0 < c1; s0 += kBlock)
      local += nn_state_tile(in, p.nb, begin, end, s0, min(s0 + kBlock, c1), s_box, s_nb, p.status);
    uint32_t tot;
    block_inclusive_scan<kBlock>(local, s_warp, &tot);
    if (threadIdx.x == 0) p.blocksum[blockIdx.x] = tot;
    if (!grid_sync(p.bar, G, p.status)) return;

    uint32_t pre = 0, all = 0;
    for (uint32_t b = threadIdx.x; b < G; b += kBlock) {
      uint32_t v = __ldcg(p.blocksum + b);
      all += v;
      if (b < blockIdx.x) pre += v;
    }
    uint32_t pre_tot, all_tot;
    block_inclusive_scan<kBlock>(pre, s_warp, &pre_tot);
    block_inclusive_scan<kBlock>(all, s_warp, &all_tot);
    const uint32_t mc = all_tot;
    if (mc == 0) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(p.status, kStatusNoMerge);
      return;
    }
    uint32_t carry = pre_tot;
    for (uint32_t s0 = c0; s0 < c1; s0 += kBlock)
      carry = place_tile(in, out, p.final_nodes, p.nb, begin, end, s0, min(s0 + kBlock, c1), carry, mc, s_word,
                         s_warp, p.status);
    if (!grid_sync(p.bar, G, p.status)) return;
    begin -= mc;
    end -= 2u * mc;
    cur ^= 1;
    ++levels;
  }

  // the last kTailNodes nodes: k_locb_tail
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.info[0] = levels;
    p.info[1] = begin;
    p.info[2] = end;
    p.info[3] = (uint32_t)cur;
  }
}

// The clustering levels of the last kTailNodes (or fewer) nodes in ONE block
// of kTailBlock threads, the whole level held in shared memory: per level the
// nearest neighbours, the merge flags and their prefix, and the placement of
// parents (next level, shared memory) and children (final node array) with
// the arithmetic of nn_tile / scatter_tile, so the nodes are the same bits.
// The level comes from p.info (written by k_locb_levels) or, for builds with
// no wide level, from the arguments.
constexpr int kTailBlock = 1024;
constexpr size_t kTailSmem = 2 * kTailNodes * sizeof(DAabb) + 2 * kTailNodes * sizeof(uint32_t);

__global__ void __launch_bounds__(kTailBlock) k_locb_tail(LocbParams p, bool from_info, uint32_t begin0,
                                                          uint32_t end0) {
  extern __shared__ __align__(16) unsigned char tail_smem[];
  __shared__ uint32_t s_warp[kTailBlock / 32];
  DAabb* x = reinterpret_cast<DAabb*>(tail_smem);
  DAabb* y = x + kTailNodes;
  uint32_t* s_nb = reinterpret_cast<uint32_t*>(y + kTailNodes);
  uint32_t* s_incl = s_nb + kTailNodes;
  const uint32_t tid = threadIdx.x;
  uint32_t levels = from_info ? __ldcg(p.info) : 0u;
  uint32_t begin = from_info ? __ldcg(p.info + 1) : begin0;
  uint32_t end = from_info ? __ldcg(p.info + 2) : end0;
  const int cur = from_info ? (int)__ldcg(p.info + 3) : 0;
  if (end <= begin || end - begin > kTailNodes || end > 2u * p.n - 1u || (cur != 0 && cur != 1)) {
    if (tid == 0) atomicOr(p.status, kStatusBadIndex);
    return;
  }
  for (uint32_t i = tid; i < end - begin; i += kTailBlock) x[i] = load_aabb_cg(p.lvl[cur] + begin + i);
  __syncthreads();
  while (end - begin > 1) {
    const uint32_t m = end - begin;
    // 1. nearest neighbour in [max(0, i - 14), min(m, i + 15)), first minimum wins
    for (uint32_t i = tid; i < m; i += kTailBlock) {
      const uint32_t sb = i > (uint32_t)kRadius ? i - kRadius : 0u;
      const uint32_t se = min(i + kRadius + 1, m);
      const SBox bi = to_sbox(x[i]);
      float best = 3.40282347e+38f;
      int32_t best_j = -1;
      for (uint32_t j = sb; j < i; ++j) {
        const float d = union_half_area(to_sbox(x[j]), bi);
        if (d < best) { best = d; best_j = (int32_t)j; }
      }
      for (uint32_t j = i + 1; j < se; ++j) {
        const float d = union_half_area(bi, to_sbox(x[j]));
        if (d < best) { best = d; best_j = (int32_t)j; }
      }
      if (best_j < 0) {
        atomicOr(p.status, kStatusNoNeighbour);
        best_j = (int32_t)i;
      }
      s_nb[i] = (uint32_t)best_j;
    }
    __syncthreads();
    // 2. merge flags (i < j, nb[j] == i) and their inclusive prefix, two per thread
    const uint32_t i0 = 2u * tid, i1 = i0 + 1u;
    const uint32_t f0 = (i0 < m && i0 < s_nb[i0] && s_nb[s_nb[i0]] == i0) ? 1u : 0u;
    const uint32_t f1 = (i1 < m && i1 < s_nb[i1] && s_nb[s_nb[i1]] == i1) ? 1u : 0u;
    uint32_t mc;
    const uint32_t incl = block_inclusive_scan<kTailBlock>(f0 + f1, s_warp, &mc);
    if (i0 < m) s_incl[i0] = incl - f1;
    if (i1 < m) s_incl[i1] = incl;
    if (mc == 0) {
      if (tid == 0) atomicOr(p.status, kStatusNoMerge);
      return;  // block-uniform
    }
    __syncthreads();
    // 3. parents of merged pairs and unmerged nodes to the next level (begin - mc ...),
    //    merged pairs' children to the final node array (locb.rs:178-215)
    const uint32_t unmerged_begin = begin - mc, children_begin = end - 2u * mc;
    for (uint32_t i = tid; i < m; i += kTailBlock) {
      const uint32_t j = s_nb[i];
      const uint32_t merged_i = s_incl[i];
      if (s_nb[j] == i) {
        if (i < j) {
          const uint32_t pos = unmerged_begin + j - s_incl[j];
          const uint32_t fc = children_begin + (merged_i - 1u) * 2u;
          const DAabb a = x[i], b = x[j];
          DAabb par;
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) {
            par.min[ax] = rs_min(b.min[ax], a.min[ax]);
            par.max[ax] = rs_max(b.max[ax], a.max[ax]);
          }
          par.count = -1;
          par.left_first = (int32_t)fc;
          if (pos >= unmerged_begin && pos < end - 2u * mc && fc + 1 < end) {
            y[pos - unmerged_begin] = par;
            store_aabb(p.final_nodes + fc, a);
            store_aabb(p.final_nodes + fc + 1, b);
          } else {
            atomicOr(p.status, kStatusBadIndex);
          }
        }
      } else {
        const uint32_t pos = unmerged_begin + i - merged_i;
        if (pos >= unmerged_begin && pos < end - 2u * mc) y[pos - unmerged_begin] = x[i];
        else atomicOr(p.status, kStatusBadIndex);
      }
    }
    __syncthreads();
    DAabb* t = x;
    x = y;
    y = t;
    begin -= mc;
    end -= 2u * mc;
    ++levels;
  }
  if (tid == 0) {
    store_aabb(p.final_nodes + begin, x[0]);
    p.info[0] = levels;
    p.info[1] = begin;
  }
}

// Leaves: sorted boxes + 1e-4, count 1, left_first = i (locb.rs:289-294).
__global__ void __launch_bounds__(kBlock)
    k_locb_leaves(const DAabb* __restrict__ aabbs, const uint32_t* __restrict__ sorted, uint32_t n,
                  DAabb* __restrict__ lvl) {
  uint32_t i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= n) return;
  DAabb b = load_aabb(aabbs + __ldg(sorted + i));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b.min[a] = b.min[a] - 0.0001f;
    b.max[a] = b.max[a] + 0.0001f;
  }
  b.count = 1;
  b.left_first = (int32_t)i;
  store_aabb(lvl + (n - 1u) + i, b);
}

// n <= 2: one root leaf holding the world box (locb.rs:258-269).
__global__ void k_locb_single(const DAabb* world, uint32_t n, DAabb* nodes, uint32_t* indices) {
  if (threadIdx.x == 0) {
    DAabb w = *world;
    w.count = (int32_t)n;
    w.left_first = 0;
    store_aabb(nodes, w);
  }
  if (threadIdx.x < n) indices[threadIdx.x] = threadIdx.x;
}


// ---------------------------------------------------------------- many meshes
// One block per mesh clusters the mesh's own node range of a concatenated
// forest. Mesh m owns primitives [off_m, off_m + n_m) and nodes
// [2 off_m - m, 2 off_m - m + 2 n_m - 1); the placement arithmetic of a level
// depends only on differences of indices, so every node, left_first and
// leaf offset comes out as the single-mesh build's shifted by the mesh's
// offsets.
struct SegParams {
  DAabb* lvl[2];
  DAabb* final_nodes;
  uint32_t* nb;
  const uint32_t* prim_off;   // mesh_count + 1
  const uint32_t* order;      // meshes in processing order (largest first)
  const DAabb* worlds;        // per-mesh union_of_list boxes
  uint32_t* indices;          // sorted primitive indices (global); identity for n <= 2
  uint32_t* status;
  uint32_t mesh_count;
};

__global__ void __launch_bounds__(kBlock) k_locb_segments(SegParams p, uint32_t first) {
  __shared__ SBox s_box[kBlock + 2 * kRadius];
  __shared__ uint32_t s_flag[kBlock + kRadius];
  __shared__ uint32_t s_warp[kBlock / 32];
  for (uint32_t q = first + blockIdx.x; q < p.mesh_count; q += gridDim.x) {
    const uint32_t m = p.order[q];
    const uint32_t off = p.prim_off[m], n = p.prim_off[m + 1] - off;
    if (n == 0) continue;
    const uint32_t nbase = 2u * off - m;
    if (n <= 2) {
      if (threadIdx.x == 0) {
        DAabb w = p.worlds[m];
        w.count = (int32_t)n;
        w.left_first = (int32_t)off;
        store_aabb(p.final_nodes + nbase, w);
      }
      if (threadIdx.x < n) p.indices[off + threadIdx.x] = off + threadIdx.x;
      continue;
    }
    uint32_t begin = nbase + n - 1u, end = nbase + 2u * n - 1u, levels = 0;
    int cur = 0;
    if (!locb_block_finish(p.lvl, p.final_nodes, p.nb, begin, end, cur, levels, s_box, s_flag, s_warp, p.status))
      return;
  }
}

// Large meshes: a cluster of kSegCluster blocks per mesh runs the wide
// levels of k_locb_levels (tiles and chunks split over the cluster's
// blocks, hardware cluster barriers between the phases) and block rank 0
// finishes the last kTailNodes nodes alone. Every block of a cluster runs
// the same mesh sequence and the same level count (all loop bounds are
// computed from values every block reads identically), so each barrier is
// reached by all of them; nothing waits on another cluster.
__device__ __forceinline__ void cluster_barrier() {
  __threadfence();
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__global__ void __cluster_dims__(kSegCluster, 1, 1) __launch_bounds__(kBlock)
    k_locb_segments_cluster(SegParams p, uint32_t* cluster_sums, uint32_t big_count) {
  __shared__ SBox s_box[kBlock + 2 * kRadius];
  __shared__ uint32_t s_flag[kBlock + kRadius];
  __shared__ uint32_t s_warp[kBlock / 32];
  const uint32_t rank = blockIdx.x % kSegCluster;  // 1-D clusters of consecutive blocks
  const uint32_t cid = blockIdx.x / kSegCluster, ncl = gridDim.x / kSegCluster;
  uint32_t* sums = cluster_sums + (size_t)cid * kSegCluster;
  for (uint32_t q = cid; q < big_count; q += ncl) {
    const uint32_t m = p.order[q];
    const uint32_t off = p.prim_off[m], n = p.prim_off[m + 1] - off;
    if (n <= 2) continue;  // the host sends only meshes above kSegClusterMinPrims
    const uint32_t nbase = 2u * off - m;
    uint32_t begin = nbase + n - 1u, end = nbase + 2u * n - 1u, levels = 0;
    int cur = 0;
    bool ok = true;
    while (end - begin > kTailNodes) {
      const uint32_t count = end - begin;
      const DAabb* in = p.lvl[cur];
      DAabb* out = p.lvl[cur ^ 1];
      for (uint32_t tile = rank; (size_t)tile * kBlock < count; tile += kSegCluster)
        nn_tile(in, p.nb, begin, end, begin + tile * kBlock, s_box, p.status);
      cluster_barrier();
      const uint32_t chunk = (count + kSegCluster - 1) / kSegCluster;
      const uint32_t c0 = min(begin + rank * chunk, end);
      const uint32_t c1 = min(c0 + chunk, end);
      uint32_t local = 0;
      for (uint32_t i = c0 + threadIdx.x; i < c1; i += kBlock) local += merge_flag(p.nb, i);
      uint32_t tot;
      block_inclusive_scan<kBlock>(local, s_warp, &tot);
      if (threadIdx.x == 0) sums[rank] = tot;
      cluster_barrier();
      uint32_t pre = 0, mc = 0;
#pragma unroll
      for (uint32_t b = 0; b < kSegCluster; ++b) {
        const uint32_t v = __ldcg(sums + b);
        mc += v;
        if (b < rank) pre += v;
      }
      if (mc == 0) {  // same value in every block of the cluster
        if (rank == 0 && threadIdx.x == 0) atomicOr(p.status, kStatusNoMerge);
        ok = false;
        break;
      }
      uint32_t carry = pre;
      for (uint32_t s0 = c0; s0 < c1; s0 += kBlock)
        carry = scatter_tile(in, out, p.final_nodes, p.nb, begin, end, s0, c1, carry, mc, s_flag, s_warp, p.status);
      cluster_barrier();
      begin -= mc;
      end -= 2u * mc;
      cur ^= 1;
      ++levels;
    }
    if (ok && rank == 0)
      locb_block_finish(p.lvl, p.final_nodes, p.nb, begin, end, cur, levels, s_box, s_flag, s_warp, p.status);
  }
}

// Leaves of every mesh: sorted position k of mesh m (off_m <= k < off_m + n_m)
// becomes node 2 off_m - m + n_m - 1 + (k - off_m) with the primitive's box
// + 1e-4, count 1, left_first = k.
__global__ void __launch_bounds__(kBlock)
    k_locb_segment_leaves(const DAabb* __restrict__ aabbs, const uint32_t* __restrict__ sorted,
                          const uint32_t* __restrict__ prim_off, uint32_t mesh_count, uint32_t total,
                          DAabb* __restrict__ lvl) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= total) return;
  uint32_t lo = 0, hi = mesh_count;  // mesh with prim_off[m] <= k < prim_off[m + 1]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(prim_off + mid) <= k) lo = mid;
    else hi = mid;
  }
  const uint32_t m = lo, off = __ldg(prim_off + m), n = __ldg(prim_off + m + 1) - off;
  if (n <= 2) return;
  DAabb b = load_aabb(aabbs + __ldg(sorted + k));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b.min[a] = b.min[a] - 0.0001f;
    b.max[a] = b.max[a] + 0.0001f;
  }
  b.count = 1;
  b.left_first = (int32_t)k;
  store_aabb(lvl + (2u * off - m) + (n - 1u) + (k - off), b);
}

}  // namespace

ResultCode build_locb(const DAabb* aabbs, const float4* centers, size_t n_, cudaStream_t s, BuildOutput* out) {
  if (n_ == 0) return NoPrimitives;
  if (n_ >= (1u << 30)) return InvalidArgument;
  const uint32_t n = (uint32_t)n_;
  const uint32_t node_count = n <= 2 ? 1u : 2u * n - 1u;
  cudaError_t e;
  DAabb* nodes = nullptr;
  uint32_t* indices = nullptr;
  if ((e = device_alloc(&nodes, node_count, s)) != cudaSuccess) return cuda_rc(e);
  if ((e = device_alloc(&indices, n, s)) != cudaSuccess) {
    pool_free(nodes, s);
    return cuda_rc(e);
  }
  auto fail = [&](ResultCode rc) {
    pool_free(nodes, s);
    pool_free(indices, s);
    return rc;
  };
  Scratch<DAabb> world;
  Scratch<uint32_t> acc, status;
  if ((e = world.alloc(1, s)) || (e = acc.alloc(8, s)) || (e = status.alloc(4, s))) return fail(cuda_rc(e));
  if ((e = cudaMemsetAsync(status.ptr, 0, 16, s))) return fail(cuda_rc(e));
  if ((e = launch_world_bounds(aabbs, n, world.ptr, acc.ptr, s))) return fail(cuda_rc(e));
  if (n <= 2) {
    k_locb_single<<<1, 32, 0, s>>>(world.ptr, n, nodes, indices);
    if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(s))) return fail(cuda_rc(e));
    out->nodes = nodes;
    out->indices = indices;
    out->node_count = 1;
    return Ok;
  }
  Scratch<uint32_t> keys;
  Scratch<char> sort_temp;
  const size_t sort_bytes = radix_sort_temp_bytes(n);
  if ((e = keys.alloc(n, s)) || (e = sort_temp.alloc(sort_bytes, s))) return fail(cuda_rc(e));
  if ((e = launch_morton(centers, n, world.ptr, keys.ptr, indices, s))) return fail(cuda_rc(e));
  if ((e = radix_sort_pairs(keys.ptr, indices, n, 30, sort_temp.ptr, sort_bytes, status.ptr, s)))
    return fail(cuda_rc(e));

  Scratch<DAabb> lvl0, lvl1;
  Scratch<uint32_t> nb, blocksum, info;
  Scratch<GridBarrier> bar;
  if ((e = lvl0.alloc(node_count, s)) || (e = lvl1.alloc(node_count, s)) || (e = nb.alloc(node_count, s)) ||
      (e = info.alloc(4, s)) || (e = bar.alloc(1, s)))
    return fail(cuda_rc(e));
  k_locb_leaves<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(aabbs, indices, n, lvl0.ptr);
  if ((e = cudaGetLastError())) return fail(cuda_rc(e));

  int dev = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_locb_levels, kBlock, 0);
  if (per_sm < 1) return fail(DeviceError);
  // at most 3 blocks per SM: fewer blocks make the grid barriers between
  // clustering levels cheaper (1.394 against 1.423 ms on 1M triangles at
  // the occupancy limit; 1 block per SM is slower, 1.74 ms)
  if (per_sm > 3) per_sm = 3;
  unsigned grid = (unsigned)(sm_count() * per_sm);
  const unsigned useful = (unsigned)((n + kBlock - 1) / kBlock);
  if (grid > useful) grid = useful;
  if (grid < 1) grid = 1;
  if ((e = blocksum.alloc(grid, s)) || (e = cudaMemsetAsync(bar.ptr, 0, sizeof(GridBarrier), s)))
    return fail(cuda_rc(e));

  if ((e = cudaMemsetAsync(info.ptr, 0, 4 * sizeof(uint32_t), s))) return fail(cuda_rc(e));
  LocbParams p;
  p.lvl[0] = lvl0.ptr;
  p.lvl[1] = lvl1.ptr;
  p.final_nodes = nodes;
  p.nb = nb.ptr;
  p.blocksum = blocksum.ptr;
  p.bar = bar.ptr;
  p.status = status.ptr;
  p.info = info.ptr;
  p.n = n;
  const bool wide = n > kTailNodes;  // levels above kTailNodes nodes in the cooperative launch
  if (wide) {
    void* args[] = {&p};
    if ((e = cudaLaunchCooperativeKernel((void*)k_locb_levels, dim3(grid), dim3(kBlock), args, 0, s)))
      return fail(cuda_rc(e));
  }
  static std::once_flag tail_attr;
  std::call_once(tail_attr, [] {
    cudaFuncSetAttribute(k_locb_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTailSmem);
  });
  k_locb_tail<<<1, kTailBlock, kTailSmem, s>>>(p, wide, n - 1u, node_count);
  if ((e = cudaGetLastError())) return fail(cuda_rc(e));
  uint32_t h_status = 0;
  if ((e = cudaMemcpyAsync(&h_status, status.ptr, 4, cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return fail(cuda_rc(e));
  if (h_status & kStatusTimeout) return fail(Timeout);
  if (h_status) return fail(Error);
  out->nodes = nodes;
  out->indices = indices;
  out->node_count = node_count;
  return Ok;
}

}  // namespace rtbvh

namespace rtbvh {

cudaError_t launch_locb_segments(const DAabb* aabbs, const uint32_t* sorted, uint32_t* indices,
                                 const uint32_t* prim_off, const uint32_t* order, const DAabb* worlds,
                                 uint32_t mesh_count, uint32_t total_prims, DAabb* lvl0, DAabb* lvl1,
                                 DAabb* final_nodes, uint32_t* nb, uint32_t* status, unsigned blocks,
                                 uint32_t big_count, uint32_t* cluster_sums, unsigned clusters, cudaStream_t s,
                                 cudaStream_t side, cudaEvent_t fork, cudaEvent_t join) {
  if (total_prims == 0 || mesh_count == 0) return cudaSuccess;
  if (big_count > mesh_count || (big_count > 0 && (clusters == 0 || cluster_sums == nullptr)))
    return cudaErrorInvalidValue;
  cudaError_t e;
  k_locb_segment_leaves<<<(total_prims + kBlock - 1) / kBlock, kBlock, 0, s>>>(aabbs, sorted, prim_off, mesh_count,
                                                                                total_prims, lvl0);
  SegParams p;
  p.lvl[0] = lvl0;
  p.lvl[1] = lvl1;
  p.final_nodes = final_nodes;
  p.nb = nb;
  p.prim_off = prim_off;
  p.order = order;
  p.worlds = worlds;
  p.indices = indices;
  p.status = status;
  p.mesh_count = mesh_count;
  // small meshes (one block each) on the side stream, concurrently with the
  // clusters of the large ones; the two sets of meshes share no memory
  const bool fork_side = side != nullptr && big_count > 0 && big_count < mesh_count;
  cudaStream_t small_s = s;
  if (fork_side) {
    if ((e = cudaEventRecord(fork, s)) || (e = cudaStreamWaitEvent(side, fork, 0))) return e;
    small_s = side;
  }
  if (big_count < mesh_count) {
    const unsigned nb_small = std::min<unsigned>(blocks, mesh_count - big_count);
    k_locb_segments<<<nb_small, kBlock, 0, small_s>>>(p, big_count);
    if ((e = cudaGetLastError())) return e;
  }
  if (big_count > 0) {
    k_locb_segments_cluster<<<clusters * kSegCluster, kBlock, 0, s>>>(p, cluster_sums, big_count);
    if ((e = cudaGetLastError())) return e;
  }
  if (fork_side) {
    if ((e = cudaEventRecord(join, side)) || (e = cudaStreamWaitEvent(s, join, 0))) return e;
  }
  return cudaSuccess;
}

}  // namespace rtbvh
