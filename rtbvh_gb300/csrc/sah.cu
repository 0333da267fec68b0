// Binned SAH build (src/builders/binned_sah.rs) on the GPU, breadth first.
//
// The reference runs one task per node (BinnedSahBuildTask::run,
// binned_sah.rs:132-282) from a depth-first work stack. Here the whole build
// is one cooperative launch (k_sah_build) that walks the tree level by
// level; the phases of a level are separated by grid barriers (bounded
// waits), so no host round trip or relaunch happens between levels:
//
//   large tasks (more than sub_max primitives): the grid bins 2048-primitive
//     chunks into per-task global bins (runs of primitives in one bin merged
//     in registers, then ordered-int atomics), one warp per task decides the
//     split, and a chunked stable partition (decoupled look-back over the
//     chunks of a task, bounded waits) scatters the primitive indices;
//   then a scan over the level's tasks numbers the children (breadth-first,
//     deterministic) and builds the next level's task list. Children of at
//     most sub_max primitives are not split level by level: they go to a
//     subtree list. sub_max = n / 2048 clamped to [32, kWarpMax], so a small
//     build keeps enough subtrees to fill the GPU.
//
// After the last level, k_sub_build builds every listed subtree depth first,
// one warp per subtree (bins in shared memory, the warp-parallel decision,
// ballot partition; tasks of at most kThreadMax primitives are finished by
// single lanes, exact sweep over the non-empty bins), with no grid-wide
// phases. The node pair of a split at primitive position m goes to scratch
// slots 2(m-1), 2(m-1)+1 -- split positions are distinct across the whole
// tree -- and a scan over the positions places the pairs after the
// breadth-first part in position order, so the numbering stays
// deterministic and gap-free.
//
// The split arithmetic is the reference's: node box + 1e-4; 16 bins per axis
// with bin = min(15, max(c * (16/diag) + off, 0) as usize) (no FMA); the
// right/left cost sweeps of find_split (empty bins give NaN costs that never
// win); axis choice with strict '>'; the max_split_cost test; the
// longest-axis fallback at 2/5 of the primitives; child boxes from the bins
// (the left one over bins [0, best_splits[axis].count), a reference quirk);
// a leaf box gets the 1e-4 offset a second time. Bin contents are exact, so
// every split equals the reference's. The partition is stable where the
// reference's Lomuto partition (src/utils.rs:74-96) is not: leaves hold the
// same primitive sets, possibly in a different order.
#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBins = 16;
constexpr uint32_t kMaxDepth = 64;
constexpr float kTraversalCost = 1.0f;
constexpr int kChunk = 2048;
constexpr int kLargeBlock = 256;
constexpr uint32_t kWarpMax = 1024;
constexpr uint32_t kCoopMaxPrims = 1u << 20;      // larger builds launch the phases separately
constexpr int kBinWords = 8;  // ordered min xyz, ordered max xyz, count, pad
constexpr int kTaskBinWords = 3 * kBins * kBinWords;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr float kF32Max = 3.40282347e+38f;

struct Task {
  uint32_t node, begin, end, depth;
};

struct Decision {
  uint32_t split, axis, split_index, n_left;
  float lbox[6];
  float rbox[6];
  uint32_t pad[4];
};
static_assert(sizeof(Decision) == 80, "Decision layout");

struct Counters {
  uint32_t large;       // tasks in the current large list
  uint32_t sub;         // subtree tasks listed so far (all levels)
  uint32_t node_count;  // nodes of the breadth-first part so far
  uint32_t chunks;      // chunks of the current large list
  uint32_t status;
  uint32_t ticket;      // chunk ticket of the partition kernel
  uint32_t sub_head;    // next subtree a warp of k_sub_build takes
  uint32_t sub_splits;  // splits inside the subtrees (the scan's total)
  uint32_t tiny;        // subtrees of at most kThreadMax primitives listed by k_sub_build
  uint32_t tiny_head;   // next one a thread of k_sub_tiny takes
};

struct BinMap {
  float c2b[3], off[3];
};

// binned_sah.rs:146-147
__device__ __forceinline__ BinMap make_binmap(const float mn[3], const float mx[3]) {
  BinMap m;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float inv = 1.0f / (mx[a] - mn[a]);
    m.c2b[a] = inv * (float)kBins;
    m.off[a] = (-mn[a]) * m.c2b[a];
  }
  return m;
}

// compute_bin_index (binned_sah.rs:119-128): min(15, max(f, 0) as usize).
__device__ __forceinline__ uint32_t bin_of(float c, float c2b, float off) {
  float f = c * c2b + off;
  if (f >= 15.0f) return 15u;
  if (f > 0.0f) return (uint32_t)f;
  return 0u;
}

__device__ __forceinline__ float ha6(const float mn[3], const float mx[3]) {
  return half_area(mn[0], mn[1], mn[2], mx[0], mx[1], mx[2]);
}

// A task's bins as ordered keys (kTaskBinWords words in shared memory).
struct BinsView {
  const uint32_t* w;
};

// One bin (or a union of bins) as ordered keys (float_to_ordered). Bin
// bounds are never NaN (triangle boxes grow with Vec3::min/max, which ignore
// NaN, from the empty box), and on non-NaN floats the unsigned min/max of the
// keys is Vec3::min/max (-0 below +0); it is commutative and associative and
// counts are integers, so a union over any grouping of the bins equals the
// reference's sequential Aabb::grow_bb bit for bit.
struct BinKey {
  uint32_t mn[3], mx[3];
  uint32_t cnt;
};

__device__ __forceinline__ BinKey load_bin(const BinsView& B, int a, int i) {
  const uint32_t* w = B.w + (a * kBins + i) * kBinWords;
  BinKey v;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v.mn[k] = w[k];
    v.mx[k] = w[3 + k];
  }
  v.cnt = w[6];
  return v;
}

__device__ __forceinline__ void bin_union(BinKey& x, const BinKey& y) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    x.mn[k] = min(x.mn[k], y.mn[k]);
    x.mx[k] = max(x.mx[k], y.mx[k]);
  }
  x.cnt += y.cnt;
}

__device__ __forceinline__ BinKey shfl_bin(const BinKey& v, int delta, bool up) {
  BinKey r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.mn[k] = up ? __shfl_up_sync(0xffffffffu, v.mn[k], delta, 16) : __shfl_down_sync(0xffffffffu, v.mn[k], delta, 16);
    r.mx[k] = up ? __shfl_up_sync(0xffffffffu, v.mx[k], delta, 16) : __shfl_down_sync(0xffffffffu, v.mx[k], delta, 16);
  }
  r.cnt = up ? __shfl_up_sync(0xffffffffu, v.cnt, delta, 16) : __shfl_down_sync(0xffffffffu, v.cnt, delta, 16);
  return r;
}

// A union of bins decoded to floats.
struct BinVal {
  float mn[3], mx[3];
  uint32_t cnt;
};

__device__ __forceinline__ BinVal decode_bin(const BinKey& k) {
  BinVal v;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    v.mn[q] = ordered_to_float(k.mn[q]);
    v.mx[q] = ordered_to_float(k.mx[q]);
  }
  v.cnt = k.cnt;
  return v;
}

// The sweeps of find_split (binned_sah.rs:80-114) for one axis, bin i =
// lane & 15 of a 16-lane segment: pre = bins [0, i], suf = bins [i, 16).
struct AxisScan {
  BinVal pre, suf;
  float best_cost;
  uint32_t best_count;
};

__device__ __forceinline__ AxisScan scan_axis(const BinsView& B, int a, int i) {
  const BinKey b = load_bin(B, a, i);
  BinKey pre = b, suf = b;
#pragma unroll
  for (int d = 1; d < kBins; d <<= 1) {
    const BinKey lo = shfl_bin(pre, d, true);
    const BinKey hi = shfl_bin(suf, d, false);
    if (i >= d) bin_union(pre, lo);
    if (i + d < kBins) bin_union(suf, hi);
  }
  // both sweeps start from Aabb::empty()
  const uint32_t emn = float_to_ordered(1e34f), emx = float_to_ordered(-1e34f);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pre.mn[k] = min(pre.mn[k], emn);
    pre.mx[k] = max(pre.mx[k], emx);
    suf.mn[k] = min(suf.mn[k], emn);
    suf.mx[k] = max(suf.mx[k], emx);
  }
  AxisScan r;
  r.pre = decode_bin(pre);
  r.suf = decode_bin(suf);
  // right_cost[i] (i >= 1) and the left sweep's cost at i (i <= 14)
  const float rc = ha6(r.suf.mn, r.suf.mx) * (float)r.suf.cnt;
  const float rc_next = __shfl_down_sync(0xffffffffu, rc, 1, 16);
  const float cost = ha6(r.pre.mn, r.pre.mx) * (float)r.pre.cnt + rc_next;
  // first minimum over i in [0, 15) of the costs below f32::MAX (strict '<'
  // from f32::MAX in ascending order; NaN costs of empty sides never win)
  bool valid = i < kBins - 1 && cost < kF32Max;
  float c = cost;
  uint32_t idx = valid ? (uint32_t)i : (uint32_t)kBins;
#pragma unroll
  for (int d = 8; d > 0; d >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, c, d, 16);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, d, 16);
    const bool ov = oi < (uint32_t)kBins;
    if (ov && (!valid || oc < c || (oc == c && oi < idx))) {
      c = oc;
      idx = oi;
      valid = true;
    }
  }
  r.best_cost = valid ? c : kF32Max;
  r.best_count = valid ? idx + 1u : (uint32_t)kBins;
  return r;
}

// Value of field f of the scan of `axis` at bin j, fetched from the lane
// holding it (A: axes 0 / 1 in lanes 0-15 / 16-31, B: axis 2 in lanes 0-15).
__device__ __forceinline__ float fetch_f(const AxisScan& A, const AxisScan& Bx, int axis, int j, bool pre, int f) {
  const BinVal& va = pre ? A.pre : A.suf;
  const BinVal& vb = pre ? Bx.pre : Bx.suf;
  const float* fa = f < 3 ? va.mn : va.mx;
  const float* fb = f < 3 ? vb.mn : vb.mx;
  const int k = f % 3;
  const float v = axis == 2 ? fb[k] : fa[k];
  return __shfl_sync(0xffffffffu, v, axis == 1 ? 16 + j : j);
}
__device__ __forceinline__ uint32_t fetch_cnt(const AxisScan& A, const AxisScan& Bx, int axis, int j) {
  const uint32_t v = axis == 2 ? Bx.pre.cnt : A.pre.cnt;
  return __shfl_sync(0xffffffffu, v, axis == 1 ? 16 + j : j);
}

// The split decision of BinnedSahBuildTask::run after binning
// (binned_sah.rs:174-247, find_split at :80-114), evaluated by a whole warp
// (every lane returns the same decision). `box` is the node box with its
// first 1e-4 offset.
__device__ void sah_decide_warp(const BinsView& B, const float bmn[3], const float bmx[3], uint32_t ws,
                                uint32_t max_leaf, Decision& d) {
  const int lane = threadIdx.x & 31, i = lane & 15;
  const AxisScan A = scan_axis(B, lane >> 4, i);  // axis 0 (lanes 0-15), axis 1 (lanes 16-31)
  const AxisScan C = scan_axis(B, 2, i);          // axis 2 (both halves)
  float best_cost[3];
  uint32_t best_count[3];
  best_cost[0] = __shfl_sync(0xffffffffu, A.best_cost, 0);
  best_count[0] = __shfl_sync(0xffffffffu, A.best_count, 0);
  best_cost[1] = __shfl_sync(0xffffffffu, A.best_cost, 16);
  best_count[1] = __shfl_sync(0xffffffffu, A.best_count, 16);
  best_cost[2] = C.best_cost;
  best_count[2] = C.best_count;
  int axis = 0;
  if (best_cost[0] > best_cost[1]) axis = 1;
  if (best_cost[axis] > best_cost[2]) axis = 2;
  uint32_t split_index = best_count[axis];
  const float max_split_cost = ha6(bmn, bmx) * ((float)ws - kTraversalCost);
  d.split = 0;
  if (best_count[axis] == (uint32_t)kBins || best_cost[axis] >= max_split_cost) {
    if (ws <= max_leaf) return;  // leaf
    // longest_axis (src/aabb.rs:353-363)
    int la = 0;
    if ((bmx[1] - bmn[1]) > (bmx[0] - bmn[0])) la = 1;
    if ((bmx[2] - bmn[2]) > (bmx[la] - bmn[la])) la = 2;
    axis = la;
    // first i < 15 whose cumulative count reaches ws * 2 / 5 + 1
    const uint64_t target = (uint64_t)ws * 2 / 5 + 1;
    const uint32_t mine = la == 2 ? C.pre.cnt : A.pre.cnt;
    const bool in_seg = la == 1 ? lane >= 16 : lane < 16;
    const uint32_t hit = __ballot_sync(0xffffffffu, in_seg && i < kBins - 1 && (uint64_t)mine >= target);
    if (hit) split_index = (uint32_t)(__ffs(hit) - 1 - (la == 1 ? 16 : 0)) + 1u;
  }
  const uint32_t n_left = fetch_cnt(A, C, axis, (int)min(split_index, (uint32_t)kBins) - 1);
  if (n_left == 0 || n_left >= ws) return;  // one side empty: leaf
  const int lb = (int)best_count[axis] - 1;     // bins [0, best_splits[axis].count)
  const int rb = (int)min(split_index, (uint32_t)kBins - 1u);  // bins [split_index, 16), split_index <= 15 here
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    d.lbox[f] = fetch_f(A, C, axis, lb, true, f);
    d.rbox[f] = fetch_f(A, C, axis, rb, false, f);
  }
  d.split = 1;
  d.axis = (uint32_t)axis;
  d.split_index = split_index;
  d.n_left = n_left;
}

__device__ __forceinline__ void init_bins(uint32_t* w, int tid, int nthreads) {
  const uint32_t kmin = float_to_ordered(1e34f), kmax = float_to_ordered(-1e34f);
  for (int i = tid; i < 3 * kBins; i += nthreads) {
    uint32_t* b = w + i * kBinWords;
    b[0] = b[1] = b[2] = kmin;
    b[3] = b[4] = b[5] = kmax;
    b[6] = 0;
    b[7] = 0;
  }
}

// Reads the node box, applies the first 1e-4 offset (binned_sah.rs:133),
// and writes it back (count/left_first untouched until the decision).
__device__ __forceinline__ void task_box(DAabb* nodes, uint32_t node, float mn[3], float mx[3]) {
  DAabb b = load_aabb_cg(nodes + node);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    mn[k] = b.min[k] - 0.0001f;
    mx[k] = b.max[k] + 0.0001f;
  }
}

// make_leaf (binned_sah.rs:134-138): second offset, left_first, count.
__device__ __forceinline__ void write_leaf(DAabb* nodes, const Task& t, const float mn[3], const float mx[3]) {
  DAabb b;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.min[k] = mn[k] - 0.0001f;
    b.max[k] = mx[k] + 0.0001f;
  }
  b.count = (int32_t)(t.end - t.begin);
  b.left_first = (int32_t)t.begin;
  store_aabb(nodes + t.node, b);
}

__device__ __forceinline__ void write_interior_box(DAabb* nodes, uint32_t node, const float mn[3], const float mx[3]) {
  DAabb b;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.min[k] = mn[k];
    b.max[k] = mx[k];
  }
  b.count = -1;
  b.left_first = -1;  // set by the emit kernel
  store_aabb(nodes + node, b);
}

struct SahParams {
  const DAabb* aabbs;
  const float4* centers;
  DAabb* nodes;
  uint32_t* idx_a;  // primitive indices (final output)
  uint32_t* idx_b;  // partition scratch
  uint32_t n;
  uint32_t max_leaf;
  uint32_t sub_max;     // largest task built as a subtree (<= kWarpMax)
  Task* large[2];       // task lists of even / odd levels
  Task* subs;           // subtree tasks (at most sub_max primitives), all levels
  void* tiny;           // SubTask list: subtrees of at most kThreadMax primitives
  Decision* dec;        // large tasks of the level
  float* tbox;          // 6 floats per large task (box with first offset)
  uint32_t* bins;       // kTaskBinWords per large task
  uint32_t* chunk_base; // large + 1
  uint32_t* chunk_status;
  uint64_t* scan_vals;  // per task of the level
  uint64_t* scan_sums;  // one per block
  DAabb* tnodes;        // subtree node pairs by split position: 2(m-1), 2(m-1)+1
  uint32_t* sflag;      // 1 at the positions m where a subtree task splits
  uint32_t* srank;      // exclusive scan of sflag
  uint32_t* tile_off;   // per 4096-position tile: sums, then exclusive offsets
  Counters* cnt;
  GridBarrier* bar;
};

// The level being built, as every block read it after the level's first
// barrier.
struct Level {
  const Task* large;
  Task* large_next;
  uint32_t L, node_base, sub_base;
};

// Reads of data written earlier in the same launch (by any block) go to L2:
// the L1 is not coherent between SMs.
__device__ __forceinline__ Task ld_task(const Task* t) {
  const uint4 v = __ldcg(reinterpret_cast<const uint4*>(t));
  return Task{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Decision ld_dec(const Decision* d) {
  Decision r;
  const uint4* q = reinterpret_cast<const uint4*>(d);
  uint4* o = reinterpret_cast<uint4*>(&r);
#pragma unroll
  for (int k = 0; k < 5; ++k) o[k] = __ldcg(q + k);
  return r;
}
__device__ __forceinline__ void ld_tbox(const float* tb, float mn[3], float mx[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    mn[a] = __ldcg(tb + a);
    mx[a] = __ldcg(tb + 3 + a);
  }
}

__device__ __forceinline__ uint32_t find_task(const uint32_t* chunk_base, uint32_t L, uint32_t chunk) {
  uint32_t lo = 0, hi = L;  // last t with chunk_base[t] <= chunk
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldcg(chunk_base + mid) <= chunk) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Shared memory of one block, reused by the phases of a level. The fields
// are ordered by the phases that need them, so a launch of a single phase
// allocates only the prefix it uses (kShSmall, kShBins, all).
struct alignas(16) SahShared {
  uint64_t scan[kLargeBlock / 32];
  uint32_t warp[32];
  uint32_t chunk, fail, prefix, pad;
  uint32_t bins[kLargeBlock / 32][kTaskBinWords];  // per-warp bins
  Decision dec[kLargeBlock / 32];
  uint32_t idx[kLargeBlock / 32][kWarpMax];        // per-warp partition buffer
};
constexpr size_t kShSmall = offsetof(SahShared, bins);  // scans, partition scalars
constexpr size_t kShBins = offsetof(SahShared, dec);    // + per-warp bins

// Bins primitives sidx-ordered positions [i0, i1) into `wb` (one warp's or
// block's shared bins). Neighbours in the index array are usually neighbours
// in space and share bins, so a run of primitives in one bin is merged in
// registers and written with atomics only when an axis changes bin.
template <class IdxFn>
__device__ __forceinline__ void bin_run(const SahParams& p, const BinMap& bm, uint32_t i0, uint32_t i1, IdxFn idx,
                                        uint32_t* wb) {
  uint32_t rbin[3], rmn[3][3], rmx[3][3], rcnt[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rbin[a] = 0xffffffffu;
    rcnt[a] = 0;
  }
  auto flush = [&](int a) {
    if (rcnt[a] == 0) return;
    uint32_t* b = wb + (a * kBins + rbin[a]) * kBinWords;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      atomicMin(b + q, rmn[a][q]);
      atomicMax(b + 3 + q, rmx[a][q]);
    }
    atomicAdd(b + 6, rcnt[a]);
  };
#pragma unroll 1
  for (uint32_t i = i0; i < i1; ++i) {
    const uint32_t prim = idx(i);
    const float4 c = __ldg(p.centers + prim);
    const DAabb box = load_aabb(p.aabbs + prim);
    const float cc[3] = {c.x, c.y, c.z};
    uint32_t kmn[3], kmx[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      kmn[q] = float_to_ordered(box.min[q]);
      kmx[q] = float_to_ordered(box.max[q]);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const uint32_t bin = bin_of(cc[a], bm.c2b[a], bm.off[a]);
      if (bin != rbin[a]) {
        flush(a);
        rbin[a] = bin;
        rcnt[a] = 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          rmn[a][q] = kmn[q];
          rmx[a][q] = kmx[q];
        }
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        rmn[a][q] = min(rmn[a][q], kmn[q]);
        rmx[a][q] = max(rmx[a][q], kmx[q]);
      }
      ++rcnt[a];
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) flush(a);
}

// ------------------------------------------------------------------ large tasks
// Block 0: task boxes (with the first 1e-4 offset) and chunk offsets of the
// level's large tasks.
__device__ void large_prep(const SahParams& p, const Level& lv, SahShared& sh) {
  uint32_t carry = 0;
  for (uint32_t base = 0; base < lv.L; base += kLargeBlock) {
    const uint32_t t = base + threadIdx.x;
    uint32_t chunks = 0;
    if (t < lv.L) {
      const Task tk = ld_task(lv.large + t);
      float mn[3], mx[3];
      task_box(p.nodes, tk.node, mn, mx);
      float* tb = p.tbox + 6 * (size_t)t;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        tb[k] = mn[k];
        tb[3 + k] = mx[k];
      }
      const uint32_t ws = tk.end - tk.begin;
      if (ws > 1 && tk.depth < kMaxDepth) chunks = (ws + kChunk - 1) / kChunk;
    }
    uint32_t total;
    const uint32_t incl = block_inclusive_scan<kLargeBlock>(chunks, sh.warp, &total);
    if (t < lv.L) p.chunk_base[t] = carry + incl - chunks;
    carry += total;
  }
  if (threadIdx.x == 0) {
    p.chunk_base[lv.L] = carry;
    p.cnt->chunks = carry;
    p.cnt->ticket = 0;
  }
}

// Empty bins for every large task (one bin per thread of the grid).
__device__ void large_bins_init(const SahParams& p, const Level& lv) {
  const uint32_t kmin = float_to_ordered(1e34f), kmax = float_to_ordered(-1e34f);
  const size_t total = (size_t)lv.L * 3 * kBins;
  for (size_t i = (size_t)blockIdx.x * kLargeBlock + threadIdx.x; i < total; i += (size_t)gridDim.x * kLargeBlock) {
    uint4* b = reinterpret_cast<uint4*>(p.bins + i * kBinWords);
    b[0] = make_uint4(kmin, kmin, kmin, kmax);
    b[1] = make_uint4(kmax, kmax, 0u, 0u);
  }
}

// Bins one 2048-primitive chunk of a large task into the task's global bins.
__device__ void large_bin_chunk(const SahParams& p, const Level& lv, uint32_t chunk, SahShared& sh) {
  const int warp = threadIdx.x >> 5;
  const uint32_t t = find_task(p.chunk_base, lv.L, chunk);
  const Task tk = ld_task(lv.large + t);
  const uint32_t k = chunk - __ldcg(p.chunk_base + t);
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  init_bins(&sh.bins[warp][0], threadIdx.x & 31, 32);
  __syncthreads();
  float mn[3], mx[3];
  ld_tbox(p.tbox + 6 * (size_t)t, mn, mx);
  const BinMap bm = make_binmap(mn, mx);
  uint32_t* wb = &sh.bins[warp][0];
  // each thread bins kChunk / kLargeBlock consecutive primitives
  constexpr uint32_t PER = kChunk / kLargeBlock;
  const uint32_t s0 = c0 + threadIdx.x * PER;
  bin_run(p, bm, min(s0, c1), min(s0 + PER, c1), [&](uint32_t i) { return __ldcg(p.idx_a + i); }, wb);
  __syncthreads();
  uint32_t* gb = p.bins + (size_t)t * kTaskBinWords;
  for (int i = threadIdx.x; i < 3 * kBins; i += kLargeBlock) {
    uint32_t cnt = 0;
    uint32_t vmn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, vmx[3] = {0u, 0u, 0u};
    for (int w = 0; w < kLargeBlock / 32; ++w) {
      const uint32_t* b = &sh.bins[w][i * kBinWords];
      cnt += b[6];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        vmn[q] = min(vmn[q], b[q]);
        vmx[q] = max(vmx[q], b[3 + q]);
      }
    }
    if (cnt) {
      uint32_t* g = gb + i * kBinWords;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        atomicMin(g + q, vmn[q]);
        atomicMax(g + 3 + q, vmx[q]);
      }
      atomicAdd(g + 6, cnt);
    }
  }
  __syncthreads();  // the shared bins are reused by the block's next chunk
}

// Split decision of large task t by one warp (its global bins are copied to
// the warp's shared bins first).
__device__ void large_decide(const SahParams& p, const Level& lv, uint32_t t, SahShared& sh) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Task tk = ld_task(lv.large + t);
  float mn[3], mx[3];
  ld_tbox(p.tbox + 6 * (size_t)t, mn, mx);
  Decision d;
  d.split = 0;
  const uint32_t ws = tk.end - tk.begin;
  if (ws > 1 && tk.depth < kMaxDepth) {
    uint32_t* wb = &sh.bins[warp][0];
    const uint32_t* gb = p.bins + (size_t)t * kTaskBinWords;
    for (int i = lane; i < kTaskBinWords; i += 32) wb[i] = __ldcg(gb + i);
    __syncwarp();
    sah_decide_warp(BinsView{wb}, mn, mx, ws, p.max_leaf, d);
    __syncwarp();
  }
  if (lane == 0) {
    if (d.split) write_interior_box(p.nodes, tk.node, mn, mx);
    else write_leaf(p.nodes, tk, mn, mx);
    p.dec[t] = d;
  }
}

// Stable partition of a large task's chunk into idx_b; the number of left
// primitives in the task's earlier chunks comes from a decoupled look-back
// (chunks are taken in ticket order, so every chunk waited on is held by a
// running block).
__device__ void large_partition_chunk(const SahParams& p, const Level& lv, uint32_t chunk, SahShared& sh) {
  const uint32_t t = find_task(p.chunk_base, lv.L, chunk);
  const Decision d = ld_dec(p.dec + t);
  if (!d.split) return;  // no chunk of this task waits on another
  const Task tk = ld_task(lv.large + t);
  const uint32_t first_chunk = __ldcg(p.chunk_base + t);
  const uint32_t k = chunk - first_chunk;
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  float mn[3], mx[3];
  ld_tbox(p.tbox + 6 * (size_t)t, mn, mx);
  const BinMap bm = make_binmap(mn, mx);
  const int ax = (int)d.axis;
  constexpr int PER = kChunk / kLargeBlock;
  uint32_t prim[PER];
  uint32_t flags = 0, mine = 0;
  const uint32_t s = c0 + threadIdx.x * PER;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const uint32_t i = s + j;
    prim[j] = 0;
    if (i < c1) {
      prim[j] = __ldcg(p.idx_a + i);
      const float4 c = __ldg(p.centers + prim[j]);
      const float cc = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
      if (bin_of(cc, bm.c2b[ax], bm.off[ax]) < d.split_index) {
        flags |= 1u << j;
        ++mine;
      }
    }
  }
  uint32_t chunk_true;
  const uint32_t incl = block_inclusive_scan<kLargeBlock>(mine, sh.warp, &chunk_true);
  const uint32_t before_me = incl - mine;
  volatile uint32_t* st = p.chunk_status;
  if (threadIdx.x == 0) {
    uint32_t excl = 0;
    sh.fail = 0;
    if (k == 0) {
      st[chunk] = kFlagInc | chunk_true;
    } else {
      st[chunk] = kFlagAgg | chunk_true;
      uint32_t j = chunk - 1;
      uint32_t spins = 0;
      for (;;) {
        const uint32_t v = st[j];
        const uint32_t f = v & ~kCountMask;
        if (f == 0u) {
          if (++spins > kSpinLimit) {
            atomicOr(&p.cnt->status, kStatusTimeout);
            sh.fail = 1;
            break;
          }
          __nanosleep(64);
          continue;
        }
        excl += v & kCountMask;
        if (f == kFlagInc || j == first_chunk) break;
        --j;
      }
      st[chunk] = kFlagInc | (excl + chunk_true);
    }
    sh.prefix = excl;
  }
  __syncthreads();
  const bool fail = sh.fail != 0;
  const uint32_t true_before = sh.prefix + before_me;
  __syncthreads();  // sh.prefix / sh.fail are rewritten by the block's next chunk
  if (fail) return;
  uint32_t tpos = tk.begin + true_before;
  uint32_t fpos = tk.begin + d.n_left + ((s - tk.begin) - true_before);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const uint32_t i = s + j;
    if (i < c1) {
      uint32_t dst = ((flags >> j) & 1u) ? tpos++ : fpos++;
      if (dst < tk.end) p.idx_b[dst] = prim[j];
      else atomicOr(&p.cnt->status, kStatusBadIndex);
    }
  }
}

__device__ void large_copyback_chunk(const SahParams& p, const Level& lv, uint32_t chunk) {
  const uint32_t t = find_task(p.chunk_base, lv.L, chunk);
  if (!__ldcg(&p.dec[t].split)) return;
  const Task tk = ld_task(lv.large + t);
  const uint32_t k = chunk - __ldcg(p.chunk_base + t);
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  for (uint32_t i = c0 + threadIdx.x; i < c1; i += kLargeBlock) p.idx_a[i] = __ldcg(p.idx_b + i);
}

// ------------------------------------------------------------------ small tasks
// A task of at most kThreadMax primitives is decided by one thread. Its
// bins hold at most kThreadMax primitives, and find_split's cost at bin i
// depends only on which primitives lie left and right of i: it is NaN while
// a side is empty and constant between two non-empty bins. So the first
// minimum over i is found by visiting the non-empty bins in ascending order
// and evaluating the cost at each (the same float expression over the same
// unions, hence the same bits). Larger small tasks take a warp each.
constexpr uint32_t kThreadMax = 8;

// Union, from Aabb::empty(), of the primitives in `sel` (keys, decoded).
__device__ __forceinline__ void union_sel(const uint32_t (&kb)[kThreadMax][6], uint32_t ws, uint32_t sel, float mn[3],
                                          float mx[3]) {
  uint32_t umn[3], umx[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    umn[k] = float_to_ordered(1e34f);
    umx[k] = float_to_ordered(-1e34f);
  }
#pragma unroll
  for (uint32_t j = 0; j < kThreadMax; ++j) {
    if (j < ws && ((sel >> j) & 1u)) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        umn[k] = min(umn[k], kb[j][k]);
        umx[k] = max(umx[k], kb[j][3 + k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    mn[k] = ordered_to_float(umn[k]);
    mx[k] = ordered_to_float(umx[k]);
  }
}

__device__ __forceinline__ uint32_t bin_at(uint32_t packed, uint32_t j) { return (packed >> (4 * j)) & 15u; }

// Mask of the primitives whose bin is below `bound`.
__device__ __forceinline__ uint32_t below(uint32_t packed, uint32_t ws, uint32_t bound) {
  uint32_t m = 0;
#pragma unroll
  for (uint32_t j = 0; j < kThreadMax; ++j)
    if (j < ws && bin_at(packed, j) < bound) m |= 1u << j;
  return m;
}

// Smallest bin above `after` (16: none) -- ascending visit of non-empty bins.
__device__ __forceinline__ uint32_t next_bin(uint32_t packed, uint32_t ws, int after) {
  uint32_t nb = (uint32_t)kBins;
#pragma unroll
  for (uint32_t j = 0; j < kThreadMax; ++j) {
    const uint32_t b = bin_at(packed, j);
    if (j < ws && (int)b > after && b < nb) nb = b;
  }
  return nb;
}

// BinnedSahBuildTask::run (binned_sah.rs:132-282) after the node box is
// known, for a task of at most kThreadMax primitives by one thread: `mn` /
// `mx` is the node box with its first offset. On a split the task's indices
// are left stably partitioned (left primitives first, in order).
__device__ void decide_thread(const SahParams& p, uint32_t begin, uint32_t ws, uint32_t depth, const float mn[3],
                              const float mx[3], Decision& d) {
  d.split = 0;
  if (ws > 1 && depth < kMaxDepth) {
    uint32_t prim[kThreadMax];
    uint32_t kb[kThreadMax][6];
    uint32_t packed[3] = {0u, 0u, 0u};
    const BinMap bm = make_binmap(mn, mx);
#pragma unroll
    for (uint32_t j = 0; j < kThreadMax; ++j) {
      if (j < ws) {
        prim[j] = p.idx_a[begin + j];
        const float4 c = __ldg(p.centers + prim[j]);
        const DAabb box = load_aabb(p.aabbs + prim[j]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          kb[j][k] = float_to_ordered(box.min[k]);
          kb[j][3 + k] = float_to_ordered(box.max[k]);
        }
        packed[0] |= bin_of(c.x, bm.c2b[0], bm.off[0]) << (4 * j);
        packed[1] |= bin_of(c.y, bm.c2b[1], bm.off[1]) << (4 * j);
        packed[2] |= bin_of(c.z, bm.c2b[2], bm.off[2]) << (4 * j);
      }
    }
    const uint32_t all = (1u << ws) - 1u;
    float best_cost[3];
    uint32_t best_count[3];
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
      float bc = kF32Max;
      uint32_t bn = (uint32_t)kBins;
      for (int b = -1;;) {
        b = (int)next_bin(packed[a], ws, b);
        if (b >= kBins) break;
        const uint32_t left = below(packed[a], ws, (uint32_t)b + 1u);
        if (left == all) break;  // right side empty from here on
        float lmn[3], lmx[3], rmn[3], rmx[3];
        union_sel(kb, ws, left, lmn, lmx);
        union_sel(kb, ws, all & ~left, rmn, rmx);
        const uint32_t nl = (uint32_t)__popc(left);
        const float cost = ha6(lmn, lmx) * (float)nl + ha6(rmn, rmx) * (float)(ws - nl);
        if (cost < bc) {
          bc = cost;
          bn = (uint32_t)b + 1u;
        }
      }
      best_cost[a] = bc;
      best_count[a] = bn;
    }
    int axis = 0;
    if (best_cost[0] > best_cost[1]) axis = 1;
    if (best_cost[axis] > best_cost[2]) axis = 2;
    uint32_t split_index = best_count[axis];
    const float max_split_cost = ha6(mn, mx) * ((float)ws - kTraversalCost);
    bool leaf = false;
    if (best_count[axis] == (uint32_t)kBins || best_cost[axis] >= max_split_cost) {
      if (ws <= p.max_leaf) {
        leaf = true;
      } else {
        int la = 0;
        if ((mx[1] - mn[1]) > (mx[0] - mn[0])) la = 1;
        if ((mx[2] - mn[2]) > (mx[la] - mn[la])) la = 2;
        axis = la;
        const uint32_t target = ws * 2 / 5 + 1;
        for (int b = -1;;) {
          b = (int)next_bin(packed[la], ws, b);
          if (b >= kBins - 1) break;  // the reference's loop stops before bin 15
          if ((uint32_t)__popc(below(packed[la], ws, (uint32_t)b + 1u)) >= target) {
            split_index = (uint32_t)b + 1u;
            break;
          }
        }
      }
    }
    if (!leaf) {
      const uint32_t left = below(packed[axis], ws, split_index);
      const uint32_t n_left = (uint32_t)__popc(left);
      if (n_left > 0 && n_left < ws) {
        d.split = 1;
        d.axis = (uint32_t)axis;
        d.split_index = split_index;
        d.n_left = n_left;
        float lmn[3], lmx[3], rmn[3], rmx[3];
        union_sel(kb, ws, below(packed[axis], ws, best_count[axis]), lmn, lmx);
        union_sel(kb, ws, all & ~left, rmn, rmx);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          d.lbox[k] = lmn[k];
          d.lbox[3 + k] = lmx[k];
          d.rbox[k] = rmn[k];
          d.rbox[3 + k] = rmx[k];
        }
        uint32_t tpos = begin, fpos = begin + n_left;
#pragma unroll
        for (uint32_t j = 0; j < kThreadMax; ++j) {
          if (j < ws) p.idx_a[((left >> j) & 1u) ? tpos++ : fpos++] = prim[j];
        }
      }
    }
  }
}

// The same for a task of more than kThreadMax primitives by one warp: bins
// in shared memory (wb), indices staged in sidx, the warp-parallel decision,
// a ballot-based stable partition. The decision is left in `d` (shared
// memory, written by lane 0) for every lane.
__device__ void decide_warp(const SahParams& p, uint32_t begin, uint32_t ws, uint32_t depth, const float mn[3],
                            const float mx[3], uint32_t* wb, uint32_t* sidx, Decision& d) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) d.split = 0;
  __syncwarp();
  if (ws > 1 && depth < kMaxDepth && ws <= kWarpMax) {
    init_bins(wb, lane, 32);
    // stage the task's indices (independent loads, all in flight at once)
    for (uint32_t i = lane; i < ws; i += 32) sidx[i] = p.idx_a[begin + i];
    __syncwarp();
    const BinMap bm = make_binmap(mn, mx);
    {
      // each lane bins a contiguous slice, merging runs of primitives that
      // fall in one bin before its shared-memory atomics
      const uint32_t per = (ws + 31) / 32;
      const uint32_t lo = min(ws, (uint32_t)lane * per);
      bin_run(p, bm, lo, min(ws, lo + per), [&](uint32_t i) { return sidx[i]; }, wb);
    }
    __syncwarp();
    {
      Decision dl;
      sah_decide_warp(BinsView{wb}, mn, mx, ws, p.max_leaf, dl);
      if (lane == 0) d = dl;
    }
    __syncwarp();
    if (d.split) {
      const int ax = (int)d.axis;
      const uint32_t lt = (1u << lane) - 1u;
      const uint32_t split_index = d.split_index, n_left = d.n_left;
      uint32_t tb = 0, fb = 0;
      for (uint32_t c0 = 0; c0 < ws; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool valid = i < ws;
        uint32_t prim = 0;
        bool pred = false;
        if (valid) {
          prim = sidx[i];
          const float4 c = __ldg(p.centers + prim);
          const float cc = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
          pred = bin_of(cc, bm.c2b[ax], bm.off[ax]) < split_index;
        }
        const uint32_t T = __ballot_sync(0xffffffffu, pred);
        const uint32_t V = __ballot_sync(0xffffffffu, valid);
        const uint32_t F = V & ~T;
        // written straight to the task's range: the staged copy is the source
        if (pred) p.idx_a[begin + tb + __popc(T & lt)] = prim;
        else if (valid) {
          const uint32_t dst = n_left + fb + __popc(F & lt);
          if (dst < ws) p.idx_a[begin + dst] = prim;
        }
        tb += __popc(T);
        fb += __popc(F);
      }
    }
  }
  __syncwarp();
}

// ------------------------------------------------------------------ subtrees
constexpr uint32_t kTemp = 0x80000000u;  // SubTask::loc bit: a scratch slot, else a node of the breadth-first part

struct SubTask {
  uint32_t loc, begin, end, depth;
  float box[6];  // the box the parent gave the node (min xyz, max xyz), before the first offset
};
constexpr int kSubStack = (int)kMaxDepth + 2;
constexpr int kSubBlock = 128;

// Shared memory of one warp of k_sub_build.
struct SubShared {
  uint32_t bins[kTaskBinWords];
  uint32_t idx[kWarpMax];
  Decision dec;
  SubTask stack[kSubStack];
};

__device__ __forceinline__ DAabb* sub_node(const SahParams& p, uint32_t loc) {
  return (loc & kTemp) ? p.tnodes + (loc & ~kTemp) : p.nodes + loc;
}

// Writes task tk's node (mn / mx: its box with the first offset): an
// interior node whose left_first is, until the relocation, the split
// position m; or a leaf (make_leaf: second offset, first primitive, count).
// On a split, notes m and returns the children.
__device__ __forceinline__ bool sub_write(const SahParams& p, const SubTask& tk, const float mn[3], const float mx[3],
                                          const Decision& d, SubTask& l, SubTask& r) {
  DAabb b;
  if (d.split) {
    const uint32_t m = tk.begin + d.n_left;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      b.min[k] = mn[k];
      b.max[k] = mx[k];
    }
    b.count = -1;
    b.left_first = (int32_t)m;
    store_aabb(sub_node(p, tk.loc), b);
    p.sflag[m] = 1u;
    l.loc = kTemp | (2u * (m - 1u));
    l.begin = tk.begin;
    l.end = m;
    l.depth = tk.depth + 1u;
    r.loc = kTemp | (2u * (m - 1u) + 1u);
    r.begin = m;
    r.end = tk.end;
    r.depth = tk.depth + 1u;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      l.box[k] = d.lbox[k];
      r.box[k] = d.rbox[k];
    }
    return true;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b.min[k] = mn[k] - 0.0001f;
    b.max[k] = mx[k] + 0.0001f;
  }
  b.count = (int32_t)(tk.end - tk.begin);
  b.left_first = (int32_t)tk.begin;
  store_aabb(sub_node(p, tk.loc), b);
  return false;
}

__device__ __forceinline__ void first_offset(const SubTask& tk, float mn[3], float mx[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    mn[k] = tk.box[k] - 0.0001f;
    mx[k] = tk.box[3 + k] + 0.0001f;
  }
}

// A subtree whose root holds at most kThreadMax primitives, by one lane,
// depth first (at most kThreadMax - 1 splits, so the stack stays below
// kThreadMax + 1 entries).
__device__ void sub_tiny(const SahParams& p, const SubTask& t0) {
  SubTask st[kThreadMax + 1];
  int sp = 0;
  st[0] = t0;
  while (sp >= 0) {
    const SubTask tk = st[sp--];
    float mn[3], mx[3];
    first_offset(tk, mn, mx);
    Decision d;
    decide_thread(p, tk.begin, tk.end - tk.begin, tk.depth, mn, mx, d);
    SubTask l, r;
    if (sub_write(p, tk, mn, mx, d, l, r)) {
      if (sp + 2 >= (int)kThreadMax + 1) {
        atomicOr(&p.cnt->status, kStatusBadIndex);
        return;
      }
      st[++sp] = r;
      st[++sp] = l;
    }
  }
}

// Appends a subtree of at most kThreadMax primitives to the list that
// k_sub_tiny finishes, one thread per subtree.
__device__ __forceinline__ void sub_list_tiny(const SahParams& p, const SubTask& t) {
  const uint32_t k = atomicAdd(&p.cnt->tiny, 1u);
  if (k < p.n) reinterpret_cast<SubTask*>(p.tiny)[k] = t;
  else atomicOr(&p.cnt->status, kStatusBadIndex);
}

// One subtree by one warp, depth first: tasks of more than kThreadMax
// primitives by the whole warp; smaller ones are listed for k_sub_tiny.
// Every write goes to a place fixed by the task's primitive range, so the
// order in which tasks run does not matter.
__device__ void sub_warp_tree(const SahParams& p, const Task& root, SubShared& sh) {
  const int lane = threadIdx.x & 31;
  int sp = -1;  // warp-uniform
  const uint32_t rws = root.end - root.begin;
  if (lane == 0) {
    const DAabb rb = load_aabb_cg(p.nodes + root.node);
    SubTask t;
    t.loc = root.node;
    t.begin = root.begin;
    t.end = root.end;
    t.depth = root.depth;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      t.box[k] = rb.min[k];
      t.box[3 + k] = rb.max[k];
    }
    if (rws <= kThreadMax) sub_list_tiny(p, t);
    else sh.stack[0] = t;
  }
  if (rws > kThreadMax) sp = 0;
  __syncwarp();
  while (sp >= 0) {
    const SubTask tk = sh.stack[sp--];
    float mn[3], mx[3];
    first_offset(tk, mn, mx);
    decide_warp(p, tk.begin, tk.end - tk.begin, tk.depth, mn, mx, sh.bins, sh.idx, sh.dec);
    const Decision d = sh.dec;
    __syncwarp();
    SubTask l, r;
    if (lane == 0) sub_write(p, tk, mn, mx, d, l, r);
    if (d.split) {
      const uint32_t nl = d.n_left, nr = (tk.end - tk.begin) - d.n_left;
      if (sp + 2 >= kSubStack) {
        if (lane == 0) atomicOr(&p.cnt->status, kStatusBadIndex);
        return;
      }
      // right child first onto the stack: the left one is taken next
      if (nr <= kThreadMax) {
        if (lane == 0) sub_list_tiny(p, r);
      } else {
        if (lane == 0) sh.stack[sp + 1] = r;
        ++sp;
      }
      if (nl <= kThreadMax) {
        if (lane == 0) sub_list_tiny(p, l);
      } else {
        if (lane == 0) sh.stack[sp + 1] = l;
        ++sp;
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ level scan + emit
__device__ __forceinline__ uint64_t children_value(const Decision& d, const Task& tk, uint32_t sub_max) {
  if (!d.split) return 0;
  const uint32_t ws = tk.end - tk.begin;
  const uint32_t nl = d.n_left, nr = ws - d.n_left;
  const uint64_t large = (uint64_t)(nl > sub_max) + (uint64_t)(nr > sub_max);
  return (large << 32) | (uint64_t)(2u - (uint32_t)large);
}

__device__ __forceinline__ Task level_task(const Level& lv, uint32_t t) { return ld_task(lv.large + t); }

template <class T>
__device__ __forceinline__ T block_scan_incl(T v, T* s_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = kLargeBlock / 32;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  if (lane == 31) s_warp[warp] = v;
  __syncthreads();
  if (warp == 0) {
    T w = lane < NW ? s_warp[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T n = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += n;
    }
    if (lane < NW) s_warp[lane] = w;
  }
  __syncthreads();
  T prefix = warp > 0 ? s_warp[warp - 1] : (T)0;
  T tt = s_warp[NW - 1];
  __syncthreads();
  *total = tt;
  return v + prefix;
}

// Block b's contiguous segment of the level's tasks.
__device__ __forceinline__ void segment(uint32_t N, uint32_t& lo, uint32_t& hi) {
  const uint32_t seg = (N + gridDim.x - 1) / gridDim.x;
  lo = min(N, blockIdx.x * seg);
  hi = min(N, lo + seg);
}

// Children values of the segment: exclusive scan within the segment
// (scan_vals) and the segment total (scan_sums[block]).
__device__ void scan_segment(const SahParams& p, const Level& lv, SahShared& sh) {
  uint32_t lo, hi;
  segment(lv.L, lo, hi);
  uint64_t carry = 0;
  for (uint32_t base = lo; base < hi; base += kLargeBlock) {
    const uint32_t t = base + threadIdx.x;
    uint64_t v = 0;
    if (t < hi) v = children_value(ld_dec(p.dec + t), level_task(lv, t), p.sub_max);
    uint64_t total;
    const uint64_t incl = block_scan_incl<uint64_t>(v, sh.scan, &total);
    if (t < hi) p.scan_vals[t] = carry + incl - v;
    carry += total;
  }
  if (threadIdx.x == 0) p.scan_sums[blockIdx.x] = carry;
}

// Node numbering (breadth first), the next level's task list and the
// subtree list.
__device__ void emit_segment(const SahParams& p, const Level& lv, SahShared& sh, bool advance) {
  // prefix of the block totals before this block, and the level total
  uint64_t before = 0, all = 0;
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += kLargeBlock) {
    const uint64_t v = __ldcg(p.scan_sums + b);
    all += v;
    if (b < blockIdx.x) before += v;
  }
  uint64_t t0, t1;
  block_scan_incl<uint64_t>(before, sh.scan, &t0);
  block_scan_incl<uint64_t>(all, sh.scan, &t1);
  before = t0;
  all = t1;
  uint32_t lo, hi;
  segment(lv.L, lo, hi);
  for (uint32_t t = lo + threadIdx.x; t < hi; t += kLargeBlock) {
    const Decision d = ld_dec(p.dec + t);
    if (!d.split) continue;
    const Task tk = level_task(lv, t);
    const uint64_t ex = __ldcg(p.scan_vals + t) + before;
    uint32_t li = (uint32_t)(ex >> 32), si = (uint32_t)(ex & 0xffffffffu);
    const uint32_t child = lv.node_base + li + si;
    DAabb nd = load_aabb_cg(p.nodes + tk.node);
    nd.left_first = (int32_t)child;
    nd.count = -1;
    store_aabb(p.nodes + tk.node, nd);
    DAabb lb, rb;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      lb.min[k] = d.lbox[k];
      lb.max[k] = d.lbox[3 + k];
      rb.min[k] = d.rbox[k];
      rb.max[k] = d.rbox[3 + k];
    }
    lb.count = rb.count = 0;
    lb.left_first = rb.left_first = 0;
    store_aabb(p.nodes + child, lb);
    store_aabb(p.nodes + child + 1, rb);
    const Task lt{child, tk.begin, tk.begin + d.n_left, tk.depth + 1};
    const Task rt{child + 1, tk.begin + d.n_left, tk.end, tk.depth + 1};
    if (lt.end - lt.begin > p.sub_max) lv.large_next[li++] = lt;
    else p.subs[lv.sub_base + si++] = lt;
    if (rt.end - rt.begin > p.sub_max) lv.large_next[li++] = rt;
    else p.subs[lv.sub_base + si++] = rt;
  }
  if (advance && blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t nl = (uint32_t)(all >> 32), ns = (uint32_t)(all & 0xffffffffu);
    p.cnt->node_count = lv.node_base + nl + ns;
    p.cnt->large = nl;
    p.cnt->sub = lv.sub_base + ns;
  }
}

// Blocks take partition chunks in ticket order until all are done.
__device__ void large_partition_phase(const SahParams& p, const Level& lv, uint32_t chunks, SahShared& sh) {
  for (;;) {
    if (threadIdx.x == 0) sh.chunk = atomicAdd(&p.cnt->ticket, 1u);
    __syncthreads();
    const uint32_t c = sh.chunk;
    __syncthreads();
    if (c >= chunks) break;
    large_partition_chunk(p, lv, c, sh);
  }
}

__device__ __forceinline__ Level read_level(const SahParams& p, uint32_t level) {
  Level lv;
  lv.L = __ldcg(&p.cnt->large);
  lv.node_base = __ldcg(&p.cnt->node_count);
  lv.sub_base = __ldcg(&p.cnt->sub);
  lv.large = p.large[level & 1];
  lv.large_next = p.large[(level + 1) & 1];
  return lv;
}

// The breadth-first part of the build: one cooperative launch, the levels of
// the tree one after another, phases separated by grid barriers. Level l
// reads task list large[l & 1] and writes the other one.
__global__ void __launch_bounds__(kLargeBlock, 2) k_sah_build(SahParams p) {
  __shared__ SahShared sh;
  const uint32_t G = gridDim.x;
  const uint32_t gwarp = (blockIdx.x * kLargeBlock + threadIdx.x) >> 5, nwarps = G * (kLargeBlock / 32);
  uint32_t* status = &p.cnt->status;
  for (uint32_t level = 0;; ++level) {
    const Level lv = read_level(p, level);
    if (lv.L == 0) break;
    if (level > kMaxDepth + 1) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, kStatusBadIndex);
      break;
    }
    uint32_t chunks = 0;
    if (lv.L > 0) {
      if (blockIdx.x == 0) large_prep(p, lv, sh);
      large_bins_init(p, lv);
      if (!grid_sync(p.bar, G, status)) return;
      chunks = __ldcg(&p.cnt->chunks);
      for (uint32_t c = blockIdx.x; c < chunks; c += G) large_bin_chunk(p, lv, c, sh);
      if (!grid_sync(p.bar, G, status)) return;
      for (uint32_t t = gwarp; t < lv.L; t += nwarps) large_decide(p, lv, t, sh);
    }
    if (!grid_sync(p.bar, G, status)) return;
    // large partitions (chunks in ticket order)
    if (lv.L > 0) large_partition_phase(p, lv, chunks, sh);
    if (!grid_sync(p.bar, G, status)) return;
    if (lv.L > 0) {
      for (uint32_t c = blockIdx.x; c < chunks; c += G) large_copyback_chunk(p, lv, c);
      for (uint32_t c = blockIdx.x * kLargeBlock + threadIdx.x; c < chunks; c += G * kLargeBlock)
        p.chunk_status[c] = 0;
    }
    scan_segment(p, lv, sh);
    if (!grid_sync(p.bar, G, status)) return;
    emit_segment(p, lv, sh, true);
    if (!grid_sync(p.bar, G, status)) return;
  }
}

// Dynamic shared memory of a per-phase launch, sized to the prefix of
// SahShared that the phase uses.
__device__ __forceinline__ SahShared& dyn_shared() {
  extern __shared__ __align__(16) unsigned char sah_dyn[];
  return *reinterpret_cast<SahShared*>(sah_dyn);
}

// ---- the same phases as separate launches (large builds): the level number
// selects the task lists, counters are read at kernel start.
__global__ void __launch_bounds__(kLargeBlock) k_ph_prep(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  if (blockIdx.x == 0) large_prep(p, lv, sh);
  large_bins_init(p, lv);
}
__global__ void __launch_bounds__(kLargeBlock) k_ph_bin(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  const uint32_t chunks = __ldcg(&p.cnt->chunks);
  for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) large_bin_chunk(p, lv, c, sh);
}
__global__ void __launch_bounds__(kLargeBlock) k_ph_decide(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  const uint32_t gwarp = (blockIdx.x * kLargeBlock + threadIdx.x) >> 5, nwarps = gridDim.x * (kLargeBlock / 32);
  for (uint32_t t = gwarp; t < lv.L; t += nwarps) large_decide(p, lv, t, sh);
}
__global__ void __launch_bounds__(kLargeBlock) k_ph_partition(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  large_partition_phase(p, lv, __ldcg(&p.cnt->chunks), sh);
}
__global__ void __launch_bounds__(kLargeBlock) k_ph_copyback_scan(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  if (lv.L > 0) {
    const uint32_t chunks = __ldcg(&p.cnt->chunks);
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) large_copyback_chunk(p, lv, c);
    for (uint32_t c = blockIdx.x * kLargeBlock + threadIdx.x; c < chunks; c += gridDim.x * kLargeBlock)
      p.chunk_status[c] = 0;
  }
  scan_segment(p, lv, sh);
}
__global__ void __launch_bounds__(kLargeBlock) k_ph_emit(SahParams p, uint32_t level) {
  SahShared& sh = dyn_shared();
  emit_segment(p, read_level(p, level), sh, false);
}
// Counters of the next level (after every block of k_ph_emit read them).
__global__ void k_ph_advance(SahParams p, uint32_t level, uint32_t blocks) {
  SahShared& sh = dyn_shared();
  const Level lv = read_level(p, level);
  uint64_t all = 0;
  for (uint32_t b = threadIdx.x; b < blocks; b += kLargeBlock) all += __ldcg(p.scan_sums + b);
  uint64_t tot;
  block_scan_incl<uint64_t>(all, sh.scan, &tot);
  if (threadIdx.x == 0) {
    const uint32_t nl = (uint32_t)(tot >> 32), ns = (uint32_t)(tot & 0xffffffffu);
    p.cnt->node_count = lv.node_base + nl + ns;
    p.cnt->large = nl;
    p.cnt->sub = lv.sub_base + ns;
  }
}

// ---- subtrees and their placement
__global__ void __launch_bounds__(kSubBlock) k_sub_build(SahParams p) {
  extern __shared__ __align__(16) unsigned char sub_dyn[];
  SubShared& sh = reinterpret_cast<SubShared*>(sub_dyn)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const uint32_t S = __ldcg(&p.cnt->sub);
  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(&p.cnt->sub_head, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= S) break;
    sub_warp_tree(p, ld_task(p.subs + t), sh);
  }
}

// The listed subtrees of at most kThreadMax primitives, one thread each
// (two blocks per SM: 128 registers, 16 bytes of spills, twice the warps of
// the unbounded 143-register form).
__global__ void __launch_bounds__(kLargeBlock, 2) k_sub_tiny(SahParams p) {
  const uint32_t T = __ldcg(&p.cnt->tiny);
  const SubTask* list = reinterpret_cast<const SubTask*>(p.tiny);
  for (uint32_t t = blockIdx.x * kLargeBlock + threadIdx.x; t < T && t < p.n; t += gridDim.x * kLargeBlock)
    sub_tiny(p, list[t]);
}

constexpr uint32_t kScanTile = 4096;  // split positions per tile: 1024 threads x 4

__global__ void __launch_bounds__(1024) k_tile_sums(const uint32_t* __restrict__ flag, uint32_t n,
                                                    uint32_t* __restrict__ tile_off) {
  __shared__ uint32_t s_warp[32];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * 4u;
  uint32_t v = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k)
    if (base + k < n) v += flag[base + k];
  uint32_t total;
  block_inclusive_scan<1024>(v, s_warp, &total);
  if (threadIdx.x == 0) tile_off[blockIdx.x] = total;
}

// Exclusive offsets of the tiles (one block); the total is the number of
// splits inside the subtrees.
__global__ void __launch_bounds__(1024) k_tile_scan(uint32_t* __restrict__ tile_off, uint32_t tiles, Counters* cnt) {
  __shared__ uint32_t s_warp[32];
  uint32_t carry = 0;
  for (uint32_t base = 0; base < tiles; base += 1024) {
    const uint32_t t = base + threadIdx.x;
    const uint32_t v = t < tiles ? tile_off[t] : 0u;
    uint32_t total;
    const uint32_t incl = block_inclusive_scan<1024>(v, s_warp, &total);
    if (t < tiles) tile_off[t] = carry + incl - v;
    carry += total;
  }
  if (threadIdx.x == 0) cnt->sub_splits = carry;
}

__global__ void __launch_bounds__(1024) k_rank(const uint32_t* __restrict__ flag, uint32_t n,
                                               const uint32_t* __restrict__ tile_off, uint32_t* __restrict__ rank) {
  __shared__ uint32_t s_warp[32];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * 4u;
  uint32_t f[4], v = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    f[k] = base + k < n ? flag[base + k] : 0u;
    v += f[k];
  }
  uint32_t total;
  uint32_t x = block_inclusive_scan<1024>(v, s_warp, &total) - v + tile_off[blockIdx.x];
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    if (base + k < n) rank[base + k] = x;
    x += f[k];
  }
}

// The node pair of subtree split m goes to top + 2 rank[m] (top: the nodes
// of the breadth-first part); interior nodes get their children's final
// index.
__global__ void __launch_bounds__(kLargeBlock) k_relocate(SahParams p) {
  const uint32_t m = blockIdx.x * kLargeBlock + threadIdx.x;
  if (m == 0 || m >= p.n || !p.sflag[m]) return;
  const uint32_t top = __ldcg(&p.cnt->node_count);
  const uint32_t pair = top + 2u * p.srank[m];
  if (pair + 1u >= 2u * p.n - 1u) {  // past the 2n - 1 nodes
    atomicOr(&p.cnt->status, kStatusBadIndex);
    return;
  }
#pragma unroll
  for (uint32_t k = 0; k < 2; ++k) {
    DAabb nd = load_aabb(p.tnodes + 2u * (m - 1u) + k);
    if (nd.count < 0) {
      const uint32_t c = (uint32_t)nd.left_first;
      if (c == 0 || c >= p.n) {
        atomicOr(&p.cnt->status, kStatusBadIndex);
        return;
      }
      nd.left_first = (int32_t)(top + 2u * p.srank[c]);
    }
    store_aabb(p.nodes + pair + k, nd);
  }
}

// Subtree roots (nodes of the breadth-first part) that split.
__global__ void __launch_bounds__(kLargeBlock) k_fix_roots(SahParams p) {
  const uint32_t S = __ldcg(&p.cnt->sub), top = __ldcg(&p.cnt->node_count);
  for (uint32_t t = blockIdx.x * kLargeBlock + threadIdx.x; t < S && t < p.n + 1u; t += gridDim.x * kLargeBlock) {
    const Task tk = p.subs[t];
    DAabb nd = load_aabb(p.nodes + tk.node);
    if (nd.count >= 0) continue;
    const uint32_t c = (uint32_t)nd.left_first;
    if (c == 0 || c >= p.n) {
      atomicOr(&p.cnt->status, kStatusBadIndex);
      continue;
    }
    nd.left_first = (int32_t)(top + 2u * p.srank[c]);
    store_aabb(p.nodes + tk.node, nd);
  }
}


__global__ void k_sah_init(SahParams p, const DAabb* world) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) p.idx_a[i] = i;
  if (i == 0) {
    store_aabb(p.nodes, *world);
    const Task root{0u, 0u, p.n, 0u};
    if (p.n > p.sub_max) {
      p.large[0][0] = root;
      p.cnt->large = 1;
      p.cnt->sub = 0;
    } else {
      p.subs[0] = root;
      p.cnt->large = 0;
      p.cnt->sub = 1;
    }
    p.cnt->node_count = 1;
    p.cnt->status = 0;
    p.cnt->chunks = 0;
    p.cnt->ticket = 0;
    p.cnt->sub_head = 0;
    p.cnt->sub_splits = 0;
    p.cnt->tiny = 0;
    p.cnt->tiny_head = 0;
  }
}

}  // namespace

ResultCode build_binned_sah(const DAabb* aabbs, const float4* centers, size_t n_, size_t prims_per_leaf,
                            cudaStream_t s, BuildOutput* out) {
  if (n_ == 0) return NoPrimitives;
  if (n_ >= (1u << 30)) return InvalidArgument;
  const uint32_t n = (uint32_t)n_;
  const uint32_t node_cap = 2u * n - 1u;
  cudaError_t e;
  DAabb* nodes = nullptr;
  uint32_t* indices = nullptr;
  if ((e = device_alloc(&nodes, node_cap, s))) return cuda_rc(e);
  if ((e = device_alloc(&indices, n, s))) {
    pool_free(nodes, s);
    return cuda_rc(e);
  }
  auto fail = [&](ResultCode rc) {
    pool_free(nodes, s);
    pool_free(indices, s);
    return rc;
  };
  // The breadth-first part of builds up to kCoopMaxPrims runs as one
  // cooperative launch on the full resident grid: the middle levels hold
  // many small tasks, each binned and partitioned as its own chunk, and a
  // grid sized to the primitive count (one block per 512) left each block
  // a long serial loop of them (6,400 triangles: 0.96 -> 0.73 ms with the
  // full grid; the cheaper barriers of the small grid did not make up for
  // it). Large builds launch the phases separately, which lets each phase
  // run at its own occupancy, and read the level's counts back between
  // levels.
  const bool coop = n <= kCoopMaxPrims;
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coop ? (const void*)k_sah_build
                                                                         : (const void*)k_ph_partition,
                                                         kLargeBlock, coop ? 0 : kShSmall)))
    return fail(cuda_rc(e));
  if (per_sm < 1) return fail(DeviceError);
  const uint32_t grid = (uint32_t)sm_count() * (uint32_t)per_sm;
  uint32_t sub_max = n / 2048u;
  sub_max = sub_max < 32u ? 32u : (sub_max > kWarpMax ? kWarpMax : sub_max);
  const uint32_t large_cap = n / (sub_max + 1) + 2;
  const uint32_t sub_cap = n + 1;
  const uint32_t chunk_cap = n / kChunk + large_cap + 2;
  const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
  Scratch<DAabb> world, tnodes;
  Scratch<uint32_t> acc, idx_b, bins, chunk_base, chunk_status, sflag, srank, tile_off;
  Scratch<Task> large0, large1, subs;
  Scratch<SubTask> tiny;
  Scratch<Decision> dec;
  Scratch<float> tbox;
  Scratch<uint64_t> scan_vals, scan_sums;
  Scratch<Counters> cnt;
  Scratch<GridBarrier> bar;
  if ((e = world.alloc(1, s)) || (e = acc.alloc(8, s)) || (e = idx_b.alloc(n, s)) ||
      (e = bins.alloc((size_t)large_cap * kTaskBinWords, s)) || (e = chunk_base.alloc(large_cap + 1, s)) ||
      (e = chunk_status.alloc(chunk_cap, s)) || (e = large0.alloc(large_cap, s)) || (e = large1.alloc(large_cap, s)) ||
      (e = subs.alloc(sub_cap, s)) || (e = dec.alloc(large_cap, s)) || (e = tbox.alloc((size_t)large_cap * 6, s)) ||
      (e = scan_vals.alloc(large_cap, s)) || (e = scan_sums.alloc(grid, s)) || (e = cnt.alloc(1, s)) ||
      (e = bar.alloc(1, s)) || (e = tnodes.alloc(2 * (size_t)n, s)) || (e = sflag.alloc(n, s)) ||
      (e = srank.alloc(n, s)) || (e = tile_off.alloc(tiles + 1, s)) || (e = tiny.alloc(n, s)))
    return fail(cuda_rc(e));
  if ((e = cudaMemsetAsync(chunk_status.ptr, 0, (size_t)chunk_cap * 4, s)) ||
      (e = cudaMemsetAsync(bar.ptr, 0, sizeof(GridBarrier), s)) ||
      (e = cudaMemsetAsync(sflag.ptr, 0, (size_t)n * 4, s)))
    return fail(cuda_rc(e));
  if ((e = launch_world_bounds(aabbs, n, world.ptr, acc.ptr, s))) return fail(cuda_rc(e));

  SahParams p;
  p.aabbs = aabbs;
  p.centers = centers;
  p.nodes = nodes;
  p.idx_a = indices;
  p.idx_b = idx_b.ptr;
  p.n = n;
  p.sub_max = sub_max;
  p.max_leaf = prims_per_leaf == 0 ? 1u : (uint32_t)(prims_per_leaf > 0xffffffffu ? 0xffffffffu : prims_per_leaf);
  p.large[0] = large0.ptr;
  p.large[1] = large1.ptr;
  p.subs = subs.ptr;
  p.tiny = tiny.ptr;
  p.dec = dec.ptr;
  p.tbox = tbox.ptr;
  p.bins = bins.ptr;
  p.chunk_base = chunk_base.ptr;
  p.chunk_status = chunk_status.ptr;
  p.scan_vals = scan_vals.ptr;
  p.scan_sums = scan_sums.ptr;
  p.tnodes = tnodes.ptr;
  p.sflag = sflag.ptr;
  p.srank = srank.ptr;
  p.tile_off = tile_off.ptr;
  p.cnt = cnt.ptr;
  p.bar = bar.ptr;
  k_sah_init<<<(n + 255) / 256, 256, 0, s>>>(p, world.ptr);
  Counters h{};
  if (n > sub_max) {
    if (coop) {
      // the subtree stage below reads the counts it needs on the device
      void* args[] = {&p};
      if ((e = cudaLaunchCooperativeKernel((void*)k_sah_build, dim3(grid), dim3(kLargeBlock), args, 0, s)))
        return fail(cuda_rc(e));
    } else {
      h.large = 1u;
      const size_t cap = (size_t)grid;
      auto blocks = [cap](size_t need) { return (unsigned)(need < 1 ? 1 : (need < cap ? need : cap)); };
      for (uint32_t level = 0; h.large > 0; ++level) {
        if (level > kMaxDepth + 1) return fail(Error);
        k_ph_prep<<<blocks(((size_t)h.large * 3 * kBins + kLargeBlock - 1) / kLargeBlock), kLargeBlock, kShSmall,
                    s>>>(p, level);
        k_ph_bin<<<grid, kLargeBlock, kShBins, s>>>(p, level);
        k_ph_decide<<<blocks((h.large + 7) / 8), kLargeBlock, kShBins, s>>>(p, level);
        k_ph_partition<<<grid, kLargeBlock, kShSmall, s>>>(p, level);
        k_ph_copyback_scan<<<grid, kLargeBlock, kShSmall, s>>>(p, level);
        k_ph_emit<<<grid, kLargeBlock, kShSmall, s>>>(p, level);
        k_ph_advance<<<1, kLargeBlock, kShSmall, s>>>(p, level, grid);
        if ((e = cudaGetLastError())) return fail(cuda_rc(e));
        if ((e = cudaMemcpyAsync(&h, cnt.ptr, sizeof(Counters), cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s)))
          return fail(cuda_rc(e));
        if (h.status) break;
      }
    }
    if (h.status) return fail(h.status & kStatusTimeout ? Timeout : Error);
    if (h.large > 0) return fail(Error);
  }
  // subtrees, then their node pairs after the breadth-first part (the
  // kernels read the subtree count and the breadth-first node count on the
  // device)
  {
    int sub_per_sm = 0;
    const size_t sub_smem = (kSubBlock / 32) * sizeof(SubShared);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sub_per_sm, k_sub_build, kSubBlock, sub_smem)))
      return fail(cuda_rc(e));
    if (sub_per_sm < 1) return fail(DeviceError);
    uint32_t sub_grid = (uint32_t)sm_count() * (uint32_t)sub_per_sm;
    const uint32_t want = (n / (sub_max > 8u ? 8u : sub_max) + kSubBlock / 32) / (kSubBlock / 32) + 1u;
    if (want < sub_grid) sub_grid = want;
    k_sub_build<<<sub_grid, kSubBlock, sub_smem, s>>>(p);
    {
      int tiny_per_sm = 0;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tiny_per_sm, k_sub_tiny, kLargeBlock, 0)))
        return fail(cuda_rc(e));
      const uint32_t tiny_grid = (uint32_t)sm_count() * (uint32_t)(tiny_per_sm < 1 ? 1 : tiny_per_sm);
      k_sub_tiny<<<tiny_grid, kLargeBlock, 0, s>>>(p);
    }
    k_tile_sums<<<tiles, 1024, 0, s>>>(sflag.ptr, n, tile_off.ptr);
    k_tile_scan<<<1, 1024, 0, s>>>(tile_off.ptr, tiles, cnt.ptr);
    k_rank<<<tiles, 1024, 0, s>>>(sflag.ptr, n, tile_off.ptr, srank.ptr);
    k_relocate<<<(n + kLargeBlock - 1) / kLargeBlock, kLargeBlock, 0, s>>>(p);
    const unsigned fix_blocks = (unsigned)((n + kLargeBlock) / kLargeBlock);
    k_fix_roots<<<fix_blocks < (unsigned)sm_count() * 4u ? fix_blocks : (unsigned)sm_count() * 4u, kLargeBlock, 0,
                  s>>>(p);
    if ((e = cudaGetLastError())) return fail(cuda_rc(e));
    if ((e = cudaMemcpyAsync(&h, cnt.ptr, sizeof(Counters), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return fail(cuda_rc(e));
    if (h.status) return fail(h.status & kStatusTimeout ? Timeout : Error);
    if (h.large > 0) return fail(Error);  // the breadth-first part did not finish
  }
  const uint64_t total = (uint64_t)h.node_count + 2ull * h.sub_splits;
  if (total > node_cap) return fail(Error);
  out->nodes = nodes;
  out->indices = indices;
  out->node_count = (uint32_t)total;
  return Ok;
}

}  // namespace rtbvh
