// Binned SAH build (src/builders/binned_sah.rs) on the GPU, breadth first.
//
// The reference runs one task per node (BinnedSahBuildTask::run,
// binned_sah.rs:132-282) from a depth-first work stack. Here every level of
// the tree is one round of kernels over all of that level's tasks:
//
//   large tasks (more than kWarpMax primitives): a grid of 2048-primitive
//     chunks bins into per-task global bins (exact min/max via ordered-int
//     atomics, counts via atomicAdd), one thread per task decides the split,
//     and a chunked stable partition (decoupled look-back over the chunks of
//     a task, bounded waits) scatters the primitive indices;
//   small tasks: one warp per task bins in shared memory, decides and
//     partitions in place;
//   then a scan over the level's tasks numbers the children (breadth-first,
//     deterministic) and builds the next level's task lists.
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
constexpr int kSmallWarps = 4;
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
  uint32_t small;       // tasks in the current small list
  uint32_t node_count;  // nodes allocated so far
  uint32_t chunks;      // chunks of the current large list
  uint32_t status;
  uint32_t ticket;      // chunk ticket of the partition kernel
  uint32_t mq_count;    // small tasks of more than kThreadMax primitives queued this level
  uint32_t mq_head;     // next queued task a warp takes
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

// Bins stored as ordered keys (global or shared memory).
struct BinsView {
  const uint32_t* w;  // kTaskBinWords words
  __device__ __forceinline__ float mn(int a, int i, int k) const { return ordered_to_float(w[(a * kBins + i) * kBinWords + k]); }
  __device__ __forceinline__ float mx(int a, int i, int k) const {
    return ordered_to_float(w[(a * kBins + i) * kBinWords + 3 + k]);
  }
  __device__ __forceinline__ uint32_t cnt(int a, int i) const { return w[(a * kBins + i) * kBinWords + 6]; }
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
  Task* large;
  Task* small;
  Task* large_next;
  Task* small_next;
  Decision* dec;        // [large tasks | small tasks]
  float* tbox;          // 6 floats per large task (box with first offset)
  uint32_t* bins;       // kTaskBinWords per large task
  uint32_t* chunk_base; // large + 1
  uint32_t* chunk_status;
  uint64_t* scan_vals;  // per task of the level
  uint64_t* scan_sums;
  uint32_t* mqueue;     // small-task indices for one warp each (small_cap)
  Counters* cnt;
};

// ------------------------------------------------------------------ large tasks
// Per level, before binning: task boxes, zeroed bins, chunk offsets.
__global__ void __launch_bounds__(1024) k_large_prep(SahParams p) {
  __shared__ uint32_t s_warp[32];
  const uint32_t L = p.cnt->large;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < L || base == 0; base += 1024) {
    const uint32_t t = base + threadIdx.x;
    uint32_t chunks = 0;
    if (t < L) {
      const Task tk = p.large[t];
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
    uint32_t incl = block_inclusive_scan<1024>(chunks, s_warp, &total);
    if (t < L) p.chunk_base[t] = carry + incl - chunks;
    carry += total;
    if (base + 1024 >= L) break;
  }
  if (threadIdx.x == 0) {
    p.chunk_base[L] = carry;
    p.cnt->chunks = carry;
    p.cnt->ticket = 0;
  }
}

// Empty bins for every large task of the level (one bin per thread).
__global__ void __launch_bounds__(256) k_bins_init(SahParams p) {
  const uint32_t L = p.cnt->large;
  const uint32_t kmin = float_to_ordered(1e34f), kmax = float_to_ordered(-1e34f);
  const size_t total = (size_t)L * 3 * kBins;
  for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < total; i += (size_t)gridDim.x * 256) {
    uint4* b = reinterpret_cast<uint4*>(p.bins + i * kBinWords);
    b[0] = make_uint4(kmin, kmin, kmin, kmax);
    b[1] = make_uint4(kmax, kmax, 0u, 0u);
  }
}

__device__ __forceinline__ uint32_t find_task(const uint32_t* chunk_base, uint32_t L, uint32_t chunk) {
  uint32_t lo = 0, hi = L;  // last t with chunk_base[t] <= chunk
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(chunk_base + mid) <= chunk) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kLargeBlock) k_large_bin(SahParams p) {
  constexpr int NW = kLargeBlock / 32;
  __shared__ uint32_t s_bins[NW][kTaskBinWords];
  const int warp = threadIdx.x >> 5;
  const uint32_t L = p.cnt->large;
  const uint32_t chunk = blockIdx.x;
  const uint32_t t = find_task(p.chunk_base, L, chunk);
  const Task tk = p.large[t];
  const uint32_t k = chunk - p.chunk_base[t];
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  init_bins(&s_bins[warp][0], threadIdx.x & 31, 32);
  __syncthreads();
  float mn[3], mx[3];
  const float* tb = p.tbox + 6 * (size_t)t;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    mn[a] = tb[a];
    mx[a] = tb[3 + a];
  }
  const BinMap bm = make_binmap(mn, mx);
  uint32_t* wb = &s_bins[warp][0];
  for (uint32_t i = c0 + threadIdx.x; i < c1; i += kLargeBlock) {
    const uint32_t prim = __ldg(p.idx_a + i);
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
      uint32_t* b = wb + (a * kBins + bin_of(cc[a], bm.c2b[a], bm.off[a])) * kBinWords;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        atomicMin(b + q, kmn[q]);
        atomicMax(b + 3 + q, kmx[q]);
      }
      atomicAdd(b + 6, 1u);
    }
  }
  __syncthreads();
  uint32_t* gb = p.bins + (size_t)t * kTaskBinWords;
  for (int i = threadIdx.x; i < 3 * kBins; i += kLargeBlock) {
    uint32_t cnt = 0;
    uint32_t vmn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, vmx[3] = {0u, 0u, 0u};
    for (int w = 0; w < NW; ++w) {
      const uint32_t* b = &s_bins[w][i * kBinWords];
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
}

// One warp per large task.
__global__ void __launch_bounds__(128) k_large_decide(SahParams p) {
  const uint32_t t = (blockIdx.x * 128 + threadIdx.x) >> 5;
  const uint32_t L = p.cnt->large;
  if (t >= L) return;
  const Task tk = p.large[t];
  float mn[3], mx[3];
  const float* tb = p.tbox + 6 * (size_t)t;
  for (int a = 0; a < 3; ++a) {
    mn[a] = tb[a];
    mx[a] = tb[3 + a];
  }
  Decision d;
  d.split = 0;
  const uint32_t ws = tk.end - tk.begin;
  if (ws > 1 && tk.depth < kMaxDepth) {
    BinsView B{p.bins + (size_t)t * kTaskBinWords};
    sah_decide_warp(B, mn, mx, ws, p.max_leaf, d);
  }
  if ((threadIdx.x & 31) == 0) {
    if (d.split) write_interior_box(p.nodes, tk.node, mn, mx);
    else write_leaf(p.nodes, tk, mn, mx);
    p.dec[t] = d;
  }
}

// Stable partition of a large task's chunk into idx_b; the number of left
// primitives in the task's earlier chunks comes from a decoupled look-back.
__global__ void __launch_bounds__(kLargeBlock) k_large_partition(SahParams p) {
  __shared__ uint32_t s_chunk, s_fail, s_prefix;
  __shared__ uint32_t s_warp[kLargeBlock / 32];
  const uint32_t L = p.cnt->large;
  if (threadIdx.x == 0) {
    s_chunk = atomicAdd(&p.cnt->ticket, 1u);
    s_fail = 0;
  }
  __syncthreads();
  const uint32_t chunk = s_chunk;
  const uint32_t t = find_task(p.chunk_base, L, chunk);
  const Decision d = p.dec[t];
  if (!d.split) return;  // no chunk of this task waits on another
  const Task tk = p.large[t];
  const uint32_t first_chunk = p.chunk_base[t];
  const uint32_t k = chunk - first_chunk;
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  float mn[3], mx[3];
  const float* tb = p.tbox + 6 * (size_t)t;
  for (int a = 0; a < 3; ++a) {
    mn[a] = tb[a];
    mx[a] = tb[3 + a];
  }
  const BinMap bm = make_binmap(mn, mx);
  const int ax = (int)d.axis;
  // each thread owns kChunk / kLargeBlock consecutive primitives
  constexpr int PER = kChunk / kLargeBlock;
  uint32_t prim[PER];
  uint32_t flags = 0, mine = 0;
  const uint32_t s = c0 + threadIdx.x * PER;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const uint32_t i = s + j;
    prim[j] = 0;
    if (i < c1) {
      prim[j] = __ldg(p.idx_a + i);
      const float4 c = __ldg(p.centers + prim[j]);
      const float cc = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
      if (bin_of(cc, bm.c2b[ax], bm.off[ax]) < d.split_index) {
        flags |= 1u << j;
        ++mine;
      }
    }
  }
  uint32_t chunk_true;
  const uint32_t incl = block_inclusive_scan<kLargeBlock>(mine, s_warp, &chunk_true);
  const uint32_t before_me = incl - mine;
  volatile uint32_t* st = p.chunk_status;
  if (threadIdx.x == 0) {
    uint32_t excl = 0;
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
            s_fail = 1;
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
    s_prefix = excl;
  }
  __syncthreads();
  if (s_fail) return;
  const uint32_t true_before = s_prefix + before_me;
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

__global__ void __launch_bounds__(kLargeBlock) k_large_copyback(SahParams p) {
  const uint32_t L = p.cnt->large;
  const uint32_t chunk = blockIdx.x;
  const uint32_t t = find_task(p.chunk_base, L, chunk);
  if (!p.dec[t].split) return;
  const Task tk = p.large[t];
  const uint32_t k = chunk - p.chunk_base[t];
  const uint32_t c0 = tk.begin + k * kChunk;
  const uint32_t c1 = min(c0 + kChunk, tk.end);
  for (uint32_t i = c0 + threadIdx.x; i < c1; i += kLargeBlock) p.idx_a[i] = p.idx_b[i];
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

__device__ void small_task_thread(const SahParams& p, uint32_t t, uint32_t L) {
  const Task tk = p.small[t];
  const uint32_t ws = tk.end - tk.begin;
  float mn[3], mx[3];
  task_box(p.nodes, tk.node, mn, mx);
  Decision d;
  d.split = 0;
  if (ws > 1 && tk.depth < kMaxDepth) {
    uint32_t prim[kThreadMax];
    uint32_t kb[kThreadMax][6];
    uint32_t packed[3] = {0u, 0u, 0u};
    const BinMap bm = make_binmap(mn, mx);
#pragma unroll
    for (uint32_t j = 0; j < kThreadMax; ++j) {
      if (j < ws) {
        prim[j] = __ldg(p.idx_a + tk.begin + j);
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
        // stable partition (left primitives first, in order)
        uint32_t tpos = tk.begin, fpos = tk.begin + n_left;
#pragma unroll
        for (uint32_t j = 0; j < kThreadMax; ++j) {
          if (j < ws) p.idx_a[((left >> j) & 1u) ? tpos++ : fpos++] = prim[j];
        }
      }
    }
  }
  if (d.split) write_interior_box(p.nodes, tk.node, mn, mx);
  else write_leaf(p.nodes, tk, mn, mx);
  p.dec[L + t] = d;
}

// A small task of more than kThreadMax primitives, by one warp: bins in
// shared memory, the warp-parallel decision, a ballot-based stable partition.
__device__ void small_task_warp(const SahParams& p, uint32_t t, uint32_t L, uint32_t* wb, uint32_t* sidx,
                                Decision& d) {
  const int lane = threadIdx.x & 31;
  const Task tk = p.small[t];
  const uint32_t ws = tk.end - tk.begin;
  float mn[3], mx[3];
  task_box(p.nodes, tk.node, mn, mx);
  if (lane == 0) d.split = 0;
  __syncwarp();
  if (ws > 1 && tk.depth < kMaxDepth && ws <= kWarpMax) {
    init_bins(wb, lane, 32);
    __syncwarp();
    const BinMap bm = make_binmap(mn, mx);
    for (uint32_t i = lane; i < ws; i += 32) {
      const uint32_t prim = __ldg(p.idx_a + tk.begin + i);
      const float4 c = __ldg(p.centers + prim);
      const DAabb box = load_aabb(p.aabbs + prim);
      const float cc[3] = {c.x, c.y, c.z};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        uint32_t* b = wb + (a * kBins + bin_of(cc[a], bm.c2b[a], bm.off[a])) * kBinWords;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          atomicMin(b + q, float_to_ordered(box.min[q]));
          atomicMax(b + 3 + q, float_to_ordered(box.max[q]));
        }
        atomicAdd(b + 6, 1u);
      }
    }
    __syncwarp();
    {
      BinsView B{wb};
      Decision dl;
      sah_decide_warp(B, mn, mx, ws, p.max_leaf, dl);
      if (lane == 0) d = dl;
    }
    __syncwarp();
    if (d.split) {
      const int ax = (int)d.axis;
      const uint32_t lt = (1u << lane) - 1u;
      uint32_t tb = 0, fb = 0;
      for (uint32_t c0 = 0; c0 < ws; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool valid = i < ws;
        uint32_t prim = 0;
        bool pred = false;
        if (valid) {
          prim = p.idx_a[tk.begin + i];
          const float4 c = __ldg(p.centers + prim);
          const float cc = ax == 0 ? c.x : (ax == 1 ? c.y : c.z);
          pred = bin_of(cc, bm.c2b[ax], bm.off[ax]) < d.split_index;
        }
        const uint32_t T = __ballot_sync(0xffffffffu, pred);
        const uint32_t V = __ballot_sync(0xffffffffu, valid);
        const uint32_t F = V & ~T;
        if (pred) sidx[tb + __popc(T & lt)] = prim;
        else if (valid) {
          const uint32_t dst = d.n_left + fb + __popc(F & lt);
          if (dst < kWarpMax) sidx[dst] = prim;
        }
        tb += __popc(T);
        fb += __popc(F);
      }
      __syncwarp();
      for (uint32_t i = lane; i < ws; i += 32) p.idx_a[tk.begin + i] = sidx[i];
    }
  }
  __syncwarp();
  if (lane == 0) {
    if (d.split) write_interior_box(p.nodes, tk.node, mn, mx);
    else write_leaf(p.nodes, tk, mn, mx);
    p.dec[L + t] = d;
  }
  __syncwarp();
}

// Each thread takes one small task: tasks of at most kThreadMax primitives
// (and leaves) are done at once; the others are queued for one warp each
// (k_small_warps). The order in which queued tasks run does not matter: each
// writes only its own node, index range and decision slot.
__global__ void __launch_bounds__(128) k_small(SahParams p) {
  const uint32_t S = p.cnt->small, L = p.cnt->large;
  const uint32_t t = blockIdx.x * 128 + threadIdx.x;
  bool big = false;
  if (t < S) {
    const Task tk = p.small[t];
    const uint32_t ws = tk.end - tk.begin;
    big = ws > kThreadMax && tk.depth < kMaxDepth;
    if (!big) small_task_thread(p, t, L);
  }
  const uint32_t m = __ballot_sync(0xffffffffu, big);
  if (m) {
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(&p.cnt->mq_count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (big) p.mqueue[base + __popc(m & ((1u << lane) - 1u))] = t;
  }
}

// Persistent: every warp takes queued small tasks until the queue is empty.
__global__ void __launch_bounds__(32 * kSmallWarps) k_small_warps(SahParams p) {
  __shared__ uint32_t s_bins[kSmallWarps][kTaskBinWords];
  __shared__ uint32_t s_idx[kSmallWarps][kWarpMax];
  __shared__ Decision s_dec[kSmallWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t Q = p.cnt->mq_count, L = p.cnt->large;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(&p.cnt->mq_head, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= Q) break;
    small_task_warp(p, __ldg(p.mqueue + q), L, &s_bins[warp][0], &s_idx[warp][0], s_dec[warp]);
  }
}

// ------------------------------------------------------------------ level scan + emit
__device__ __forceinline__ uint64_t children_value(const Decision& d, const Task& tk) {
  if (!d.split) return 0;
  const uint32_t ws = tk.end - tk.begin;
  const uint32_t nl = d.n_left, nr = ws - d.n_left;
  const uint64_t large = (uint64_t)(nl > kWarpMax) + (uint64_t)(nr > kWarpMax);
  return (large << 32) | (uint64_t)(2u - (uint32_t)large);
}

__device__ __forceinline__ Task level_task(const SahParams& p, uint32_t t, uint32_t L) {
  return t < L ? p.large[t] : p.small[t - L];
}

constexpr int kScanBlock = 256;
constexpr int kScanItems = 4;

template <class T>
__device__ __forceinline__ T block_scan_incl(T v, T* s_warp, T* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = kScanBlock / 32;
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

// Stage 1: values and per-block exclusive scans.
__global__ void __launch_bounds__(kScanBlock) k_scan_local(SahParams p) {
  __shared__ uint64_t s_warp[kScanBlock / 32];
  const uint32_t L = p.cnt->large, N = L + p.cnt->small;
  const uint32_t base = blockIdx.x * kScanBlock * kScanItems + threadIdx.x * kScanItems;
  uint64_t v[kScanItems], sum = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t t = base + j;
    v[j] = 0;
    if (t < N) v[j] = children_value(p.dec[t], level_task(p, t, L));
    sum += v[j];
  }
  uint64_t total;
  uint64_t incl = block_scan_incl<uint64_t>(sum, s_warp, &total);
  uint64_t run = incl - sum;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t t = base + j;
    if (t < N) p.scan_vals[t] = run;
    run += v[j];
  }
  if (threadIdx.x == 0) p.scan_sums[blockIdx.x] = total;
}

// Stage 2: one block scans the block sums (exclusive, total at [nb]).
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(SahParams p, uint32_t nb) {
  __shared__ uint64_t s_warp[kScanBlock / 32];
  uint64_t carry = 0;
  for (uint32_t base = 0; base < nb; base += kScanBlock) {
    const uint32_t i = base + threadIdx.x;
    uint64_t v = i < nb ? p.scan_sums[i] : 0;
    uint64_t total;
    uint64_t incl = block_scan_incl<uint64_t>(v, s_warp, &total);
    if (i < nb) p.scan_sums[i] = carry + incl - v;
    carry += total;
  }
  if (threadIdx.x == 0) p.scan_sums[nb] = carry;
}

// Stage 3: node numbering and the next level's task lists.
__global__ void __launch_bounds__(kScanBlock) k_emit(SahParams p, uint32_t nb) {
  const uint32_t L = p.cnt->large, N = L + p.cnt->small;
  const uint32_t t = blockIdx.x * kScanBlock + threadIdx.x;
  const uint64_t total = p.scan_sums[nb];
  const uint32_t node_base = p.cnt->node_count;
  if (t < N) {
    const Decision d = p.dec[t];
    if (d.split) {
      const Task tk = level_task(p, t, L);
      const uint64_t ex = p.scan_vals[t] + p.scan_sums[t / (kScanBlock * kScanItems)];
      uint32_t li = (uint32_t)(ex >> 32), si = (uint32_t)(ex & 0xffffffffu);
      const uint32_t child = node_base + li + si;
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
      if (lt.end - lt.begin > kWarpMax) p.large_next[li++] = lt;
      else p.small_next[si++] = lt;
      if (rt.end - rt.begin > kWarpMax) p.large_next[li++] = rt;
      else p.small_next[si++] = rt;
    }
  }
  if (t == 0) {
    // every block reads cnt before thread 0 of block 0 could change it: the
    // counters are advanced by k_advance after this kernel.
    (void)total;
  }
}

__global__ void k_advance(SahParams p, uint32_t nb) {
  if (threadIdx.x == 0) {
    const uint64_t total = p.scan_sums[nb];
    const uint32_t nl = (uint32_t)(total >> 32), ns = (uint32_t)(total & 0xffffffffu);
    p.cnt->node_count += nl + ns;
    p.cnt->large = nl;
    p.cnt->small = ns;
    p.cnt->mq_count = 0;
    p.cnt->mq_head = 0;
  }
}

__global__ void k_sah_init(SahParams p, const DAabb* world) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) p.idx_a[i] = i;
  if (i == 0) {
    store_aabb(p.nodes, *world);
    const Task root{0u, 0u, p.n, 0u};
    if (p.n > kWarpMax) {
      p.large[0] = root;
      p.cnt->large = 1;
      p.cnt->small = 0;
    } else {
      p.small[0] = root;
      p.cnt->large = 0;
      p.cnt->small = 1;
    }
    p.cnt->node_count = 1;
    p.cnt->status = 0;
    p.cnt->chunks = 0;
    p.cnt->ticket = 0;
    p.cnt->mq_count = 0;
    p.cnt->mq_head = 0;
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
  if ((e = cudaMalloc(&nodes, (size_t)node_cap * sizeof(DAabb)))) return cuda_rc(e);
  if ((e = cudaMalloc(&indices, (size_t)n * 4))) {
    cudaFree(nodes);
    return cuda_rc(e);
  }
  auto fail = [&](ResultCode rc) {
    cudaFree(nodes);
    cudaFree(indices);
    return rc;
  };
  const uint32_t large_cap = n / (kWarpMax + 1) + 2;
  const uint32_t small_cap = n + 1;
  const uint32_t task_cap = large_cap + small_cap;
  const uint32_t chunk_cap = n / kChunk + large_cap + 2;
  Scratch<DAabb> world;
  Scratch<uint32_t> acc, idx_b, bins, chunk_base, chunk_status;
  Scratch<Task> large0, large1, small0, small1;
  Scratch<Decision> dec;
  Scratch<float> tbox;
  Scratch<uint64_t> scan_vals, scan_sums;
  Scratch<Counters> cnt;
  Scratch<uint32_t> mqueue;
  const uint32_t scan_blocks_cap = (task_cap + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems) + 1;
  if ((e = world.alloc(1, s)) || (e = acc.alloc(8, s)) || (e = idx_b.alloc(n, s)) ||
      (e = bins.alloc((size_t)large_cap * kTaskBinWords, s)) || (e = chunk_base.alloc(large_cap + 1, s)) ||
      (e = chunk_status.alloc(chunk_cap, s)) || (e = large0.alloc(large_cap, s)) || (e = large1.alloc(large_cap, s)) ||
      (e = small0.alloc(small_cap, s)) || (e = small1.alloc(small_cap, s)) || (e = dec.alloc(task_cap, s)) ||
      (e = tbox.alloc((size_t)large_cap * 6, s)) || (e = scan_vals.alloc(task_cap, s)) ||
      (e = scan_sums.alloc(scan_blocks_cap + 1, s)) || (e = cnt.alloc(1, s)) || (e = mqueue.alloc(small_cap, s)))
    return fail(cuda_rc(e));
  if ((e = launch_world_bounds(aabbs, n, world.ptr, acc.ptr, s))) return fail(cuda_rc(e));

  SahParams p;
  p.aabbs = aabbs;
  p.centers = centers;
  p.nodes = nodes;
  p.idx_a = indices;
  p.idx_b = idx_b.ptr;
  p.n = n;
  p.max_leaf = prims_per_leaf == 0 ? 1u : (uint32_t)(prims_per_leaf > 0xffffffffu ? 0xffffffffu : prims_per_leaf);
  p.large = large0.ptr;
  p.small = small0.ptr;
  p.large_next = large1.ptr;
  p.small_next = small1.ptr;
  p.dec = dec.ptr;
  p.tbox = tbox.ptr;
  p.bins = bins.ptr;
  p.chunk_base = chunk_base.ptr;
  p.chunk_status = chunk_status.ptr;
  p.scan_vals = scan_vals.ptr;
  p.scan_sums = scan_sums.ptr;
  p.mqueue = mqueue.ptr;
  p.cnt = cnt.ptr;
  int small_warp_blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&small_warp_blocks, k_small_warps, 32 * kSmallWarps, 0);
  if (small_warp_blocks < 1) small_warp_blocks = 1;
  k_sah_init<<<(n + 255) / 256, 256, 0, s>>>(p, world.ptr);
  k_large_prep<<<1, 1024, 0, s>>>(p);
  Counters h{};
  if ((e = cudaMemcpyAsync(&h, cnt.ptr, sizeof(Counters), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return fail(cuda_rc(e));
  for (uint32_t level = 0; level <= kMaxDepth + 1 && (h.large + h.small) > 0; ++level) {
    if (h.large > 0) {
      const size_t nbins = (size_t)h.large * 3 * kBins;
      const size_t ib = (nbins + 255) / 256, icap = (size_t)sm_count() * 8;
      k_bins_init<<<(unsigned)(ib < icap ? ib : icap), 256, 0, s>>>(p);
      k_large_bin<<<h.chunks, kLargeBlock, 0, s>>>(p);
      k_large_decide<<<(h.large + 3) / 4, 128, 0, s>>>(p);
      if ((e = cudaMemsetAsync(chunk_status.ptr, 0, (size_t)h.chunks * 4, s))) return fail(cuda_rc(e));
      k_large_partition<<<h.chunks, kLargeBlock, 0, s>>>(p);
      k_large_copyback<<<h.chunks, kLargeBlock, 0, s>>>(p);
    }
    if (h.small > 0) {
      k_small<<<(h.small + 127) / 128, 128, 0, s>>>(p);
      // at most one queued task per 9 primitives of the level's small tasks
      const size_t wcap = (size_t)sm_count() * small_warp_blocks, wneed = (h.small + kSmallWarps - 1) / kSmallWarps;
      k_small_warps<<<(unsigned)(wneed < wcap ? wneed : wcap), 32 * kSmallWarps, 0, s>>>(p);
    }
    const uint32_t N = h.large + h.small;
    const uint32_t nb = (N + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
    k_scan_local<<<nb, kScanBlock, 0, s>>>(p);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(p, nb);
    k_emit<<<(N + kScanBlock - 1) / kScanBlock, kScanBlock, 0, s>>>(p, nb);
    k_advance<<<1, 32, 0, s>>>(p, nb);
    std::swap(p.large, p.large_next);
    std::swap(p.small, p.small_next);
    k_large_prep<<<1, 1024, 0, s>>>(p);
    if ((e = cudaGetLastError())) return fail(cuda_rc(e));
    if ((e = cudaMemcpyAsync(&h, cnt.ptr, sizeof(Counters), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return fail(cuda_rc(e));
    if (h.status) return fail(h.status & kStatusTimeout ? Timeout : Error);
  }
  if (h.large + h.small > 0) return fail(Error);
  out->nodes = nodes;
  out->indices = indices;
  out->node_count = h.node_count;
  return Ok;
}

}  // namespace rtbvh
