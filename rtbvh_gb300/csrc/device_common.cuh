// Device-side building blocks shared by the build and traversal kernels.
//
// Every translation unit that includes this file is compiled with
// --fmad=false and IEEE division/sqrt, so plain float expressions round
// exactly like the reference's scalar Rust code (no contraction into FMA).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rtbvh {

// ------------------------------------------------------------- status words
// Bits a kernel ORs into its status word instead of trapping.
enum DeviceStatus : uint32_t {
  kStatusOk = 0,
  kStatusTimeout = 1u << 0,        // a bounded spin gave up
  kStatusStackOverflow = 1u << 1,  // a traversal stack bound was hit
  kStatusNoMerge = 1u << 2,        // a clustering level merged nothing
  kStatusBadIndex = 1u << 3,       // an index failed its bounds check
  kStatusNoNeighbour = 1u << 4,    // a cluster found no neighbour
};

// Spin budget of every device-side wait: ~2^22 polls with a 256 ns back-off,
// i.e. about a second, after which the waiter sets kStatusTimeout and leaves.
constexpr uint32_t kSpinLimit = 1u << 22;

// ------------------------------------------------------------- node layouts
// RTAabb / BvhNode (src/aabb.rs:13-20): min, count(extra1), max, left_first(extra2).
struct alignas(16) DAabb {
  float min[3];
  int32_t count;
  float max[3];
  int32_t left_first;
};
static_assert(sizeof(DAabb) == 32, "DAabb must be 32 bytes");

// RTMbvhNode (src/mbvh_node.rs:29-38).
struct alignas(128) DMNode {
  float min_x[4], max_x[4], min_y[4], max_y[4], min_z[4], max_z[4];
  int32_t children[4];
  int32_t counts[4];
};
static_assert(sizeof(DMNode) == 128, "DMNode must be 128 bytes");

// Half-size copy of a quad node for the closest-hit traversal. Per axis the
// four slot boxes are stored as 8-bit steps on a power-of-two grid starting
// at lo[axis], rounded outwards, so every decoded box contains the exact one;
// children and counts are exact (counts as int16). A closest-hit traversal
// over boxes that contain the reference's finds the same nearest triangle
// (only its visit order, and so the winner among triangles hit at exactly
// the same t, can differ). Flags (exps >> 24): kQFlagExact -- the bounds do
// not fit the grid (or a count not int16), read the exact node instead;
// kQFlagOutOfRange -- a bound beyond kCompactRange, the ray leaves the
// compact walk and is traced again over the exact Mbvh.
struct alignas(64) DQNode {
  float lo[3];
  uint32_t exps;          // biased exponents of the steps: x | y << 8 | z << 16 | flags << 24
  uint32_t qx[2], qy[2];  // [0] lower bounds, [1] upper bounds; slot i in byte i
  uint32_t qz[2];
  int32_t children[4];
  int16_t counts[4];
};
static_assert(sizeof(DQNode) == 64, "DQNode must be 64 bytes");
// The boxes of a quad node's four slots computed from their subtrees'
// triangles (each triangle's vertex box grown by 1e-4, united up the
// subtree), for the exact-order walk of binned-SAH trees, whose own slot
// boxes can miss triangles: a slot whose subtree box the ray cannot enter
// below its current t holds no hit. Slots with a bound beyond
// kCompactRange (or a NaN) get the infinite box, which every finite ray
// enters. Three 256-bit loads.
struct alignas(32) DTBox {
  float min_x[4], max_x[4], min_y[4], max_y[4], min_z[4], max_z[4];
};
static_assert(sizeof(DTBox) == 96, "DTBox must be 96 bytes");
constexpr uint32_t kQFlagExact = 1u;
constexpr uint32_t kQFlagOutOfRange = 2u;
constexpr float kQuantRange = 1e18f;  // larger inverse-direction components use the exact nodes
// Magnitude bound of the compact walk: ray origins and node bounds within
// +-kCompactRange. Every leaf box of the trees that get a traversal tree is
// its primitive's box grown by 1e-4, and below this magnitude the rounding of
// a slab test, about 2^-23 * (|bound| + |origin|) <= 3.1e-5 in space, stays
// well inside that margin: a box that holds a triangle hit by the ray passes
// the test in both the compact (one fma per plane) and the exact (subtract,
// multiply) arithmetic, and a box that one form rejects and the other keeps
// holds no nearer hit. Beyond it the two forms can disagree on a box that
// matters, so such rays and nodes use the exact Mbvh in the reference's order.
constexpr float kCompactRange = 128.0f;

// ------------------------------------------------------------- float helpers
// Vec3::min / Vec3::max of the reference (Rust f32::min/max): NaN operands are
// ignored; on a -0/+0 tie min gives -0 and max gives +0 (order-independent).
__device__ __forceinline__ float rs_min(float a, float b) {
  float r = fminf(a, b);
  if (a == b) r = __int_as_float(__float_as_int(a) | __float_as_int(b));
  return r;
}
__device__ __forceinline__ float rs_max(float a, float b) {
  float r = fmaxf(a, b);
  if (a == b) r = __int_as_float(__float_as_int(a) & __float_as_int(b));
  return r;
}
// _mm_min_ps / _mm_max_ps: the second operand wins on NaN or equality.
__device__ __forceinline__ float sse_min(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float sse_max(float a, float b) { return a > b ? a : b; }

// Order-preserving map of floats to uint32 (-0 sorts below +0) for atomic
// min/max reductions.
__device__ __forceinline__ uint32_t float_to_ordered(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Aabb::half_area (src/aabb.rs:342-346), no FMA.
__device__ __forceinline__ float half_area(float mnx, float mny, float mnz, float mxx, float mxy, float mxz) {
  float d0 = mxx - mnx, d1 = mxy - mny, d2 = mxz - mnz;
  float t = (d0 + d1) * d2;
  float u = d0 * d1;
  return t + u;
}

__device__ __forceinline__ DAabb load_aabb(const DAabb* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  float4 a = __ldg(q), b = __ldg(q + 1);
  DAabb r;
  r.min[0] = a.x; r.min[1] = a.y; r.min[2] = a.z; r.count = __float_as_int(a.w);
  r.max[0] = b.x; r.max[1] = b.y; r.max[2] = b.z; r.left_first = __float_as_int(b.w);
  return r;
}
// Load that bypasses L1 (data written by other blocks of the same launch).
__device__ __forceinline__ DAabb load_aabb_cg(const DAabb* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  float4 a = __ldcg(q), b = __ldcg(q + 1);
  DAabb r;
  r.min[0] = a.x; r.min[1] = a.y; r.min[2] = a.z; r.count = __float_as_int(a.w);
  r.max[0] = b.x; r.max[1] = b.y; r.max[2] = b.z; r.left_first = __float_as_int(b.w);
  return r;
}
__device__ __forceinline__ void store_aabb(DAabb* p, const DAabb& r) {
  float4* q = reinterpret_cast<float4*>(p);
  q[0] = make_float4(r.min[0], r.min[1], r.min[2], __int_as_float(r.count));
  q[1] = make_float4(r.max[0], r.max[1], r.max[2], __int_as_float(r.left_first));
}

// ------------------------------------------------------------- grid barrier
// Sense-counting barrier for cooperative launches. Waits are bounded: on
// timeout the status word gets kStatusTimeout and the caller must return.
struct GridBarrier {
  unsigned int count;
  unsigned int generation;
};

__device__ __forceinline__ bool grid_sync(GridBarrier* bar, unsigned int nblocks, uint32_t* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int* vgen = &bar->generation;
    unsigned int gen = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd(&bar->count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->generation, 1u);
    } else {
      uint32_t it = 0;
      while (*vgen == gen) {
        if (++it > kSpinLimit) {
          atomicOr(status, kStatusTimeout);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (ok && (*(volatile uint32_t*)status & kStatusTimeout)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ------------------------------------------------------------- block scan
// Inclusive scan of one value per thread over a block of BLOCK threads.
template <int BLOCK>
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = BLOCK / 32;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  if (lane == 31) s_warp[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < NW ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t n = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += n;
    }
    if (lane < NW) s_warp[lane] = w;
  }
  __syncthreads();
  uint32_t prefix = warp > 0 ? s_warp[warp - 1] : 0u;
  uint32_t t = s_warp[NW - 1];
  __syncthreads();
  if (total) *total = t;
  return v + prefix;
}

}  // namespace rtbvh
