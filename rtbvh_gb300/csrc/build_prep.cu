// Primitive preparation for the builds: boxes and centres of triangles or
// points, the world box, 30-bit Morton codes and the leaf-ordered triangle
// layout used by the traversal kernels.
#include <mutex>
#include <vector>

#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kPrepBlock = 256;

// shared/src/lib.rs:27-39 -- Aabb::empty() grown by v0, v1, v2; centre
// ((v0 + v1) + v2) * (1/3).
__global__ void __launch_bounds__(kPrepBlock)
    k_triangle_prep(const float* __restrict__ v, size_t n, DAabb* __restrict__ aabbs, float4* __restrict__ centers) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* t = v + 9 * i;
  float p[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) p[k] = __ldg(t + k);
  DAabb b;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float mn = 1e34f, mx = -1e34f;
    mn = rs_min(mn, p[a]);
    mx = rs_max(mx, p[a]);
    mn = rs_min(mn, p[3 + a]);
    mx = rs_max(mx, p[3 + a]);
    mn = rs_min(mn, p[6 + a]);
    mx = rs_max(mx, p[6 + a]);
    b.min[a] = mn;
    b.max[a] = mx;
  }
  b.count = 0;
  b.left_first = 0;
  store_aabb(aabbs + i, b);
  const float third = 1.0f / 3.0f;
  float cx = ((p[0] + p[3]) + p[6]) * third;
  float cy = ((p[1] + p[4]) + p[7]) * third;
  float cz = ((p[2] + p[5]) + p[8]) * third;
  centers[i] = make_float4(cx, cy, cz, 0.0f);
}

// rtbvh_ffi/src/lib.rs:396-422 -- Vector3/Vector4 primitives.
__global__ void __launch_bounds__(kPrepBlock)
    k_point_prep(const float* __restrict__ c, size_t stride, size_t n, DAabb* __restrict__ aabbs,
                 float4* __restrict__ centers) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float x = __ldg(c + stride * i), y = __ldg(c + stride * i + 1), z = __ldg(c + stride * i + 2);
  if (aabbs) {
    DAabb b;
    b.min[0] = rs_min(1e34f, x); b.min[1] = rs_min(1e34f, y); b.min[2] = rs_min(1e34f, z);
    b.max[0] = rs_max(-1e34f, x); b.max[1] = rs_max(-1e34f, y); b.max[2] = rs_max(-1e34f, z);
    b.count = 0;
    b.left_first = 0;
    store_aabb(aabbs + i, b);
  }
  centers[i] = make_float4(x, y, z, 0.0f);
}

// Aabb::union_of_list, stage 1: per-block min/max folded into six ordered
// keys with atomics (min/max are exact, so the order does not matter).
__global__ void __launch_bounds__(kPrepBlock)
    k_bounds_reduce(const DAabb* __restrict__ aabbs, size_t n, uint32_t* __restrict__ acc) {
  float mn[3] = {1e34f, 1e34f, 1e34f}, mx[3] = {-1e34f, -1e34f, -1e34f};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    DAabb b = load_aabb(aabbs + i);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mn[a] = rs_min(mn[a], b.min[a]);
      mx[a] = rs_max(mx[a], b.max[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = rs_min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = rs_max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(acc + a, float_to_ordered(mn[a]));
      atomicMax(acc + 3 + a, float_to_ordered(mx[a]));
    }
  }
}

// stage 2: the folded box plus the 1e-4 offset (Aabb::with_offset).
__global__ void k_bounds_finalize(const uint32_t* __restrict__ acc, DAabb* __restrict__ world) {
  if (threadIdx.x != 0) return;
  DAabb w;
  for (int a = 0; a < 3; ++a) {
    float mn = rs_min(1e34f, ordered_to_float(acc[a]));
    float mx = rs_max(-1e34f, ordered_to_float(acc[3 + a]));
    w.min[a] = mn - 0.0001f;
    w.max[a] = mx + 0.0001f;
  }
  w.count = 0;
  w.left_first = 0;
  store_aabb(world, w);
}

__global__ void k_bounds_init(uint32_t* acc) {
  if (threadIdx.x < 3) acc[threadIdx.x] = 0xffffffffu;
  else if (threadIdx.x < 6) acc[threadIdx.x] = 0u;
}

// morton_split (src/morton.rs:10-25) for values below 1024: the bits of v
// spread to every third position.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// min(1023, max(g as i32, 0)) with Rust's saturating, NaN->0 cast.
__device__ __forceinline__ uint32_t grid_cell(float g) {
  if (g >= 1023.0f) return 1023u;
  if (g >= 0.0f) return (uint32_t)(int)g;
  return 0u;
}

// MortonEncoder::new (src/morton.rs:36-46, grid 1024) + encode (:52-61).
__global__ void __launch_bounds__(kPrepBlock)
    k_morton(const float4* __restrict__ centers, size_t n, const DAabb* __restrict__ world,
             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  __shared__ float s_w2g[3], s_off[3];
  if (threadIdx.x < 3) {
    const int a = threadIdx.x;
    float mn = world->min[a], mx = world->max[a];
    float w2g = 1024.0f * (1.0f / (mx - mn));
    s_w2g[a] = w2g;
    s_off[a] = (-mn) * w2g;
  }
  __syncthreads();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 c = __ldg(centers + i);
  uint32_t x = grid_cell(c.x * s_w2g[0] + s_off[0]);
  uint32_t y = grid_cell(c.y * s_w2g[1] + s_off[1]);
  uint32_t z = grid_cell(c.z * s_w2g[2] + s_off[2]);
  keys[i] = spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
  vals[i] = (uint32_t)i;
}

__global__ void __launch_bounds__(kPrepBlock)
    k_gather_triangles(const float* __restrict__ v, const uint32_t* __restrict__ idx, size_t n,
                       float4* __restrict__ out) {
  size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t p = __ldg(idx + k);
  const float* t = v + 9 * (size_t)p;
  float x0 = __ldg(t), y0 = __ldg(t + 1), z0 = __ldg(t + 2);
  float x1 = __ldg(t + 3), y1 = __ldg(t + 4), z1 = __ldg(t + 5);
  float x2 = __ldg(t + 6), y2 = __ldg(t + 7), z2 = __ldg(t + 8);
  float4* o = out + (size_t)kTriFloat4 * k;
  o[0] = make_float4(x0, y0, z0, __uint_as_float(p));
  o[1] = make_float4(x1 - x0, y1 - y0, z1 - z0, 0.0f);
  o[2] = make_float4(x2 - x0, y2 - y0, z2 - z0, 0.0f);
  o[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

inline unsigned grid_for(size_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t launch_triangle_prep(const float* vertices, size_t n, DAabb* aabbs, float4* centers, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_triangle_prep<<<grid_for(n, kPrepBlock), kPrepBlock, 0, s>>>(vertices, n, aabbs, centers);
  return cudaGetLastError();
}

cudaError_t launch_point_prep(const float* centers, size_t stride_floats, size_t n, DAabb* aabbs, float4* centers4,
                              cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_point_prep<<<grid_for(n, kPrepBlock), kPrepBlock, 0, s>>>(centers, stride_floats, n, aabbs, centers4);
  return cudaGetLastError();
}

cudaError_t launch_pack_centers(const float* centers, size_t stride_floats, size_t n, float4* centers4,
                                cudaStream_t s) {
  return launch_point_prep(centers, stride_floats, n, nullptr, centers4, s);
}

cudaError_t launch_world_bounds(const DAabb* aabbs, size_t n, DAabb* world, uint32_t* acc6, cudaStream_t s) {
  k_bounds_init<<<1, 32, 0, s>>>(acc6);
  if (n > 0) {
    unsigned blocks = grid_for(n, kPrepBlock);
    unsigned cap = (unsigned)sm_count() * 8u;
    if (blocks > cap) blocks = cap;
    k_bounds_reduce<<<blocks, kPrepBlock, 0, s>>>(aabbs, n, acc6);
  }
  k_bounds_finalize<<<1, 32, 0, s>>>(acc6, world);
  return cudaGetLastError();
}

cudaError_t launch_morton(const float4* centers, size_t n, const DAabb* world, uint32_t* keys, uint32_t* vals,
                          cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_morton<<<grid_for(n, kPrepBlock), kPrepBlock, 0, s>>>(centers, n, world, keys, vals);
  return cudaGetLastError();
}

cudaError_t launch_gather_triangles(const float* vertices, const uint32_t* indices, size_t n, float4* out,
                                    cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_gather_triangles<<<grid_for(n, kPrepBlock), kPrepBlock, 0, s>>>(vertices, indices, n, out);
  return cudaGetLastError();
}

namespace {
std::mutex g_pool_mu;
std::vector<cudaMemPool_t> g_pools;
}  // namespace

// Per-device pool; up to an eighth of the device memory (at most 8 GiB) of
// freed allocations stays reserved between calls.
static cudaError_t library_pool(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev))) return e;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1, nullptr);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    if ((e = cudaMemPoolCreate(&pool, &props))) return e;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    uint64_t keep = (uint64_t)total_b / 8;
    if (keep > (8ull << 30)) keep = 8ull << 30;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}

cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (bytes == 0) return cudaSuccess;
  // under stream capture the allocation becomes a graph memory node of the
  // default pool
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e;
  if ((e = cudaStreamIsCapturing(s, &cap))) return e;
  if (cap != cudaStreamCaptureStatusNone) return cudaMallocAsync(p, bytes, s);
  cudaMemPool_t pool;
  if ((e = library_pool(&pool))) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

void pool_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

void pool_free_now(void* const* ptrs, int count) {
  bool any = false;
  for (int i = 0; i < count; ++i) any = any || ptrs[i] != nullptr;
  if (!any) return;
  cudaDeviceSynchronize();
  for (int i = 0; i < count; ++i)
    if (ptrs[i]) cudaFreeAsync(ptrs[i], 0);
}

int sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached = v > 0 ? v : 1;
  }
  return cached;
}

}  // namespace rtbvh
