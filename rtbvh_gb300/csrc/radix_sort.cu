// Stable LSD radix sort of (uint32 key, uint32 value) pairs, one pass per
// 8-bit digit, in the onesweep style: one upfront histogram kernel for all
// digit passes, then one kernel per pass that ranks a tile in shared memory,
// resolves the tile's global digit offsets with a decoupled look-back over
// its predecessors, and scatters. Tiles take their index from an atomic
// counter in launch order, so every look-back waits only on tiles that are
// already running; each wait is still bounded and reports kStatusTimeout
// instead of hanging.
//
// Used for the Morton-code sort of the clustering builder
// (src/morton.rs:63-102 sorts the indices by code with a stable sort).
#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 256;  // threads per tile == number of digits
constexpr int kItems = 15;   // keys per thread
constexpr int kTile = kBlock * kItems;
constexpr int kWarps = kBlock / 32;
constexpr int kRadix = 256;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;

struct SortTemp {
  uint32_t* hist;          // passes x 256 (counts, then exclusive offsets)
  uint32_t* tile_counter;  // passes
  uint32_t* lookback;      // passes x tiles x 256
  uint32_t* keys_alt;
  uint32_t* vals_alt;
};

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

inline int passes_for(int bits) { return (bits + 7) / 8; }

SortTemp carve(void* temp, size_t n, int passes) {
  size_t tiles = (n + kTile - 1) / kTile;
  char* p = static_cast<char*>(temp);
  SortTemp t;
  t.hist = reinterpret_cast<uint32_t*>(p);
  p += align256(4 * kRadix * 4);
  t.tile_counter = reinterpret_cast<uint32_t*>(p);
  p += align256(4 * 4);
  t.lookback = reinterpret_cast<uint32_t*>(p);
  p += align256((size_t)4 * tiles * kRadix * 4);
  t.keys_alt = reinterpret_cast<uint32_t*>(p);
  p += align256(n * 4);
  t.vals_alt = reinterpret_cast<uint32_t*>(p);
  (void)passes;
  return t;
}

__global__ void __launch_bounds__(kBlock)
    k_histogram(const uint32_t* __restrict__ keys, size_t n, int passes, uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_hist[4][kRadix];
  for (int i = threadIdx.x; i < 4 * kRadix; i += kBlock) (&s_hist[0][0])[i] = 0;
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * kBlock + threadIdx.x; i < n; i += (size_t)gridDim.x * kBlock) {
    uint32_t k = __ldg(keys + i);
    for (int p = 0; p < passes; ++p) atomicAdd(&s_hist[p][(k >> (8 * p)) & 0xffu], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; ++p) {
    uint32_t c = s_hist[p][threadIdx.x];
    if (c) atomicAdd(hist + p * kRadix + threadIdx.x, c);
  }
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void __launch_bounds__(kBlock) k_hist_scan(uint32_t* __restrict__ hist) {
  __shared__ uint32_t s_warp[kWarps];
  uint32_t* h = hist + blockIdx.x * kRadix;
  uint32_t v = h[threadIdx.x];
  uint32_t incl = block_inclusive_scan<kBlock>(v, s_warp, nullptr);
  h[threadIdx.x] = incl - v;
}

__global__ void __launch_bounds__(kBlock)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, size_t n, int shift,
               const uint32_t* __restrict__ digit_offsets, uint32_t* __restrict__ lookback,
               uint32_t* __restrict__ tile_counter, uint32_t* __restrict__ status) {
  __shared__ uint32_t s_tile;
  __shared__ int s_fail;
  __shared__ uint32_t s_whist[kWarps][kRadix];
  __shared__ uint32_t s_local_off[kRadix];
  __shared__ uint32_t s_global_base[kRadix];
  __shared__ uint32_t s_warp[kWarps];
  __shared__ uint32_t s_keys[kTile];
  __shared__ uint32_t s_vals[kTile];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_tile = atomicAdd(tile_counter, 1u);
    s_fail = 0;
  }
  for (int i = tid; i < kWarps * kRadix; i += kBlock) (&s_whist[0][0])[i] = 0;
  __syncthreads();
  const size_t tile = s_tile;
  const size_t tile_base = tile * kTile;
  const size_t warp_base = tile_base + (size_t)warp * (kItems * 32);

  uint32_t key[kItems], val[kItems], rank[kItems];
  uint32_t dig[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    size_t idx = warp_base + (size_t)k * 32 + lane;
    bool valid = idx < n;
    key[k] = valid ? __ldg(keys_in + idx) : 0xffffffffu;
    val[k] = valid ? __ldg(vals_in + idx) : 0u;
    dig[k] = valid ? ((key[k] >> shift) & 0xffu) : (uint32_t)kRadix;
  }
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    uint32_t d = dig[k];
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t base = 0;
    if (d < (uint32_t)kRadix) base = s_whist[warp][d];
    rank[k] = base + __popc(peers & lt_mask);
    __syncwarp();
    if (d < (uint32_t)kRadix && (__ffs(peers) - 1) == lane) s_whist[warp][d] = base + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Thread `tid` owns digit `tid`: warp-exclusive offsets and the tile count.
  const uint32_t d = tid;
  uint32_t run = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) {
    uint32_t c = s_whist[w][d];
    s_whist[w][d] = run;
    run += c;
  }
  volatile uint32_t* lb = lookback;
  lb[tile * kRadix + d] = (tile == 0 ? kFlagInc : kFlagAgg) | run;
  uint32_t incl = block_inclusive_scan<kBlock>(run, s_warp, nullptr);
  s_local_off[d] = incl - run;

  uint32_t excl = 0;
  if (tile > 0) {
    size_t j = tile - 1;
    uint32_t spins = 0;
    for (;;) {
      uint32_t v = lb[j * kRadix + d];
      uint32_t flag = v & ~kCountMask;
      if (flag == 0u) {
        if (++spins > kSpinLimit) {
          atomicOr(status, kStatusTimeout);
          s_fail = 1;
          break;
        }
        __nanosleep(64);
        continue;
      }
      excl += v & kCountMask;
      if (flag == kFlagInc || j == 0) break;
      --j;
    }
    lb[tile * kRadix + d] = kFlagInc | (excl + run);
  }
  s_global_base[d] = __ldg(digit_offsets + d) + excl;
  __syncthreads();
  if (s_fail) return;

#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    if (dig[k] < (uint32_t)kRadix) {
      uint32_t pos = s_local_off[dig[k]] + s_whist[warp][dig[k]] + rank[k];
      s_keys[pos] = key[k];
      s_vals[pos] = val[k];
    }
  }
  __syncthreads();
  const size_t remaining = n - tile_base;
  const uint32_t tile_count = remaining < (size_t)kTile ? (uint32_t)remaining : (uint32_t)kTile;
  for (uint32_t i = tid; i < tile_count; i += kBlock) {
    uint32_t k = s_keys[i];
    uint32_t dd = (k >> shift) & 0xffu;
    size_t g = (size_t)s_global_base[dd] + (i - s_local_off[dd]);
    if (g < n) {
      keys_out[g] = k;
      vals_out[g] = s_vals[i];
    } else {
      atomicOr(status, kStatusBadIndex);
    }
  }
}

}  // namespace

size_t radix_sort_temp_bytes(size_t n) {
  size_t tiles = (n + kTile - 1) / kTile;
  return align256(4 * kRadix * 4) + align256(16) + align256((size_t)4 * tiles * kRadix * 4) + 2 * align256(n * 4) +
         256;
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, size_t n, int bits, void* temp, size_t temp_bytes,
                             uint32_t* status, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  if (n > kCountMask || temp_bytes < radix_sort_temp_bytes(n)) return cudaErrorInvalidValue;
  const int passes = passes_for(bits);
  const size_t tiles = (n + kTile - 1) / kTile;
  SortTemp t = carve(temp, n, passes);
  cudaError_t e;
  if ((e = cudaMemsetAsync(t.hist, 0, 4 * kRadix * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(t.tile_counter, 0, 16, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(t.lookback, 0, (size_t)passes * tiles * kRadix * 4, s)) != cudaSuccess) return e;
  unsigned hblocks = (unsigned)((n + kBlock - 1) / kBlock);
  unsigned cap = (unsigned)sm_count() * 4u;
  if (hblocks > cap) hblocks = cap;
  k_histogram<<<hblocks, kBlock, 0, s>>>(keys, n, passes, t.hist);
  k_hist_scan<<<passes, kBlock, 0, s>>>(t.hist);
  uint32_t *kin = keys, *vin = vals, *kout = t.keys_alt, *vout = t.vals_alt;
  for (int p = 0; p < passes; ++p) {
    k_onesweep<<<(unsigned)tiles, kBlock, 0, s>>>(kin, vin, kout, vout, n, 8 * p, t.hist + p * kRadix,
                                                  t.lookback + (size_t)p * tiles * kRadix, t.tile_counter + p,
                                                  status);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != keys) {
    if ((e = cudaMemcpyAsync(keys, kin, n * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(vals, vin, n * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace rtbvh
