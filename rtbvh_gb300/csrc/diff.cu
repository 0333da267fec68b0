// Backward pass of the closest-hit triangle test (differentiable ray cast).
//
// The forward test (SpatialTriangle::intersect, src/builders/spatial_sah.rs:
// 132-163) returns (t, u, v) of the hit triangle, which solve
//     [-d | e1 | e2] (t, u, v)^T = o - v0,   e1 = v1 - v0, e2 = v2 - v0.
// With M = [-d | e1 | e2] and upstream g = (dL/dt, dL/du, dL/dv), the adjoint
// lambda = M^-T g = f * (g_t (e1 x e2) + g_u (d x e2) + g_v (e1 x d)), f = 1/det,
// gives
//     dL/do  = lambda,                dL/dd  = t * lambda,
//     dL/dv0 = -(1 - u - v) lambda,   dL/dv1 = -u lambda,   dL/dv2 = -v lambda.
// The BVH walk is an index selection: the hit ids stored by the forward pass
// are used, nothing is re-traversed.
//
// Per-triangle sums are deterministic: (prim, ray) pairs are sorted by prim
// with the stable radix sort (rays stay in index order within a prim) and
// one thread per triangle adds its rays' contributions in that order. Rays
// that missed (prim < 0) contribute nothing and get zero ray gradients.
//
// This file may contract to FMA: the gradients carry a tolerance, not a
// bit-exactness requirement.
#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 256;

struct Adjoint {
  float lx, ly, lz;  // lambda
  float t, u, v;
};

__device__ __forceinline__ Adjoint adjoint(const float* __restrict__ tri, const float* __restrict__ ray,
                                           const float4 hit, const float* __restrict__ g) {
  const float v0x = tri[0], v0y = tri[1], v0z = tri[2];
  const float e1x = tri[3] - v0x, e1y = tri[4] - v0y, e1z = tri[5] - v0z;
  const float e2x = tri[6] - v0x, e2y = tri[7] - v0y, e2z = tri[8] - v0z;
  const float dx = ray[3], dy = ray[4], dz = ray[5];
  // h = d x e2, det = e1 . h
  const float hx = dy * e2z - dz * e2y, hy = dz * e2x - dx * e2z, hz = dx * e2y - dy * e2x;
  const float det = e1x * hx + e1y * hy + e1z * hz;
  const float f = 1.0f / det;
  // n = e1 x e2, w = e1 x d
  const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const float wx = e1y * dz - e1z * dy, wy = e1z * dx - e1x * dz, wz = e1x * dy - e1y * dx;
  const float gt = g[0], gu = g[1], gv = g[2];
  Adjoint a;
  a.lx = f * (gt * nx + gu * hx + gv * wx);
  a.ly = f * (gt * ny + gu * hy + gv * wy);
  a.lz = f * (gt * nz + gu * hz + gv * wz);
  a.t = hit.x;
  a.u = hit.y;
  a.v = hit.z;
  return a;
}

// Ray gradients and the (prim, ray) sort keys.
__global__ void __launch_bounds__(kBlock)
    k_bwd_rays(const float* __restrict__ vertices, uint32_t prim_count, const float* __restrict__ rays,
               const float4* __restrict__ hits, const float* __restrict__ grad_tuv, size_t ray_count,
               float* __restrict__ grad_rays, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const size_t r = (size_t)blockIdx.x * kBlock + threadIdx.x;
  if (r >= ray_count) return;
  const float4 h = hits[r];
  const int32_t prim = __float_as_int(h.w);
  const bool valid = prim >= 0 && (uint32_t)prim < prim_count;
  keys[r] = valid ? (uint32_t)prim : prim_count;
  vals[r] = (uint32_t)r;
  if (grad_rays == nullptr) return;
  float* gr = grad_rays + 6 * r;
  if (!valid) {
#pragma unroll
    for (int k = 0; k < 6; ++k) gr[k] = 0.0f;
    return;
  }
  const Adjoint a = adjoint(vertices + 9 * (size_t)prim, rays + 6 * r, h, grad_tuv + 3 * r);
  gr[0] = a.lx;
  gr[1] = a.ly;
  gr[2] = a.lz;
  gr[3] = a.t * a.lx;
  gr[4] = a.t * a.ly;
  gr[5] = a.t * a.lz;
}

// Each triangle's range [begin, end) in the sorted (prim, ray) pairs: the
// first and last position of every run of equal keys (triangles hit by no
// ray keep begin = end = 0 from the memset).
__global__ void __launch_bounds__(kBlock) k_bwd_ranges(const uint32_t* __restrict__ keys, uint32_t ray_count,
                                                       uint32_t prim_count, uint2* __restrict__ range) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= ray_count) return;
  const uint32_t key = __ldg(keys + k);
  if (key >= prim_count) return;  // rays without a hit sort last
  if (k == 0 || __ldg(keys + k - 1) != key) range[key].x = k;
  if (k + 1 == ray_count || __ldg(keys + k + 1) != key) range[key].y = k + 1;
}

// One warp per triangle: lane l takes the triangle's rays l, l + 32, ...
// (in ray-index order within the lane), then the nine sums are reduced
// across the lanes by a fixed butterfly, so the result is the same on
// every run.
__global__ void __launch_bounds__(kBlock)
    k_bwd_vertices(const float* __restrict__ vertices, uint32_t prim_count, const float* __restrict__ rays,
                   const float4* __restrict__ hits, const float* __restrict__ grad_tuv, uint32_t ray_count,
                   const uint2* __restrict__ range, const uint32_t* __restrict__ vals,
                   float* __restrict__ grad_vertices) {
  const uint32_t p = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= prim_count) return;  // warp-uniform
  const uint2 rg = range[p];
  const uint32_t lo = rg.x, hi = rg.y <= ray_count ? rg.y : ray_count;
  float g[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const float* tri = vertices + 9 * (size_t)p;
  for (uint32_t k = lo + (uint32_t)lane; k < hi; k += 32) {
    const uint32_t r = __ldg(vals + k);
    const Adjoint a = adjoint(tri, rays + 6 * (size_t)r, hits[r], grad_tuv + 3 * (size_t)r);
    const float w0 = -(1.0f - a.u - a.v), w1 = -a.u, w2 = -a.v;
    g[0] += w0 * a.lx; g[1] += w0 * a.ly; g[2] += w0 * a.lz;
    g[3] += w1 * a.lx; g[4] += w1 * a.ly; g[5] += w1 * a.lz;
    g[6] += w2 * a.lx; g[7] += w2 * a.ly; g[8] += w2 * a.lz;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int q = 0; q < 9; ++q) g[q] += __shfl_xor_sync(0xffffffffu, g[q], off);
  }
  if (lane < 9) {
    float v = g[0];
#pragma unroll
    for (int q = 1; q < 9; ++q)
      if (lane == q) v = g[q];
    grad_vertices[9 * (size_t)p + lane] = v;
  }
}

}  // namespace

cudaError_t launch_intersect_backward(const float* vertices, size_t prim_count, const float* rays,
                                      const float4* hits, const float* grad_tuv, size_t ray_count,
                                      float* grad_vertices, float* grad_rays, cudaStream_t s) {
  if (prim_count >= (1u << 30) || ray_count >= (1u << 30)) return cudaErrorInvalidValue;
  cudaError_t e;
  if (ray_count == 0) {
    if (prim_count) return cudaMemsetAsync(grad_vertices, 0, prim_count * 36, s);
    return cudaSuccess;
  }
  const uint32_t n = (uint32_t)prim_count, R = (uint32_t)ray_count;
  Scratch<uint32_t> keys, vals, status;
  Scratch<uint2> range;
  Scratch<char> temp;
  const size_t tb = radix_sort_temp_bytes(R);
  if ((e = keys.alloc(R, s)) || (e = vals.alloc(R, s)) || (e = status.alloc(1, s)) || (e = temp.alloc(tb, s)) ||
      (e = range.alloc(n + 1, s)))
    return e;
  if ((e = cudaMemsetAsync(status.ptr, 0, 4, s)) || (e = cudaMemsetAsync(range.ptr, 0, (size_t)(n + 1) * 8, s)))
    return e;
  k_bwd_rays<<<(R + kBlock - 1) / kBlock, kBlock, 0, s>>>(vertices, n, rays, hits, grad_tuv, R, grad_rays, keys.ptr,
                                                         vals.ptr);
  int bits = 1;
  while (bits < 31 && (1u << bits) <= n) ++bits;  // keys are in [0, n]
  if ((e = radix_sort_pairs(keys.ptr, vals.ptr, R, bits, temp.ptr, tb, status.ptr, s))) return e;
  if (n) {
    k_bwd_ranges<<<(R + kBlock - 1) / kBlock, kBlock, 0, s>>>(keys.ptr, R, n, range.ptr);
    const size_t threads = (size_t)n * 32;
    k_bwd_vertices<<<(unsigned)((threads + kBlock - 1) / kBlock), kBlock, 0, s>>>(vertices, n, rays, hits, grad_tuv,
                                                                                 R, range.ptr, vals.ptr,
                                                                                 grad_vertices);
  }
  return cudaGetLastError();
}

}  // namespace rtbvh
