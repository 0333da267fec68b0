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

__device__ __forceinline__ uint32_t lower_bound(const uint32_t* __restrict__ keys, uint32_t n, uint32_t key) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(keys + mid) < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// One thread per triangle sums its rays in ray-index order.
__global__ void __launch_bounds__(kBlock)
    k_bwd_vertices(const float* __restrict__ vertices, uint32_t prim_count, const float* __restrict__ rays,
                   const float4* __restrict__ hits, const float* __restrict__ grad_tuv, uint32_t ray_count,
                   const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                   float* __restrict__ grad_vertices) {
  const uint32_t p = blockIdx.x * kBlock + threadIdx.x;
  if (p >= prim_count) return;
  const uint32_t lo = lower_bound(keys, ray_count, p);
  const uint32_t hi = lower_bound(keys, ray_count, p + 1);
  float g0x = 0, g0y = 0, g0z = 0, g1x = 0, g1y = 0, g1z = 0, g2x = 0, g2y = 0, g2z = 0;
  const float* tri = vertices + 9 * (size_t)p;
  for (uint32_t k = lo; k < hi; ++k) {
    const uint32_t r = __ldg(vals + k);
    const Adjoint a = adjoint(tri, rays + 6 * (size_t)r, hits[r], grad_tuv + 3 * (size_t)r);
    const float w0 = -(1.0f - a.u - a.v), w1 = -a.u, w2 = -a.v;
    g0x += w0 * a.lx; g0y += w0 * a.ly; g0z += w0 * a.lz;
    g1x += w1 * a.lx; g1y += w1 * a.ly; g1z += w1 * a.lz;
    g2x += w2 * a.lx; g2y += w2 * a.ly; g2z += w2 * a.lz;
  }
  float* gv = grad_vertices + 9 * (size_t)p;
  gv[0] = g0x; gv[1] = g0y; gv[2] = g0z;
  gv[3] = g1x; gv[4] = g1y; gv[5] = g1z;
  gv[6] = g2x; gv[7] = g2y; gv[8] = g2z;
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
  Scratch<char> temp;
  const size_t tb = radix_sort_temp_bytes(R);
  if ((e = keys.alloc(R, s)) || (e = vals.alloc(R, s)) || (e = status.alloc(1, s)) || (e = temp.alloc(tb, s)))
    return e;
  if ((e = cudaMemsetAsync(status.ptr, 0, 4, s))) return e;
  k_bwd_rays<<<(R + kBlock - 1) / kBlock, kBlock, 0, s>>>(vertices, n, rays, hits, grad_tuv, R, grad_rays, keys.ptr,
                                                         vals.ptr);
  int bits = 1;
  while (bits < 31 && (1u << bits) <= n) ++bits;  // keys are in [0, n]
  if ((e = radix_sort_pairs(keys.ptr, vals.ptr, R, bits, temp.ptr, tb, status.ptr, s))) return e;
  if (n) {
    k_bwd_vertices<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(vertices, n, rays, hits, grad_tuv, R, keys.ptr,
                                                               vals.ptr, grad_vertices);
  }
  return cudaGetLastError();
}

}  // namespace rtbvh
