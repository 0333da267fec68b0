// Batched build + trace of many independent meshes.
//
// The meshes are concatenated (triangles [off_m, off_m + n_m), rays
// [roff_m, roff_m + r_m)) and built as one forest with global indices:
//   1. triangle boxes/centres; per-mesh world boxes (Aabb::union_of_list);
//   2. Morton codes against each mesh's own world box, then a stable sort by
//      code followed by a stable sort by mesh id: (mesh, code) order, i.e.
//      every mesh's own MortonEncoder::get_sorted_indices order;
//   3. the clustering levels (locb.cu): a thread-block cluster per large
//      mesh, one block per small mesh, the two sets concurrently;
//   4. parent pointers and quad-subtree counts over the whole forest, then
//      one block per mesh for the top-down MBVH collapse (mbvh.cu);
//   5. leaf-ordered triangles, per-mesh closest-hit traversal trees (one
//      block per mesh, see build_wide) and ONE persistent traversal launch
//      for all rays, each ray starting at its mesh's root.
// Every buffer is allocated when the plan is created, and the whole
// pipeline is captured in a CUDA graph that rtbvh_gpu_batch_run replays.
// Per mesh, the result equals the single-mesh build's, with node, leaf and
// quad indices shifted by the mesh's offsets.
#include <algorithm>
#include <memory>
#include <mutex>
#include <numeric>
#include <vector>

#include "lib_internal.h"

namespace rtbvh {

namespace {

constexpr int kBlock = 256;

// Aabb::union_of_list per mesh, one block per mesh.
__global__ void __launch_bounds__(kBlock)
    k_seg_world(const DAabb* __restrict__ aabbs, const uint32_t* __restrict__ prim_off, uint32_t mesh_count,
                DAabb* __restrict__ worlds) {
  __shared__ uint32_t s_acc[6];
  for (uint32_t m = blockIdx.x; m < mesh_count; m += gridDim.x) {
    if (threadIdx.x < 3) s_acc[threadIdx.x] = float_to_ordered(1e34f);
    else if (threadIdx.x < 6) s_acc[threadIdx.x] = float_to_ordered(-1e34f);
    __syncthreads();
    const uint32_t b = prim_off[m], e = prim_off[m + 1];
    float mn[3] = {1e34f, 1e34f, 1e34f}, mx[3] = {-1e34f, -1e34f, -1e34f};
    for (uint32_t i = b + threadIdx.x; i < e; i += kBlock) {
      const DAabb a = load_aabb(aabbs + i);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        mn[k] = rs_min(mn[k], a.min[k]);
        mx[k] = rs_max(mx[k], a.max[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      atomicMin(s_acc + k, float_to_ordered(mn[k]));
      atomicMax(s_acc + 3 + k, float_to_ordered(mx[k]));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      DAabb w;
      for (int k = 0; k < 3; ++k) {
        w.min[k] = ordered_to_float(s_acc[k]) - 0.0001f;
        w.max[k] = ordered_to_float(s_acc[3 + k]) + 0.0001f;
      }
      w.count = 0;
      w.left_first = 0;
      store_aabb(worlds + m, w);
    }
    __syncthreads();
  }
}

__device__ __forceinline__ uint32_t segment_of(const uint32_t* __restrict__ off, uint32_t count, uint32_t i) {
  uint32_t lo = 0, hi = count;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t spread3b(uint32_t v) {
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ uint32_t cell1024(float g) {
  if (g >= 1023.0f) return 1023u;
  if (g >= 0.0f) return (uint32_t)(int)g;
  return 0u;
}

// MortonEncoder::encode of each centre against its mesh's world box.
__global__ void __launch_bounds__(kBlock)
    k_seg_morton(const float4* __restrict__ centers, const uint32_t* __restrict__ prim_off, uint32_t mesh_count,
                 uint32_t total, const DAabb* __restrict__ worlds, uint32_t* __restrict__ keys,
                 uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= total) return;
  const uint32_t m = segment_of(prim_off, mesh_count, i);
  const DAabb w = load_aabb(worlds + m);
  const float4 c = __ldg(centers + i);
  const float cc[3] = {c.x, c.y, c.z};
  uint32_t g[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float w2g = 1024.0f * (1.0f / (w.max[a] - w.min[a]));
    const float off = (-w.min[a]) * w2g;
    g[a] = cell1024(cc[a] * w2g + off);
  }
  keys[i] = spread3b(g[0]) | (spread3b(g[1]) << 1) | (spread3b(g[2]) << 2);
  vals[i] = i;
}

__global__ void __launch_bounds__(kBlock)
    k_seg_mesh_keys(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ prim_off, uint32_t mesh_count,
                    uint32_t total, uint32_t* __restrict__ keys) {
  const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= total) return;
  keys[k] = segment_of(prim_off, mesh_count, __ldg(vals + k));
}

template <class T>
struct DevBuf {
  T* ptr = nullptr;
  cudaError_t alloc(size_t n) { return n ? cudaMalloc(reinterpret_cast<void**>(&ptr), n * sizeof(T)) : cudaSuccess; }
  ~DevBuf() {
    if (ptr) cudaFree(ptr);
  }
};

struct Plan {
  uint32_t mesh_count = 0, total_prims = 0, node_cap = 0;
  size_t total_rays = 0;
  const float* vertices = nullptr;
  const float* rays = nullptr;
  const float* t_max = nullptr;
  float* hits = nullptr;
  uint32_t flags = 0;
  DevBuf<uint32_t> prim_off, ray_off, order, keys, vals, nb, parent, arrive, cnt_e, cnt_o, mbase, status, sort_tmp_u;
  DevBuf<DAabb> aabbs, worlds, lvl0, lvl1, nodes;
  DevBuf<float4> centers, tris;
  DevBuf<DMNode> mnodes;
  DevBuf<DMNode> wnodes;  // per-mesh closest-hit traversal trees (exact), mesh m at [off_m, off_m + n_m)
  DevBuf<DQNode> qnodes;  // the same, compact
  DevBuf<uint2> q0, q1;
  DevBuf<char> sort_temp;
  size_t sort_bytes = 0;
  // meshes order[0, big_count) get a thread-block cluster each (locb.cu)
  uint32_t big_count = 0;
  unsigned clusters = 0;
  DevBuf<uint32_t> cluster_sums;
  std::vector<uint32_t> sizes_in_order;  // host: primitive count of order[q]
  // launch parameters (RTBatchTuning; 0 = default)
  uint32_t trace_blocks_per_sm = 0, trace_ray_batch = 0, cluster_min = kSegClusterMinPrims, trace_stack = 0;
  cudaStream_t side = nullptr;  // small meshes' clustering runs here, forked from the main stream
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~Plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (side) cudaStreamDestroy(side);
  }
};

std::mutex g_plans_mu;
std::vector<std::unique_ptr<Plan>> g_plans;

constexpr uint32_t kMaxClusters = 8192;

// Meshes above `min_prims` primitives (a prefix of the size-ordered mesh
// list) are clustered by block clusters; meshes of at most 2 primitives
// always take the single-block path.
void set_cluster_min(Plan& p, uint32_t min_prims) {
  p.cluster_min = min_prims < 2u ? 2u : min_prims;
  p.big_count = 0;
  while (p.big_count < p.mesh_count && p.sizes_in_order[p.big_count] > p.cluster_min) ++p.big_count;
  p.clusters = std::min<uint32_t>(p.big_count, kMaxClusters);
}

unsigned mesh_blocks(uint32_t mesh_count) {
  const unsigned cap = (unsigned)sm_count() * 4u;
  return mesh_count < cap ? mesh_count : cap;
}

cudaError_t run_build(Plan& p, cudaStream_t s) {
  cudaError_t e;
  const uint32_t N = p.total_prims, M = p.mesh_count;
  const unsigned gN = (N + kBlock - 1) / kBlock;
  if ((e = launch_triangle_prep(p.vertices, N, p.aabbs.ptr, p.centers.ptr, s))) return e;
  k_seg_world<<<mesh_blocks(M), kBlock, 0, s>>>(p.aabbs.ptr, p.prim_off.ptr, M, p.worlds.ptr);
  k_seg_morton<<<gN, kBlock, 0, s>>>(p.centers.ptr, p.prim_off.ptr, M, N, p.worlds.ptr, p.keys.ptr, p.vals.ptr);
  if ((e = radix_sort_pairs(p.keys.ptr, p.vals.ptr, N, 30, p.sort_temp.ptr, p.sort_bytes, p.status.ptr, s)))
    return e;
  k_seg_mesh_keys<<<gN, kBlock, 0, s>>>(p.vals.ptr, p.prim_off.ptr, M, N, p.keys.ptr);
  int mbits = 1;
  while (mbits < 31 && (1u << mbits) < M) ++mbits;
  if ((e = radix_sort_pairs(p.keys.ptr, p.vals.ptr, N, mbits, p.sort_temp.ptr, p.sort_bytes, p.status.ptr, s)))
    return e;
  if ((e = cudaMemsetAsync(p.nodes.ptr, 0xff, (size_t)p.node_cap * sizeof(DAabb), s))) return e;
  if ((e = launch_locb_segments(p.aabbs.ptr, p.vals.ptr, p.vals.ptr, p.prim_off.ptr, p.order.ptr, p.worlds.ptr, M, N,
                                p.lvl0.ptr, p.lvl1.ptr, p.nodes.ptr, p.nb.ptr, p.status.ptr, mesh_blocks(M),
                                p.big_count, p.cluster_sums.ptr, p.clusters, s, p.side, p.fork, p.join)))
    return e;
  if ((e = launch_collapse_segments(p.nodes.ptr, p.node_cap, p.prim_off.ptr, p.order.ptr, M, p.parent.ptr,
                                    p.arrive.ptr, p.cnt_e.ptr, p.cnt_o.ptr, p.mbase.ptr, p.q0.ptr, p.q1.ptr,
                                    p.mnodes.ptr, p.node_cap, p.status.ptr, mesh_blocks(M), s)))
    return e;
  if ((e = launch_gather_triangles(p.vertices, p.vals.ptr, N, p.tris.ptr, s))) return e;
  // closest-hit traversal trees (LOCB trees are nested, see build_wide)
  if (!(p.flags & (RTBVH_TRACE_ANY_HIT | RTBVH_TRACE_EXACT_NODES)) &&
      (e = launch_wide_segments(p.nodes.ptr, p.node_cap, p.prim_off.ptr, p.order.ptr, M, N, p.wnodes.ptr,
                                p.qnodes.ptr, p.q0.ptr, p.q1.ptr, p.status.ptr, mesh_blocks(M), s)))
    return e;
  return cudaGetLastError();
}

cudaError_t run_trace(Plan& p, cudaStream_t s) {
  cudaError_t e;
  const uint32_t N = p.total_prims, M = p.mesh_count;
  if (p.total_rays) {
    TraceArgs a;
    a.mnodes = p.mnodes.ptr;
    a.node_count = p.node_cap;
    a.tris = p.tris.ptr;
    a.prim_count = N;
    a.rays = p.rays;
    a.t_max = p.t_max;
    a.ray_count = p.total_rays;
    a.hits = reinterpret_cast<float4*>(p.hits);
    a.status = p.status.ptr;
    a.any_hit = (p.flags & RTBVH_TRACE_ANY_HIT) != 0;
    a.seg_ray_off = p.ray_off.ptr;
    a.seg_root = p.mbase.ptr;
    a.seg_count = M;
    if (!(p.flags & (RTBVH_TRACE_ANY_HIT | RTBVH_TRACE_EXACT_NODES))) {
      a.qnodes = p.qnodes.ptr;
      a.qexact = p.wnodes.ptr;
      a.q_count = N;
      a.seg_qroot = p.prim_off.ptr;  // mesh m's traversal tree starts at off_m
    }
    a.blocks_per_sm = p.trace_blocks_per_sm;
    a.ray_batch = p.trace_ray_batch;
    a.stack_limit = p.trace_stack;
    if ((e = launch_trace_mbvh(a, s))) return e;
  }
  return cudaGetLastError();
}

cudaError_t run_pipeline(Plan& p, cudaStream_t s) {
  cudaError_t e = run_build(p, s);
  if (e != cudaSuccess) return e;
  return run_trace(p, s);
}

// (Re)captures the whole pipeline into p.graph / p.exec.
cudaError_t capture(Plan& p) {
  if (p.exec) {
    cudaGraphExecDestroy(p.exec);
    p.exec = nullptr;
  }
  if (p.graph) {
    cudaGraphDestroy(p.graph);
    p.graph = nullptr;
  }
  cudaStream_t cap;
  cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t run = run_pipeline(p, cap);
    e = cudaStreamEndCapture(cap, &p.graph);
    if (run != cudaSuccess) e = run;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p.exec, p.graph, 0);
  cudaStreamDestroy(cap);
  return e;
}

// Best of `reps` timed runs of fn after one untimed run, in milliseconds.
template <class F>
cudaError_t time_ms(F fn, cudaStream_t s, int reps, float* best) {
  cudaEvent_t a, b;
  cudaError_t e;
  if ((e = cudaEventCreate(&a))) return e;
  if ((e = cudaEventCreate(&b))) {
    cudaEventDestroy(a);
    return e;
  }
  *best = 3.4e38f;
  e = fn();
  for (int i = 0; i < reps && e == cudaSuccess; ++i) {
    if ((e = cudaEventRecord(a, s)) || (e = fn()) || (e = cudaEventRecord(b, s)) || (e = cudaEventSynchronize(b)))
      break;
    float ms = 0.0f;
    if ((e = cudaEventElapsedTime(&ms, a, b))) break;
    *best = std::min(*best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return e;
}

Plan* find_plan(uint32_t id) {
  std::lock_guard<std::mutex> lock(g_plans_mu);
  if (id >= g_plans.size()) return nullptr;
  return g_plans[id].get();
}

}  // namespace

}  // namespace rtbvh

using namespace rtbvh;

extern "C" {

ResultCode rtbvh_gpu_batch_create(const float* vertices, const uint32_t* prim_offsets, uint32_t mesh_count,
                                  const float* rays, const float* t_max, const uint32_t* ray_offsets, float* hits,
                                  uint32_t flags, rtbvh_stream_t stream, RTBatch* result) {
  if (result == nullptr || prim_offsets == nullptr || ray_offsets == nullptr || mesh_count == 0) return Error;
  if (prim_offsets[0] != 0 || ray_offsets[0] != 0) return InvalidArgument;
  for (uint32_t m = 0; m < mesh_count; ++m)
    if (prim_offsets[m + 1] <= prim_offsets[m] || ray_offsets[m + 1] < ray_offsets[m]) return InvalidArgument;
  const uint64_t N = prim_offsets[mesh_count];
  const uint64_t R = ray_offsets[mesh_count];
  if (N == 0) return NoPrimitives;
  if (N >= (1u << 29) || R >= (1ull << 31)) return InvalidArgument;
  if (vertices == nullptr || (R > 0 && (rays == nullptr || hits == nullptr))) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto p = std::make_unique<Plan>();
  p->mesh_count = mesh_count;
  p->total_prims = (uint32_t)N;
  p->total_rays = R;
  p->node_cap = (uint32_t)(2 * N - mesh_count);  // sum over meshes of 2 n_m - 1
  p->vertices = vertices;
  p->rays = rays;
  p->t_max = t_max;
  p->hits = hits;
  p->flags = flags;
  std::vector<uint32_t> order(mesh_count);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    return prim_offsets[a + 1] - prim_offsets[a] > prim_offsets[b + 1] - prim_offsets[b];
  });
  p->sort_bytes = radix_sort_temp_bytes(N);
  p->sizes_in_order.resize(mesh_count);
  for (uint32_t q = 0; q < mesh_count; ++q) p->sizes_in_order[q] = prim_offsets[order[q] + 1] - prim_offsets[order[q]];
  set_cluster_min(*p, kSegClusterMinPrims);
  cudaError_t e;
  if ((e = p->cluster_sums.alloc((size_t)kSegCluster * std::min<uint32_t>(mesh_count, kMaxClusters))) ||
      (e = cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking)) ||
      (e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) ||
      (e = cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming)))
    return cuda_rc(e);
  if ((e = p->prim_off.alloc(mesh_count + 1)) || (e = p->ray_off.alloc(mesh_count + 1)) ||
      (e = p->order.alloc(mesh_count)) || (e = p->keys.alloc(N)) || (e = p->vals.alloc(N)) ||
      (e = p->nb.alloc(p->node_cap)) || (e = p->parent.alloc(p->node_cap)) || (e = p->arrive.alloc(p->node_cap)) ||
      (e = p->cnt_e.alloc(p->node_cap)) || (e = p->cnt_o.alloc(p->node_cap)) || (e = p->mbase.alloc(mesh_count + 1)) ||
      (e = p->status.alloc(4)) || (e = p->aabbs.alloc(N)) || (e = p->worlds.alloc(mesh_count)) ||
      (e = p->lvl0.alloc(p->node_cap)) || (e = p->lvl1.alloc(p->node_cap)) || (e = p->nodes.alloc(p->node_cap)) ||
      (e = p->centers.alloc(N)) || (e = p->tris.alloc((size_t)kTriFloat4 * N)) ||
      (e = p->mnodes.alloc(p->node_cap)) || (e = p->qnodes.alloc(N)) || (e = p->wnodes.alloc(N)) || (e = p->q0.alloc(2 * (size_t)p->node_cap)) ||
      (e = p->q1.alloc(2 * (size_t)p->node_cap)) || (e = p->sort_temp.alloc(p->sort_bytes)))
    return cuda_rc(e);
  if ((e = cudaMemcpyAsync(p->prim_off.ptr, prim_offsets, 4 * (size_t)(mesh_count + 1), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(p->ray_off.ptr, ray_offsets, 4 * (size_t)(mesh_count + 1), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(p->order.ptr, order.data(), 4 * (size_t)mesh_count, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(p->status.ptr, 0, 16, s)) || (e = cudaStreamSynchronize(s)))
    return cuda_rc(e);
  // one direct run (also warms every lazily initialised path), then capture
  if ((e = run_pipeline(*p, s)) || (e = cudaStreamSynchronize(s))) return cuda_rc(e);
  if ((e = capture(*p))) return cuda_rc(e);
  std::lock_guard<std::mutex> lock(g_plans_mu);
  g_plans.push_back(std::move(p));
  result->id = (uint32_t)(g_plans.size() - 1);
  return Ok;
}

ResultCode rtbvh_gpu_batch_run(RTBatch batch, rtbvh_stream_t stream) {
  Plan* p = find_plan(batch.id);
  if (!p || !p->exec) return Error;
  return cuda_rc(cudaGraphLaunch(p->exec, static_cast<cudaStream_t>(stream)));
}

ResultCode rtbvh_gpu_batch_run_uncaptured(RTBatch batch, rtbvh_stream_t stream) {
  Plan* p = find_plan(batch.id);
  if (!p) return Error;
  return cuda_rc(run_pipeline(*p, static_cast<cudaStream_t>(stream)));
}

ResultCode rtbvh_gpu_batch_view(RTBatch batch, RTGpuBatchView* view) {
  Plan* p = find_plan(batch.id);
  if (!p || view == nullptr) return Error;
  view->nodes = reinterpret_cast<const RTBvhNode*>(p->nodes.ptr);
  view->node_capacity = p->node_cap;
  view->indices = p->vals.ptr;
  view->mnodes = reinterpret_cast<const RTMbvhNode*>(p->mnodes.ptr);
  view->mnode_base = p->mbase.ptr;
  view->prim_offsets = p->prim_off.ptr;
  view->mesh_count = p->mesh_count;
  view->leaf_triangles = reinterpret_cast<const float*>(p->tris.ptr);
  return Ok;
}

ResultCode rtbvh_gpu_batch_status(RTBatch batch) {
  Plan* p = find_plan(batch.id);
  if (!p) return Error;
  uint32_t st = 0;
  cudaError_t e;
  if ((e = cudaDeviceSynchronize()) || (e = cudaMemcpy(&st, p->status.ptr, 4, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemset(p->status.ptr, 0, 4)))
    return cuda_rc(e);
  if (st & kStatusStackOverflow) return StackOverflow;
  if (st & kStatusTimeout) return Timeout;
  return st ? Error : Ok;
}

ResultCode rtbvh_gpu_batch_get_tuning(RTBatch batch, RTBatchTuning* result) {
  Plan* p = find_plan(batch.id);
  if (!p || result == nullptr) return Error;
  result->trace_blocks_per_sm = p->trace_blocks_per_sm;
  result->trace_ray_batch = p->trace_ray_batch;
  result->cluster_min_prims = p->cluster_min;
  result->pipeline_ms = 0.0f;
  result->trace_stack = p->trace_stack ? p->trace_stack : 64u;
  return Ok;
}

ResultCode rtbvh_gpu_batch_set_tuning(RTBatch batch, const RTBatchTuning* t, rtbvh_stream_t stream) {
  Plan* p = find_plan(batch.id);
  if (!p || t == nullptr) return Error;
  if (t->trace_blocks_per_sm > 64 || t->trace_ray_batch > 4096u) return InvalidArgument;
  if (t->trace_stack != 0 && t->trace_stack != 32 && t->trace_stack != 48 && t->trace_stack != 64)
    return InvalidArgument;
  cudaError_t e;
  if ((e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream)))) return cuda_rc(e);
  p->trace_blocks_per_sm = t->trace_blocks_per_sm;
  p->trace_ray_batch = t->trace_ray_batch;
  p->trace_stack = t->trace_stack;
  set_cluster_min(*p, t->cluster_min_prims ? t->cluster_min_prims : kSegClusterMinPrims);
  return cuda_rc(capture(*p));
}

ResultCode rtbvh_gpu_batch_tune(RTBatch batch, rtbvh_stream_t stream, RTBatchTuning* result) {
  Plan* p = find_plan(batch.id);
  if (!p) return Error;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if ((e = cudaStreamSynchronize(s))) return cuda_rc(e);
  // 1. clustering threshold, timed on the build alone
  static const uint32_t kClusterMin[] = {2048u, 4096u, 8192u, 16384u, 65536u};
  uint32_t best_c = p->cluster_min;
  float best = 3.4e38f;
  for (uint32_t c : kClusterMin) {
    set_cluster_min(*p, c);
    float ms;
    if ((e = time_ms([&] { return run_build(*p, s); }, s, 2, &ms))) return cuda_rc(e);
    if (ms < best) {
      best = ms;
      best_c = c;
    }
  }
  set_cluster_min(*p, best_c);
  if ((e = run_build(*p, s))) return cuda_rc(e);
  // 2. traversal launch shape, timed on the trace alone
  static const uint32_t kBlocksPerSm[] = {2u, 4u, 0u};
  static const uint32_t kRayBatch[] = {32u, 64u, 128u, 256u};
  uint32_t best_b = 0, best_r = 0;
  best = 3.4e38f;
  if (p->total_rays) {
    for (uint32_t b : kBlocksPerSm) {
      for (uint32_t r : kRayBatch) {
        p->trace_blocks_per_sm = b;
        p->trace_ray_batch = r;
        float ms;
        if ((e = time_ms([&] { return run_trace(*p, s); }, s, 2, &ms))) return cuda_rc(e);
        if (ms < best) {
          best = ms;
          best_b = b;
          best_r = r;
        }
      }
    }
  }
  p->trace_blocks_per_sm = best_b;
  p->trace_ray_batch = best_r;
  // 3. stack bound of the closest-hit walk (local memory per lane): the
  // fastest of the bounds that no ray of this batch overflows. The status
  // word is saved and restored around the trial runs, whose overflow bits
  // only rate the candidates.
  uint32_t best_st = 64u;
  if (p->total_rays && !(p->flags & (RTBVH_TRACE_ANY_HIT | RTBVH_TRACE_EXACT_NODES))) {
    uint32_t prior = 0;
    if ((e = cudaMemcpy(&prior, p->status.ptr, 4, cudaMemcpyDeviceToHost))) return cuda_rc(e);
    static const uint32_t kStack[] = {32u, 48u, 64u};
    best = 3.4e38f;
    for (uint32_t st : kStack) {
      p->trace_stack = st;
      float ms;
      uint32_t word = 0;
      if ((e = cudaMemsetAsync(p->status.ptr, 0, 4, s)) ||
          (e = time_ms([&] { return run_trace(*p, s); }, s, 2, &ms)) ||
          (e = cudaMemcpy(&word, p->status.ptr, 4, cudaMemcpyDeviceToHost)))
        return cuda_rc(e);
      if (!(word & kStatusStackOverflow) && ms < best) {
        best = ms;
        best_st = st;
      }
    }
    if ((e = cudaMemcpy(p->status.ptr, &prior, 4, cudaMemcpyHostToDevice))) return cuda_rc(e);
  }
  p->trace_stack = best_st;
  if ((e = capture(*p))) return cuda_rc(e);
  float total = 0.0f;
  if ((e = time_ms([&] { return cudaGraphLaunch(p->exec, s); }, s, 3, &total))) return cuda_rc(e);
  if (result) {
    result->trace_blocks_per_sm = best_b;
    result->trace_ray_batch = best_r;
    result->cluster_min_prims = best_c;
    result->pipeline_ms = total;
    result->trace_stack = best_st;
  }
  return Ok;
}

void rtbvh_gpu_batch_free(RTBatch batch) {
  std::lock_guard<std::mutex> lock(g_plans_mu);
  if (batch.id < g_plans.size()) g_plans[batch.id].reset();
}

}  // extern "C"
