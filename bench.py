"""Benchmark: closest-hit traversal throughput (Mrays/s) and build time on the
incoherent 1M-triangle scene.

Workload (one "step"): closest-hit traversal of 16,777,216 incoherent rays
through the 4-wide MBVH of 1,000,000 triangles (centroids uniform in the unit
cube, vertices at centroid + unit direction x log-normal(median 0.005,
sigma 0.5)), built with locally-ordered clustering and collapsed to an MBVH.
Rays start uniformly on a radius-2 sphere around the cube centre and point at
uniform points in the cube. All data is seeded synthetic input.

Default arm: the CUDA library. ``value`` is device-resident throughput
(CUDA events around each traversal launch, L2 flushed between steps);
``e2e`` is the same metric through the C ABI's host-buffer entry point
(rtbvh_intersect_mbvh_batch) with the ray upload and hit download inside the
timed region. ``--impl reference`` times the CPU restatement of the
reference's rayon traversal on all host cores over bounded ray samples.

Multi-GPU (torchrun, one rank per GPU): replicas only -- every rank traces its
own copy of the workload; ``value`` is the sum over ranks of rays divided by
the slowest rank's time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 1_000_000
N_RAYS = 16_777_216
SCENE_SEED, RAY_SEED = 2, 3
CLUSTER_TRIS, CLUSTER_CAMERA = 10_000_000, 4096  # clustered spheres: triangles, camera width
METRIC = "closest-hit Mrays/s (1M-tri incoherent LOCB+MBVH, 16.7M rays)"
B_IN, B_OUT, B_NODE, B_TRI = 24, 16, 128, 40  # algorithmic bytes: ray in, hit out, quad node, triangle (36 + index 4)
# algorithmic build bytes per primitive: triangle in 36, box 32, Morton code 4,
# index 4, two 32-byte nodes out
B_BUILD = 36 + 32 + 4 + 4 + 2 * 32


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_scene():
    from rtbvh_gb300 import scenes
    tris = scenes.incoherent(N_TRIS, seed=SCENE_SEED)
    rays, tmax = scenes.incoherent_rays(N_RAYS, seed=RAY_SEED)
    return tris, rays, tmax


def apply_size_overrides(args):
    """--rays/--tris shrink the workload for profiling captures only; the
    benchmark line is always taken at the full size. With --only
    clustered_10M_binned_sah they set the clustered scene's triangle count
    and its camera (the square image with about --rays pixels)."""
    global N_RAYS, N_TRIS, METRIC, CLUSTER_TRIS, CLUSTER_CAMERA
    if args.rays:
        N_RAYS = args.rays
        CLUSTER_CAMERA = max(16, math.isqrt(args.rays))
    if args.tris:
        N_TRIS = args.tris
        CLUSTER_TRIS = args.tris
    if args.rays or args.tris:
        METRIC = METRIC + f" [reduced: {N_TRIS} tris, {N_RAYS} rays]"


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def t_error_vs_fp64(tris, rays, hits, sample=1 << 20):
    """Relative error of the kernel's hit t against Möller-Trumbore in
    float64 on the same hit triangle, over the first `sample` hitting rays."""
    h = np.asarray(hits[:sample])
    prim = np.ascontiguousarray(h[:, 3]).view(np.int32)
    ok = prim >= 0
    if not ok.any():
        return None
    t = tris[prim[ok]].astype(np.float64)
    r = rays[:sample][ok].astype(np.float64)
    o, d = r[:, :3], r[:, 3:]
    e1, e2 = t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]
    q = np.cross(o - t[:, 0], e1)
    det = np.einsum("ij,ij->i", e1, np.cross(d, e2))
    t64 = np.einsum("ij,ij->i", e2, q) / det
    rel = np.abs(h[ok, 0].astype(np.float64) - t64) / np.abs(t64)
    return {"rays": int(ok.sum()), "max_rel": float(f"{rel.max():.3g}"), "p99_rel": float(f"{np.quantile(rel, 0.99):.3g}"),
            "median_rel": float(f"{np.median(rel):.3g}")}


def _mt_t32(tri, rays):
    """t of the reference's triangle test (SpatialTriangle::intersect,
    src/builders/spatial_sah.rs:132-163) in float32 without contraction, per
    row; NaN where the test rejects before t."""
    f32 = np.float32
    v0, v1, v2 = tri[:, 0].astype(f32), tri[:, 1].astype(f32), tri[:, 2].astype(f32)
    o, d = rays[:, :3].astype(f32), rays[:, 3:].astype(f32)
    e1, e2 = v1 - v0, v2 - v0

    def cross(a, b):
        return np.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                         a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], axis=1)

    def dot(a, b):
        return (a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1]) + a[:, 2] * b[:, 2]

    h = cross(d, e2)
    det = dot(e1, h)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = f32(1.0) / det
        q = cross(o - v0, e1)
        t = f * dot(e2, q)
    return np.where((det > -1e-5) & (det < 1e-5), np.float32(np.nan), t)


def nearest_hit_parity(gpu, ref, tris, rays):
    """GPU hits against the oracle's on the same rays: rays whose t differs
    in any bit; rays whose triangle differs, and how many of those are ties
    (the reported triangle is hit at exactly the same t by the reference's
    triangle test, so both answers are a nearest hit); u/v differences on
    rays with the same triangle."""
    g32, r32 = np.ascontiguousarray(gpu).view(np.uint32), np.ascontiguousarray(ref).view(np.uint32)
    t_bad = g32[:, 0] != r32[:, 0]
    pg, pr = g32[:, 3].view(np.int32), r32[:, 3].view(np.int32)
    diff = np.nonzero((pg != pr) & ~t_bad)[0]
    ties = 0
    if len(diff):
        ok = (pg[diff] >= 0) & (pr[diff] >= 0)
        t = _mt_t32(tris[np.maximum(pg[diff], 0)], rays[diff])
        ties = int((ok & (t.view(np.uint32) == g32[diff, 0])).sum())
    same = (pg == pr) & ~t_bad
    uv_bad = int(((g32[same, 1] != r32[same, 1]) | (g32[same, 2] != r32[same, 2])).sum())
    return {"rays": int(len(gpu)), "t_bit_mismatch": int(t_bad.sum()), "prim_mismatch": int(len(diff)),
            "ties_proven": ties, "uv_mismatch_same_prim": uv_bad}


B_QNODE, B_QTRI, B_XNODE = 64, 64, 128  # bytes the default walk reads: compact node, triangle record, exact node


def own_walk_roofline(mbvh, d_rays, ref_stats, ms, peak, peak_kind):
    """Roofline of the default walk over the bytes it reads itself: per ray
    24 in + 16 out, 64 per traversal-tree node visit and 64 per triangle
    record, counted by the walk's own statistics (RTBVH_TRACE_WALK_STATS);
    rays it hands on to the exact walk add that walk's 128-byte node visits
    and 64-byte triangle records (its counts are the reference iterator's)."""
    import torch
    _, w = mbvh.intersect(d_rays, walk_stats=True)
    w = w.to(torch.int64)
    n = w.shape[0]
    handed = w[:, 2] != 0
    wv, wt = float(w[:, 0].sum()), float(w[:, 1].sum())
    xb = 0.0
    if bool(handed.any()):
        xb = float(B_XNODE * ref_stats[handed, 0].sum() + B_QTRI * ref_stats[handed, 1].sum())
    own = n * (B_IN + B_OUT) + B_QNODE * wv + B_QTRI * wt + xb
    ach = own / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "unit": "GB/s", "achieved": round(ach, 1), "peak": peak, "frac": round(ach / peak, 3),
            "peak_source": peak_kind, "bytes_per_ray": round(own / n, 1), "mean_node_visits": round(wv / n, 3),
            "mean_tri_tests": round(wt / n, 3), "rays_handed_to_exact_walk": int(handed.sum()),
            "bytes": "24 ray + 16 hit + 64 per compact node + 64 per triangle record (+ 128 per exact node of "
                     "handed-on rays)"}


def replica_value(total_ms, rays_per_step, steps, world_size, dist=None, device="cpu"):
    """Replicas (no exchange between ranks): every rank traces its own copy
    of the workload. Returns (whole-job Mrays/s = all ranks' rays / the
    slowest rank's timed total, that total in ms)."""
    if dist is not None:
        import torch
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t)
    return world_size * rays_per_step * steps / (total_ms * 1e-3) / 1e6, total_ms


def run_gpu(args):
    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import build as libbuild

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    libbuild.build()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tris, rays, tmax = make_scene()
    d_tris = torch.from_numpy(tris).cuda()
    d_rays = torch.from_numpy(rays).cuda()
    d_tmax = torch.from_numpy(tmax).cuda()

    # ------------------------------------------------------------ build
    build_ms, mbvh_ms = [], []
    for i in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bvh = rb.Builder(primitives=rb.Triangles(d_tris)).construct_locally_ordered_clustered(host_mirror=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        mbvh = rb.Mbvh.construct(bvh, host_mirror=False)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if i > 0:
            build_ms.append((t1 - t0) * 1e3)
            mbvh_ms.append((t2 - t1) * 1e3)

    # ------------------------------------------------------------ roofline inputs
    _, st = mbvh.intersect(d_rays, stats=True)
    st = st.to(torch.int64)
    visits = float(st[:, 0].sum())
    tests = float(st[:, 1].sum())
    max_stack = int(st[:, 2].max())
    alg_bytes = N_RAYS * (B_IN + B_OUT) + B_NODE * visits + B_TRI * tests
    status = mbvh.status()
    if status != rb.ResultCode.Ok:
        raise RuntimeError(f"traversal reported {status!r}")

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        hits, _ = mbvh.intersect(d_rays, exact_nodes=args.exact_nodes)
        return hits

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(float(len(times)))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
    ms = statistics.mean(times)
    value, total_ms = replica_value(sum(times), N_RAYS, args.steps, ws, dist, "cuda")
    if dist:
        dist.barrier()

    # any-hit on the same structure (tmax = 0.5 x distance)
    for _ in range(2):
        mbvh.intersect(d_rays, t_max=d_tmax, any_hit=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    any_hits, _ = mbvh.intersect(d_rays, t_max=d_tmax, any_hit=True)
    e1.record(stream)
    e1.synchronize()
    any_ms = e0.elapsed_time(e1)
    any_hit_frac = float((any_hits[:, 3].contiguous().view(torch.int32) >= 0).float().mean())
    # rays whose [0, t_max] segment enters the scene's root box (slab test in float64)
    world = d_tris.reshape(-1, 3)
    lo, hi = world.min(0).values.double(), world.max(0).values.double()
    o64, d64 = d_rays[:, :3].double(), d_rays[:, 3:].double()
    with torch.no_grad():
        t0s, t1s = (lo - o64) / d64, (hi - o64) / d64
        tn = torch.minimum(t0s, t1s).max(1).values.clamp_min(0.0)
        tx = torch.maximum(t0s, t1s).min(1).values.minimum(d_tmax.double())
        any_enter_frac = float((tx >= tn).double().mean())
    del any_hits, o64, d64, t0s, t1s, tn, tx

    # ------------------------------------------------------------ e2e through the C ABI with host buffers
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((N_RAYS, 4), dtype=torch.float32).pin_memory()
    lib = rb.load_library()
    import ctypes
    for _ in range(2):
        lib.rtbvh_intersect_mbvh_batch(mbvh.handle, ctypes.c_void_p(h_rays.data_ptr()), None, N_RAYS,
                                       ctypes.c_void_p(h_hits.data_ptr()), 0)
    e2e_times = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        rc = lib.rtbvh_intersect_mbvh_batch(mbvh.handle, ctypes.c_void_p(h_rays.data_ptr()), None, N_RAYS,
                                            ctypes.c_void_p(h_hits.data_ptr()), 0)
        e2e_times.append(time.perf_counter() - t0)
        if rc != 0:
            raise RuntimeError(f"rtbvh_intersect_mbvh_batch -> {rc}")
    e2e = ws * N_RAYS / statistics.median(e2e_times) / 1e6

    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    roofline_own = own_walk_roofline(mbvh, d_rays, st, ms, peak, peak_kind)
    traffic = None
    tp = os.path.join(ROOT, "profiles", "trace_mbvh_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get("bytes_per_launch")

    cpu = None
    parity = None
    workloads = {}
    t_err = None
    if rank == 0:
        sample = 1 << 20
        gpu_sample = step()[:sample].cpu().numpy()
        t_err = t_error_vs_fp64(tris, rays, gpu_sample)
        if not args.no_cpu_baseline:
            cpu, ref_hits = cpu_baseline(tris, rays, sample=sample)
            exact_sample, _ = mbvh.intersect(d_rays[:sample], exact_nodes=True)
            parity = {"against": "oracle (CPU restatement of the reference's LOCB build and Mbvh traversal)",
                      "default_walk": nearest_hit_parity(gpu_sample, ref_hits, tris, rays[:sample]),
                      "exact_node_walk": nearest_hit_parity(exact_sample.cpu().numpy(), ref_hits, tris,
                                                            rays[:sample]),
                      "sample": f"first {sample} of the {N_RAYS} rays (the default walk's hits taken from one "
                                "full-size launch)"}
    build_roofline = {"bytes_per_primitive": B_BUILD, "unit": "GB/s", "peak": peak, "peak_source": peak_kind,
                      "locb_1M": round(B_BUILD * N_TRIS / (statistics.median(build_ms) * 1e-3) / 1e9, 1)}
    build_roofline["locb_1M_frac"] = round(build_roofline["locb_1M"] / peak, 4)
    if rank == 0 and not args.no_extra:
        workloads["sphere_6400_binned_sah"] = workload_sphere_sah(not args.no_cpu_baseline)
        workloads["spatial_sah_teapot"] = workload_spatial("teapot", not args.no_cpu_baseline)
        workloads["spatial_sah_slivers_20k"] = workload_spatial("slivers", not args.no_cpu_baseline)
        workloads["differentiable_200k"] = workload_differentiable()
        workloads["batched_512_meshes"] = workload_batched()
        workloads["clustered_10M_binned_sah"] = workload_clustered()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "incoherent-1M-locb-mbvh", "triangles": N_TRIS, "rays": N_RAYS,
                       "builder": "locally-ordered clustering (radius 14, grid 1024) + 4-wide MBVH",
                       "query": "closest-hit t/u/v/prim", "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if ws > 1 else "single"},
            "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 24,
                    "d2h_bytes_per_step": N_RAYS * 16},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 3), "traffic": traffic,
                         "peak_source": peak_kind,
                         "bytes_per_ray": round(alg_bytes / N_RAYS, 1),
                         "mean_node_visits": round(visits / N_RAYS, 3),
                         "mean_tri_tests": round(tests / N_RAYS, 3),
                         "bytes": "24 ray + 16 hit + 128 per quad node + 40 per triangle, visit counts of the "
                                  "reference's iterator over its Mbvh"},
            "roofline_own_walk": roofline_own,
            "cpu_baseline": cpu,
            # per step: the compact walk and the exact-node pass over the rays it hands on
            "gpu_launches": 2 * args.steps,
            "clocks": clk.summary(),
            "build_ms": {"locb": round(statistics.median(build_ms), 3), "mbvh": round(statistics.median(mbvh_ms), 3)},
            "any_hit": {"value": round(ws * N_RAYS / (any_ms * 1e-3) / 1e6, 2), "unit": "Mrays/s",
                        "t_max": "0.5 x distance", "rays_entering_root_box": round(any_enter_frac, 4),
                        "rays_reporting_a_hit": round(any_hit_frac, 4)},
            "build_roofline": build_roofline,
            "max_stack_depth": max_stack,
            "t_error_vs_fp64": t_err,
            "parity": parity,
            "workloads": workloads,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _cuda_time(fn, reps=5, warmup=2):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def workload_sphere_sah(with_cpu):
    """6,400-triangle sphere, binned SAH + MBVH, 1024x1024 camera rays."""
    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import scenes
    tris = scenes.sphere()
    rays = scenes.camera_rays(1024, 1024)
    d_tris, d_rays = torch.from_numpy(tris).cuda(), torch.from_numpy(rays).cuda()
    holder = {}

    def build():
        holder["bvh"] = rb.Builder(primitives=rb.Triangles(d_tris)).construct_binned_sah(host_mirror=False)
        holder["mbvh"] = rb.Mbvh.construct(holder["bvh"], host_mirror=False)

    sah_ms = _cuda_time(lambda: rb.Builder(primitives=rb.Triangles(d_tris)).construct_binned_sah(host_mirror=False))
    build()
    mbvh_ms = _cuda_time(lambda: rb.Mbvh.construct(holder["bvh"], host_mirror=False))
    m = holder["mbvh"]
    trace_ms = _cuda_time(lambda: m.intersect(d_rays), reps=10)
    # packets of four horizontally adjacent pixels, as examples/benchmark.rs:127-140
    pk_mbvh_ms = _cuda_time(lambda: m.intersect_packets(d_rays), reps=10)
    pk_bvh_ms = _cuda_time(lambda: holder["bvh"].intersect_packets(d_rays), reps=10)
    out = {"triangles": len(tris), "rays": len(rays), "sah_build_ms": round(sah_ms, 3),
           "mbvh_ms": round(mbvh_ms, 3), "closest_hit_mrays": round(len(rays) / (trace_ms * 1e-3) / 1e6, 1),
           "packets": {"mbvh_mrays": round(len(rays) / (pk_mbvh_ms * 1e-3) / 1e6, 1),
                       "bvh_mrays": round(len(rays) / (pk_bvh_ms * 1e-3) / 1e6, 1),
                       "packet": "4 horizontally adjacent pixels, packet triangle test"}}
    if with_cpu:
        import oracle
        threads = os.cpu_count() or 1
        a, c = oracle.triangle_prep(tris)
        t0 = time.perf_counter()
        for _ in range(5):
            nodes, idx = oracle.build(a, c, "sah", spawn_threshold=1024, threads=threads)
        cpu_build = (time.perf_counter() - t0) / 5 * 1e3
        mn = oracle.mbvh(nodes)
        t0 = time.perf_counter()
        oracle.trace("mbvh", mn, idx, tris.reshape(-1, 9), rays, threads=threads, stats=False)
        cpu_rays = len(rays) / (time.perf_counter() - t0) / 1e6
        t0 = time.perf_counter()
        oracle.trace_packets("mbvh", mn, idx, tris.reshape(-1, 9), rays, threads=threads)
        cpu_pk = len(rays) / (time.perf_counter() - t0) / 1e6
        out["cpu_baseline"] = {"sah_build_ms": round(cpu_build, 3), "closest_hit_mrays": round(cpu_rays, 2),
                               "packets_mbvh_mrays": round(cpu_pk, 2), "cores": threads, "kind": "port"}
    return out


def workload_spatial(name, with_cpu):
    """Spatial-split SAH builds (src/builders/spatial_sah.rs) as the reference
    writes them and with every correction, then MBVH closest hit over each
    tree (exact nodes, the reference's order): the 6,320-triangle teapot the
    reference's README times, or 20,000 long thin triangles."""
    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import _ffi, scenes
    if name == "teapot":
        tris = np.load(os.path.join(ROOT, "tests", "golden", "teapot_tris.npy")).astype(np.float32)
        rays = scenes.camera_rays(1024, 1024, eye=(0.0, 1.5, 8.0), fov_deg=40.0)
    else:
        tris = scenes.slivers(20000, seed=5, length=0.2)
        rays, _ = scenes.incoherent_rays(1 << 20, seed=8)
    d_tris, d_rays = torch.from_numpy(tris).cuda(), torch.from_numpy(rays).cuda()
    b = rb.Builder(primitives=rb.Triangles(d_tris))
    out = {"triangles": len(tris), "rays": len(rays)}
    for label, fixes in (("as_written", 0), ("corrected", _ffi.SPATIAL_FIX_ALL)):
        build_ms = _cuda_time(lambda: b.construct_spatial_sah(fixes=fixes, host_mirror=False))
        g = b.construct_spatial_sah(fixes=fixes)
        m = rb.Mbvh.construct(g, host_mirror=False)
        trace_ms = _cuda_time(lambda: m.intersect(d_rays), reps=10)
        ints = g.nodes().view(np.int32)
        out[label] = {"build_ms": round(build_ms, 3), "nodes": len(ints),
                      "leaf_references": int(ints[ints[:, 3] >= 0, 3].sum()),
                      "every_primitive_referenced": g.validate(len(tris)),
                      "closest_hit_mrays": round(len(rays) / (trace_ms * 1e-3) / 1e6, 1)}
    if with_cpu:
        # the reference's threading: a thread per task of more than 1024
        # references (TaskSpawner), the rest on the spawning thread
        import oracle
        cpu = {}
        for label, fixes in (("as_written", 0), ("corrected", oracle.SPATIAL_FIX_ALL)):
            t0 = time.perf_counter()
            oracle.build_spatial(tris, fixes=fixes, spawn_threshold=1024)
            cpu[label + "_build_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        out["cpu_baseline"] = {**cpu, "cores": os.cpu_count() or 1, "kind": "port",
                               "threads": "a thread per task above 1024 references, as TaskSpawner"}
    return out


def workload_differentiable():
    """200,000-triangle sphere, 2048x2048 camera: forward (closest hit),
    backward (hand-written kernel + deterministic per-triangle sums), one
    vertex step and the GPU refit; against the plain per-call path that
    recomputes the triangle test and its gradient in PyTorch ops. The
    workload names no builder: both of the reference's object-split
    builders are timed (LOCB gives the closest hit its compact walk; a
    binned-SAH tree keeps the exact walk until its first refit)."""
    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import diff, scenes
    tris = scenes.sphere_fast(500, 200, radius=1.0, noise=0.05, seed=5)
    rays = scenes.camera_rays(2048, 2048)
    verts = torch.from_numpy(tris).cuda()
    d_rays = torch.from_numpy(rays).cuda()
    g = torch.from_numpy(np.random.default_rng(7).normal(size=(len(rays), 3)).astype(np.float32)).cuda()
    tri_v = verts.view(-1, 3, 3)
    o, d = d_rays[:, :3], d_rays[:, 3:]
    pgv = torch.empty_like(tri_v)

    def cross(a, b):
        return torch.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                            a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], dim=1)

    out = {"triangles": len(tris), "rays": len(rays),
           "plain": "same trace, then the triangle test of the hit triangles recomputed and its gradient "
                    "written in PyTorch ops (no autograd), index_add_ scatter to the triangles"}
    for kind in ("locb", "sah"):
        b = rb.Builder(primitives=rb.Triangles(verts))
        bvh = (b.construct_locally_ordered_clustered(host_mirror=False) if kind == "locb"
               else b.construct_binned_sah(host_mirror=False))
        m = rb.Mbvh.construct(bvh, host_mirror=False)
        gv = torch.empty_like(verts)
        gr = torch.empty_like(d_rays)

        def fused():
            h, _ = m.intersect(d_rays)
            diff.intersect_backward(verts, d_rays, h, g, gv, gr)

        def plain():
            # the per-call path without the library's backward: the same
            # trace, then the triangle test recomputed for the hit triangles
            # and its gradient written out in PyTorch ops (no autograd
            # graph), scattered to the triangles with index_add_
            h, _ = m.intersect(d_rays)
            prim = h[:, 3].contiguous().view(torch.int32)
            hit = (prim >= 0).unsqueeze(1)
            idx = prim.clamp(min=0).long()
            tri = tri_v[idx]
            v0 = tri[:, 0]
            e1, e2 = tri[:, 1] - v0, tri[:, 2] - v0
            hh = cross(d, e2)
            f = (1.0 / (e1 * hh).sum(1, keepdim=True))
            sv = o - v0
            q = cross(sv, e1)
            u = f * (sv * hh).sum(1, keepdim=True)
            vv = f * (d * q).sum(1, keepdim=True)
            t = f * (e2 * q).sum(1, keepdim=True)
            lam = f * (g[:, 0:1] * cross(e1, e2) + g[:, 1:2] * hh + g[:, 2:3] * cross(e1, d))
            lam = torch.where(hit, lam, 0.0)  # misses contribute nothing (their triangle 0 may be degenerate)
            dv = torch.where(hit.unsqueeze(2), torch.stack([-(1.0 - u - vv) * lam, -u * lam, -vv * lam], dim=1),
                             0.0)
            pgv.zero_()
            pgv.index_add_(0, idx, dv)
            return pgv, torch.cat([lam, torch.where(hit, t * lam, 0.0)], dim=1)

        fwd_ms = _cuda_time(lambda: m.intersect(d_rays))
        fused_ms = _cuda_time(fused)
        plain_ms = _cuda_time(plain)
        # both paths give the same gradients (the plain one sums in atomic order)
        fused()
        pv, pr = plain()
        torch.cuda.synchronize()
        rel_v = float((pv.reshape(-1) - gv.reshape(-1)).norm() / gv.norm())
        rel_r = float((pr - gr).norm() / gr.norm())
        step_ms = _cuda_time(lambda: bvh.refit(triangles=verts, mbvh=m), reps=3)
        out[kind] = {"forward_ms": round(fwd_ms, 3), "forward_backward_ms": round(fused_ms, 3),
                     "plain_forward_backward_ms": round(plain_ms, 3),
                     "speedup_vs_plain": round(plain_ms / fused_ms, 2),
                     "refit_and_recollapse_ms": round(step_ms, 3),
                     "plain_vs_fused_rel_diff": {"vertices": float(f"{rel_v:.3g}"), "rays": float(f"{rel_r:.3g}")}}
    out["builder"] = "locally-ordered clustering (the keys below the builder names hold each builder's numbers)"
    for k in ("forward_ms", "forward_backward_ms", "plain_forward_backward_ms", "speedup_vs_plain"):
        out[k] = out["locb"][k]
    return out


def secondary_rays(rays, hits, vertices, per_hit=3, total_hits=None, seed=9):
    """Cosine-weighted hemisphere rays at closest-hit points: origin = hit
    point + 1e-4 * geometric normal (facing the incoming ray), ``per_hit``
    directions per hit point. Hit points are cycled until ``total_hits``
    points are used (default: one per primary ray)."""
    import torch
    R = rays.shape[0]
    total_hits = total_hits or R
    prim = hits[:, 3].contiguous().view(torch.int32)
    hit_idx = torch.nonzero(prim >= 0).squeeze(1)
    if hit_idx.numel() == 0:
        raise RuntimeError("no primary hits to spawn secondary rays from")
    slots = hit_idx[torch.arange(total_hits, device=rays.device) % hit_idx.numel()]
    d = rays[slots, 3:]
    p = rays[slots, :3] + hits[slots, 0:1] * d
    tri = vertices.reshape(-1, 3, 3)[prim[slots].long()]
    n = torch.linalg.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    n = n / n.norm(dim=1, keepdim=True).clamp_min(1e-30)
    n = torch.where(((n * d).sum(1, keepdim=True) > 0), -n, n)
    origin = p + 1e-4 * n
    # orthonormal frame around n
    a = torch.where(n[:, 0:1].abs() > 0.9, torch.tensor([0.0, 1.0, 0.0], device=rays.device),
                    torch.tensor([1.0, 0.0, 0.0], device=rays.device))
    t1 = torch.linalg.cross(n, a)
    t1 = t1 / t1.norm(dim=1, keepdim=True)
    t2 = torch.linalg.cross(n, t1)
    g = torch.Generator(device=rays.device)
    g.manual_seed(seed)
    out = []
    for _ in range(per_hit):
        u1 = torch.rand(total_hits, 1, device=rays.device, generator=g)
        u2 = torch.rand(total_hits, 1, device=rays.device, generator=g)
        r, phi = torch.sqrt(u1), 2.0 * math.pi * u2
        w = r * torch.cos(phi) * t1 + r * torch.sin(phi) * t2 + torch.sqrt((1.0 - u1).clamp_min(0.0)) * n
        w = w / w.norm(dim=1, keepdim=True)
        out.append(torch.cat([origin, w], dim=1))
    return torch.stack(out, dim=1).reshape(-1, 6).contiguous()


def workload_clustered(with_stats=True):
    """64 spheres (10,000,000 triangles, radii log-uniform in [0.01, 0.2],
    Gaussian-mixture centres), binned SAH + MBVH; 4096x4096 camera rays plus
    3 cosine-weighted secondary rays per primary hit point (64M rays)."""
    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import scenes
    tris = scenes.clustered(CLUSTER_TRIS)
    d_tris = torch.from_numpy(tris).cuda()
    del tris
    sah_ms = _cuda_time(lambda: rb.Builder(primitives=rb.Triangles(d_tris)).construct_binned_sah(host_mirror=False),
                        reps=2, warmup=1)
    bvh = rb.Builder(primitives=rb.Triangles(d_tris)).construct_binned_sah(host_mirror=False)
    mbvh_ms = _cuda_time(lambda: rb.Mbvh.construct(bvh, host_mirror=False), reps=3, warmup=1)
    m = rb.Mbvh.construct(bvh, host_mirror=False)
    primary = torch.from_numpy(scenes.camera_rays(CLUSTER_CAMERA, CLUSTER_CAMERA)).cuda()
    ph, _ = m.intersect(primary)
    primary_hits = int((ph[:, 3].contiguous().view(torch.int32) >= 0).sum())
    sec = secondary_rays(primary, ph, d_tris, per_hit=3)
    del ph
    allr = torch.cat([primary, sec])
    del sec
    R = allr.shape[0]
    ms = _cuda_time(lambda: m.intersect(allr), reps=3, warmup=2)
    sec_ms = _cuda_time(lambda: m.intersect(allr[primary.shape[0]:]), reps=3, warmup=1)
    peak, kind = measured_peak()
    sah_gbs = B_BUILD * int(d_tris.shape[0]) / (sah_ms * 1e-3) / 1e9
    out = {"triangles": int(d_tris.shape[0]), "rays": int(R), "primary_hits": primary_hits,
           "sah_build_ms": round(sah_ms, 2), "mbvh_ms": round(mbvh_ms, 2),
           "build_roofline": {"bytes_per_primitive": B_BUILD, "achieved_gbs": round(sah_gbs, 1),
                              "frac": round(sah_gbs / peak, 4), "peak_source": kind},
           "closest_hit_mrays": round(R / (ms * 1e-3) / 1e6, 1),
           "secondary_only_mrays": round((R - primary.shape[0]) / (sec_ms * 1e-3) / 1e6, 1)}
    if with_stats:
        _, st = m.intersect(allr, stats=True)
        st = st.to(torch.int64)
        nv, nt = float(st[:, 0].sum()) / R, float(st[:, 1].sum()) / R
        bpr = B_IN + B_OUT + B_NODE * nv + B_TRI * nt
        ach = bpr * R / (ms * 1e-3) / 1e9
        out["roofline"] = {"bytes_per_ray": round(bpr, 1), "mean_node_visits": round(nv, 3),
                           "mean_tri_tests": round(nt, 3), "achieved_gbs": round(ach, 1),
                           "frac": round(ach / peak, 3), "peak_source": kind}
        out["roofline_own_walk"] = own_walk_roofline(m, allr, st, ms, peak, kind)
    if m.status() != rb.ResultCode.Ok:
        raise RuntimeError("clustered traversal reported an error")
    return out


def workload_batched(mesh_count=512, seed=44):
    """512 perturbed spheres, triangle counts log-uniform in [64, 200,000],
    round(2000 sqrt(n)) incoherent rays each: one captured build + trace for
    all meshes against the per-mesh loop (build, collapse, trace per mesh)."""
    import math

    import torch

    import rtbvh_gb300 as rb
    from rtbvh_gb300 import scenes
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(math.log(64), math.log(200_000), size=mesh_count)).astype(np.int64)
    parts, rays, po, ro = [], [], [0], [0]
    for m, n in enumerate(counts):
        cells = max(2, int(n) // 2)
        n_lat = max(2, int(round(math.sqrt(cells / 2.0))))
        n_lon = max(3, int(round(cells / n_lat)))
        centre = tuple(rng.uniform(-5, 5, size=3))
        t = scenes.sphere_fast(n_lon, n_lat, radius=1.0, noise=0.05, seed=seed * 10000 + m, center=centre)
        r, _ = scenes.incoherent_rays(int(round(2000 * math.sqrt(len(t)))), seed=seed * 10000 + 5000 + m,
                                      center=(0.0, 0.0, 0.0), radius=2.0, lo=-1.0, hi=1.0)
        r[:, :3] += np.asarray(centre, dtype=np.float32)  # origins and targets move with the mesh
        parts.append(t)
        rays.append(r)
        po.append(po[-1] + len(t))
        ro.append(ro[-1] + len(r))
    tris = np.concatenate(parts)
    allr = np.concatenate(rays)
    d_tris, d_rays = torch.from_numpy(tris).cuda(), torch.from_numpy(allr).cuda()
    batch = rb.Batch(d_tris, po, d_rays, ro)
    default_ms = _cuda_time(lambda: batch.run(), reps=5, warmup=1)
    tuning = batch.tune()
    graph_ms = _cuda_time(lambda: batch.run(), reps=5, warmup=1)
    eager_ms = _cuda_time(lambda: batch.run(graph=False), reps=3, warmup=1)
    if batch.status() != rb.ResultCode.Ok:
        raise RuntimeError("batched run reported an error")

    def per_mesh():
        for m in range(mesh_count):
            b = rb.Builder(primitives=rb.Triangles(d_tris[po[m]:po[m + 1]])).construct_locally_ordered_clustered(
                host_mirror=False)
            mb = rb.Mbvh.construct(b, host_mirror=False)
            mb.intersect(d_rays[ro[m]:ro[m + 1]])

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    per_mesh()
    torch.cuda.synchronize()
    loop_ms = (time.perf_counter() - t0) * 1e3
    return {"meshes": mesh_count, "triangles": int(po[-1]), "rays": int(ro[-1]),
            "graph_build_trace_ms": round(graph_ms, 2), "untuned_graph_ms": round(default_ms, 2),
            "tuning": {k: (round(v, 2) if isinstance(v, float) else v) for k, v in tuning.items()},
            "uncaptured_build_trace_ms": round(eager_ms, 2),
            "per_mesh_loop_ms": round(loop_ms, 2), "speedup_vs_per_mesh_loop": round(loop_ms / graph_ms, 2),
            "mrays_including_build": round(ro[-1] / (graph_ms * 1e-3) / 1e6, 1)}


def cpu_baseline(tris, rays, threads=None, sample=1 << 20):
    """CPU restatement of the reference (oracle) on the host cores: LOCB +
    MBVH build once, then the rayon-style chunked traversal of a ray sample.
    Returns (the cpu_baseline entry, the oracle's hits of the sample)."""
    import oracle
    threads = threads or os.cpu_count() or 1
    a, c = oracle.triangle_prep(tris)
    t0 = time.perf_counter()
    nodes, idx = oracle.build(a, c, "locb", threads=threads)
    m = oracle.mbvh(nodes)
    build_s = time.perf_counter() - t0
    sub = rays[:sample]
    t0 = time.perf_counter()
    hits, _, _ = oracle.trace("mbvh", m, idx, tris.reshape(-1, 9), sub, threads=threads, stats=False)
    dt = time.perf_counter() - t0
    return {"value": round(len(sub) / dt / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"first {len(sub)} of the {N_RAYS} rays; LOCB+MBVH build {build_s:.2f} s (not in value)"}, hits


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's traversal on
    all host cores, each step a bounded sample of the same workload."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from oracle import buildlib
    buildlib.build()
    tris, rays, _ = make_scene()
    threads = os.cpu_count() or 1
    a, c = oracle.triangle_prep(tris)
    nodes, idx = oracle.build(a, c, "locb", threads=threads)
    m = oracle.mbvh(nodes)
    flat = tris.reshape(-1, 9)
    sample = min(500_000, N_RAYS // 2)
    times = []
    for s in range(args.warmup + args.steps):
        lo = (s * sample) % (N_RAYS - sample)
        sub = rays[lo:lo + sample]
        t0 = time.perf_counter()
        oracle.trace("mbvh", m, idx, flat, sub, threads=threads, stats=False)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    ms = statistics.mean(times) * 1e3
    value = sample * len(times) / sum(times) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "incoherent-1M-locb-mbvh", "triangles": N_TRIS, "rays": N_RAYS,
                   "sample_rays_per_step": sample,
                   "sampling": f"each step times a {sample}-ray slice of the {N_RAYS}-ray set (the CPU needs "
                               "about 8 s for all of them); value = sampled rays / their time"},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} consecutive rays per step of the {N_RAYS}-ray set"},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


ONLY_WORKLOADS = {
    "sphere_6400_binned_sah": lambda: workload_sphere_sah(False),
    "spatial_sah_teapot": lambda: workload_spatial("teapot", True),
    "spatial_sah_slivers_20k": lambda: workload_spatial("slivers", True),
    "differentiable_200k": lambda: workload_differentiable(),
    "batched_512_meshes": lambda: workload_batched(),
    "clustered_10M_binned_sah": lambda: workload_clustered(False),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--rays", type=int, default=0, help="profiling only: fewer rays")
    ap.add_argument("--tris", type=int, default=0, help="profiling only: fewer triangles")
    ap.add_argument("--exact-nodes", action="store_true",
                    help="profiling only: time the closest hit over the exact 128-byte quad nodes")
    ap.add_argument("--only", default="", choices=["", *ONLY_WORKLOADS],
                    help="profiling only: run one secondary workload and print its JSON")
    args = ap.parse_args()
    apply_size_overrides(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        import torch
        from rtbvh_gb300 import build as libbuild
        torch.cuda.set_device(0)
        libbuild.build()
        print(json.dumps({args.only: ONLY_WORKLOADS[args.only]()}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
