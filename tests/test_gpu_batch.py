"""GPU parity: many meshes built and traced in one captured pipeline
(rtbvh_gpu_batch_*) against the same meshes built and traced one by one.
Per mesh, nodes, primitive order, quad nodes and hits must be the
single-mesh results with indices shifted by the mesh's offsets."""
import numpy as np
import pytest
import torch

import rtbvh_gb300 as rb
from rtbvh_gb300 import scenes
from gpu_helpers import gpu_build, to_cuda, u32

pytestmark = pytest.mark.gpu


def make_meshes(sizes, seed=0):
    tris, rays, po, ro = [], [], [0], [0]
    for i, n in enumerate(sizes):
        t = scenes.incoherent(n, seed=seed * 1000 + i)
        t = (t * np.float32(0.5 + 0.1 * i)).astype(np.float32)  # different world boxes per mesh
        r, _ = scenes.incoherent_rays(max(64, int(round(20 * np.sqrt(n)))), seed=seed * 1000 + 500 + i,
                                      center=tuple(0.25 * (1 + 0.1 * i) * np.ones(3)), radius=1.5)
        tris.append(t)
        rays.append(r)
        po.append(po[-1] + n)
        ro.append(ro[-1] + len(r))
    return np.concatenate(tris), np.concatenate(rays), po, ro


def shifted_nodes(nodes, nbase, off):
    out = nodes.copy()
    ints = out.view(np.int32)
    leaf = ints[:, 3] >= 0
    ints[leaf, 7] += off
    ints[~leaf, 7] += nbase
    return out


def shifted_quads(q, mbase, off):
    out = q.copy()
    ints = out.view(np.int32)
    ch, cnt = ints[:, 24:28], ints[:, 28:32]
    leaf = cnt >= 0
    inner = (cnt < 0) & (ch >= 0)
    ch[leaf] += off
    ch[inner] += mbase
    return out


@pytest.mark.parametrize("sizes", [[1, 2, 3, 17, 300, 5000, 2, 40000, 1, 900, 64, 12000],
                                   [2049, 2048, 2047, 4096, 33, 7],
                                   [4097, 8193, 65537, 3, 100000, 6000, 4096]])
def test_batch_matches_single_mesh_builds(lib, sizes):
    torch.cuda.set_device(0)
    tris, rays, po, ro = make_meshes(sizes, seed=len(sizes))
    batch = rb.Batch(to_cuda(tris), po, to_cuda(rays), ro)
    hits = batch.run().cpu().numpy()
    assert batch.status() == rb.ResultCode.Ok
    v = batch.view()
    M = len(sizes)
    nodes = rb.device_copy(v.nodes, (v.node_capacity, 8))
    idx = rb.device_copy(v.indices, (po[-1],), np.uint32)
    mbase = rb.device_copy(v.mnode_base, (M + 1,), np.uint32)
    quads = rb.device_copy(v.mnodes, (int(mbase[-1]), 32))
    for m, n in enumerate(sizes):
        off, nbase = po[m], 2 * po[m] - m
        g = gpu_build(tris[off:off + n], "locb")
        gn = g.nodes()
        assert np.array_equal(u32(nodes[nbase:nbase + len(gn)]), u32(shifted_nodes(gn, nbase, off))), m
        assert np.array_equal(idx[off:off + n], g.indices() + off), m
        gm = rb.Mbvh.construct(g)
        gq = gm.quad_nodes()
        assert mbase[m + 1] - mbase[m] == len(gq), m
        assert np.array_equal(u32(quads[mbase[m]:mbase[m + 1]]), u32(shifted_quads(gq, mbase[m], off))), m
        h1, _ = gm.intersect(to_cuda(rays[ro[m]:ro[m + 1]]))
        h1 = h1.cpu().numpy()
        hb = hits[ro[m]:ro[m + 1]]
        assert np.array_equal(u32(hb[:, :3]), u32(h1[:, :3])), m
        p1 = rb.hit_prims(h1)
        assert np.array_equal(rb.hit_prims(hb), np.where(p1 >= 0, p1 + off, p1)), m


def test_batch_graph_replay_and_uncaptured_agree(lib):
    torch.cuda.set_device(0)
    tris, rays, po, ro = make_meshes([500, 3000, 40, 8000, 2], seed=3)
    d_tris = to_cuda(tris)
    batch = rb.Batch(d_tris, po, to_cuda(rays), ro)
    a = batch.run().clone()
    b = batch.run().clone()
    c = batch.run(graph=False).clone()
    torch.cuda.synchronize()
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    assert torch.equal(a.view(torch.int32), c.view(torch.int32))
    # the graph reads the bound vertex buffer: moving the geometry in place changes the result
    d_tris.mul_(1.5)
    d = batch.run().clone()
    torch.cuda.synchronize()
    assert not torch.equal(a.view(torch.int32), d.view(torch.int32))


def test_batch_rejects_empty_meshes(lib):
    tris, rays, po, ro = make_meshes([10, 20], seed=4)
    with pytest.raises(rb.RtbvhError):
        rb.Batch(to_cuda(tris), [0, 10, 10, 30], to_cuda(rays), [0, ro[1], ro[1], ro[2]])


def test_batch_tuning_keeps_results(lib):
    """Launch parameters change the schedule, never the hits."""
    torch.cuda.set_device(0)
    tris, rays, po, ro = make_meshes([5000, 3, 20000, 700, 4097, 9000], seed=6)
    batch = rb.Batch(to_cuda(tris), po, to_cuda(rays), ro)
    ref = batch.run().clone()
    torch.cuda.synchronize()
    chosen = batch.tune()
    assert chosen["cluster_min_prims"] in (2048, 4096, 8192, 16384, 65536)
    assert chosen["trace_ray_batch"] in (32, 64, 128, 256)
    assert chosen["trace_blocks_per_sm"] in (0, 2, 4)
    assert chosen["pipeline_ms"] > 0
    assert chosen["trace_stack"] in (32, 48, 64)
    assert batch.tuning["cluster_min_prims"] == chosen["cluster_min_prims"]
    assert batch.tuning["trace_stack"] == chosen["trace_stack"]
    out = batch.run().clone()
    torch.cuda.synchronize()
    assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
    assert batch.status() == rb.ResultCode.Ok
    # extreme settings: every mesh of > 2 primitives clustered, one block per SM, 1-ray batches
    for stack in (32, 48, 64):
        batch.set_tuning(trace_blocks_per_sm=1, trace_ray_batch=1, cluster_min_prims=2, trace_stack=stack)
        out = batch.run().clone()
        torch.cuda.synchronize()
        assert torch.equal(out.view(torch.int32), ref.view(torch.int32)), f"stack bound {stack}"
        assert batch.status() == rb.ResultCode.Ok
    with pytest.raises(rb.RtbvhError):
        batch.set_tuning(trace_stack=40)



def test_batch_config_sized_meshes_match_the_oracle(lib):
    """Meshes built as the batched workload builds them (perturbed spheres,
    round(2000 sqrt(n)) incoherent rays each), the largest at the workload's
    upper size of 200,000 triangles: every mesh's nodes equal the oracle's
    LOCB build and its hits the oracle's traversal (the same nearest hit;
    primitive ids shifted by the mesh's offset)."""
    import math
    import os

    import oracle
    from gpu_helpers import assert_same_nearest
    torch.cuda.set_device(0)
    rng = np.random.Generator(np.random.PCG64(45))
    sizes = [200_000, 64, 37_000, 1_500]
    parts, rays, po, ro = [], [], [0], [0]
    for m, n in enumerate(sizes):
        cells = max(2, n // 2)
        n_lat = max(2, int(round(math.sqrt(cells / 2.0))))
        n_lon = max(3, int(round(cells / n_lat)))
        centre = tuple(rng.uniform(-5, 5, size=3))
        t = scenes.sphere_fast(n_lon, n_lat, radius=1.0, noise=0.05, seed=450000 + m, center=centre)
        r, _ = scenes.incoherent_rays(int(round(2000 * math.sqrt(len(t)))), seed=455000 + m,
                                      center=(0.0, 0.0, 0.0), radius=2.0, lo=-1.0, hi=1.0)
        r[:, :3] += np.asarray(centre, dtype=np.float32)
        parts.append(t)
        rays.append(r)
        po.append(po[-1] + len(t))
        ro.append(ro[-1] + len(r))
    tris, allr = np.concatenate(parts), np.concatenate(rays)
    batch = rb.Batch(to_cuda(tris), po, to_cuda(allr), ro)
    hits = batch.run().cpu().numpy()
    assert batch.status() == rb.ResultCode.Ok
    v = batch.view()
    nodes = rb.device_copy(v.nodes, (v.node_capacity, 8))
    threads = os.cpu_count() or 1
    for m in range(len(sizes)):
        off, n, nbase = po[m], po[m + 1] - po[m], 2 * po[m] - m
        mt = tris[off:off + n]
        a, c = oracle.triangle_prep(mt)
        on, oi = oracle.build(a, c, "locb", threads=threads)
        assert np.array_equal(u32(nodes[nbase:nbase + len(on)]), u32(shifted_nodes(on, nbase, off))), m
        mr = allr[ro[m]:ro[m + 1]]
        oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, mt.reshape(-1, 9), mr, threads=threads, stats=False)
        hb = hits[ro[m]:ro[m + 1]].copy()
        p = rb.hit_prims(hb)
        hb[:, 3] = np.where(p >= 0, p - off, p).astype(np.int32).view(np.float32)
        assert_same_nearest(hb, oh, mt, mr)
