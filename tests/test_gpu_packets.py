"""GPU parity of the packet traversal (four rays per walk) against the
oracle's restatement of the reference's packet iterators
(src/iter_indices.rs:110-414) and packet triangle test
(src/builders/spatial_sah.rs:165-244): hits bit for bit, per-packet node and
triangle counts equal."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import _ffi, scenes
from gpu_helpers import gpu_build, oracle_build, rays_for, scene, to_cuda, u32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


def _gpu_packets(structure, rays, t=None):
    hits, st = structure.intersect_packets(to_cuda(rays), t=None if t is None else to_cuda(t), stats=True)
    torch.cuda.synchronize()
    assert structure.status() == rb.ResultCode.Ok
    return hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("name", ["teapot", "sphere", "incoherent_20k"])
@pytest.mark.parametrize("kind", ["mbvh", "bvh"])
def test_packets_locb_bit_exact(name, kind):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    rays, _ = rays_for(name, count=8192)
    on, oi = oracle_build(tris, "locb")
    if kind == "mbvh":
        s, nodes = rb.Mbvh.construct(g), oracle.mbvh(on)
    else:
        s, nodes = g, on
    hits, st = _gpu_packets(s, rays)
    oh, ost, bad = oracle.trace_packets(kind, nodes, oi, tris.reshape(-1, 9), rays)
    assert bad == 0
    assert np.array_equal(u32(hits), u32(oh)), "t/u/v/prim differ"
    assert np.array_equal(st, ost), "node / triangle / stack counts differ"
    assert (rb.hit_prims(hits) >= 0).sum() > 0


def test_packets_sah_mbvh_bit_exact():
    tris = scene("sphere")
    g = gpu_build(tris, "sah")
    m = rb.Mbvh.construct(g)
    rays, _ = rays_for("sphere")
    hits, st = _gpu_packets(m, rays)
    on, oi = oracle_build(tris, "sah")
    om = oracle.mbvh(on)
    assert np.array_equal(u32(m.quad_nodes()), u32(om))
    oh, ost, _ = oracle.trace_packets("mbvh", om, oi, tris.reshape(-1, 9), rays)
    assert np.array_equal(u32(hits), u32(oh))
    assert np.array_equal(st, ost)


def test_packets_sah_bvh_same_nearest():
    # the GPU SAH build numbers nodes breadth-first and orders leaf members
    # stably, so the BVH2 walk is the same tree in another numbering: t and
    # the counts agree exactly; a leaf's members may be tested in another order
    tris = scenes.incoherent(20000, seed=31)
    g = gpu_build(tris, "sah")
    rays, _ = scenes.incoherent_rays(8192, seed=32)
    hits, st = _gpu_packets(g, rays)
    on, oi = oracle_build(tris, "sah")
    oh, ost, _ = oracle.trace_packets("bvh", on, oi, tris.reshape(-1, 9), rays)
    assert np.array_equal(u32(hits[:, 0]), u32(oh[:, 0]))
    assert np.array_equal(st[:, :2], ost[:, :2])
    same = rb.hit_prims(hits) == rb.hit_prims(oh)
    assert same.mean() > 0.999


@pytest.mark.parametrize("kind", ["mbvh", "bvh"])
def test_packets_t_bound_in_and_out(kind):
    tris = scene("incoherent_20k")
    rays, tmax = scenes.incoherent_rays(4096, seed=33)
    g = gpu_build(tris, "locb")
    on, oi = oracle_build(tris, "locb")
    s, nodes = (rb.Mbvh.construct(g), oracle.mbvh(on)) if kind == "mbvh" else (g, on)
    hits, st = _gpu_packets(s, rays, t=tmax)
    oh, ost, _ = oracle.trace_packets(kind, nodes, oi, tris.reshape(-1, 9), rays, t=tmax)
    assert np.array_equal(u32(hits), u32(oh))
    assert np.array_equal(st, ost)
    # t is in/out through the C ABI
    r = to_cuda(rays)
    soa = r.t().contiguous()
    t = to_cuda(tmax).clone()
    fn = s._lib.rtbvh_gpu_intersect_mbvh_packets if kind == "mbvh" else s._lib.rtbvh_gpu_intersect_bvh_packets
    ptrs = [ctypes.c_void_p(soa[k].data_ptr()) for k in range(6)]
    rc = fn(s.handle, *ptrs, ctypes.c_void_p(t.data_ptr()), len(rays) // 4, None, 0, None, None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(u32(t.cpu().numpy()), u32(oh[:, 0]))


@pytest.mark.parametrize("kind", ["mbvh", "bvh"])
def test_packets_axis_aligned_and_nan_lanes(kind):
    # zero direction components (infinite inverses, NaN slab values) and NaN
    # lanes follow the iterators' select rules; a NaN lane stops a BVH2 packet
    tris = scenes.incoherent(3000, seed=34)
    rng = np.random.default_rng(35)
    R = 2048
    o = rng.uniform(-0.5, 1.5, size=(R, 3)).astype(np.float32)
    d = np.zeros((R, 3), np.float32)
    axis = rng.integers(0, 3, size=R)
    d[np.arange(R), axis] = rng.choice([-1.0, 1.0], size=R)
    o[::7, axis[::7]] = 0.25  # origins on a plane through box faces
    rays = np.concatenate([o, d], 1).astype(np.float32)
    rays[5, 0] = np.nan
    rays[42, 4] = np.nan
    g = gpu_build(tris, "locb")
    on, oi = oracle_build(tris, "locb")
    s, nodes = (rb.Mbvh.construct(g), oracle.mbvh(on)) if kind == "mbvh" else (g, on)
    hits, st = _gpu_packets(s, rays)
    oh, ost, _ = oracle.trace_packets(kind, nodes, oi, tris.reshape(-1, 9), rays)
    assert np.array_equal(u32(hits), u32(oh))
    assert np.array_equal(st, ost)


def test_packets_reject_unsupported_flags():
    tris = scenes.incoherent(500, seed=36)
    m = rb.Mbvh.construct(gpu_build(tris, "locb"))
    r = torch.zeros((8, 6), dtype=torch.float32, device="cuda")
    soa = r.t().contiguous()
    t = torch.full((8,), 1e34, dtype=torch.float32, device="cuda")
    ptrs = [ctypes.c_void_p(soa[k].data_ptr()) for k in range(6)]
    for flag in (_ffi.TRACE_ANY_HIT, _ffi.TRACE_REORDER):
        rc = m._lib.rtbvh_gpu_intersect_mbvh_packets(m.handle, *ptrs, ctypes.c_void_p(t.data_ptr()), 2, None, flag,
                                                     None, None)
        assert rc == rb.ResultCode.InvalidArgument
    with pytest.raises(ValueError):
        m.intersect_packets(torch.zeros((6, 6), device="cuda"))
