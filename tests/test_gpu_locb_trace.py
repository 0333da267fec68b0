"""GPU parity: locally-ordered clustering, MBVH collapse and traversal
against the oracle, bit for bit (integer results exactly; float results by
their bit patterns, since the arithmetic is the same IEEE single sequence)."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import _ffi, scenes
from gpu_helpers import assert_same_nearest, gpu_build, oracle_build, rays_for, scene, to_cuda, u32

pytestmark = pytest.mark.gpu

SCENES = ["teapot", "sphere", "incoherent_20k", "incoherent_300k"]


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", SCENES)
def test_locb_nodes_bit_exact(name):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    on, oi = oracle_build(tris, "locb")
    assert np.array_equal(g.indices(), oi), "Morton order differs"
    assert np.array_equal(u32(g.nodes()), u32(on)), "node arrays differ"


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 16, 17, 31, 100, 257, 2047, 2048, 2049, 4097, 9000])
def test_locb_sizes(n):
    tris = scenes.incoherent(n, seed=100 + n)
    g = gpu_build(tris, "locb")
    on, oi = oracle_build(tris, "locb")
    assert np.array_equal(g.indices(), oi)
    assert np.array_equal(u32(g.nodes()), u32(on))


def test_locb_identical_primitives():
    # every box and centre equal: all distances tie, the lowest index wins
    t = np.tile(np.asarray([[[0.1, 0.2, 0.3], [0.4, 0.2, 0.3], [0.1, 0.6, 0.3]]], np.float32), (777, 1, 1))
    g = gpu_build(t, "locb")
    on, oi = oracle_build(t, "locb")
    assert np.array_equal(g.indices(), oi)
    assert np.array_equal(u32(g.nodes()), u32(on))


@pytest.mark.parametrize("name", SCENES)
def test_mbvh_bit_exact(name):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    on, oi = oracle_build(tris, "locb")
    om = oracle.mbvh(on)
    assert np.array_equal(u32(m.quad_nodes()), u32(om))
    assert np.array_equal(m.indices(), oi)


@pytest.mark.parametrize("name", SCENES)
def test_trace_closest_bit_exact(name):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    rays, _ = rays_for(name)
    hits, st = m.intersect(to_cuda(rays), stats=True)
    assert m.status() == rb.ResultCode.Ok
    hits, st = hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)
    on, oi = oracle_build(tris, "locb")
    om = oracle.mbvh(on)
    oh, ost, bad = oracle.trace("mbvh", om, oi, tris.reshape(-1, 9), rays)
    assert bad == 0
    assert np.array_equal(u32(hits), u32(oh)), "t/u/v/prim differ"
    assert np.array_equal(st, ost), "node-visit / triangle-test / stack counts differ"
    assert (rb.hit_prims(hits) >= 0).sum() > 0


@pytest.mark.parametrize("name", ["teapot", "incoherent_300k"])
def test_trace_any_hit_bit_exact(name):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    rays, tmax = rays_for(name)
    if tmax is None:
        tmax = np.full(len(rays), 9.0, np.float32)
    hits, st = m.intersect(to_cuda(rays), t_max=to_cuda(tmax), any_hit=True, stats=True)
    hits, st = hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)
    on, oi = oracle_build(tris, "locb")
    oh, ost, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays, t_max=tmax, any_hit=True)
    assert np.array_equal(u32(hits), u32(oh))
    assert np.array_equal(st, ost)


@pytest.mark.parametrize("name", ["teapot", "incoherent_20k"])
def test_trace_bvh2_bit_exact(name):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    rays, _ = rays_for(name)
    hits, st = g.intersect(to_cuda(rays), stats=True)
    hits, st = hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)
    on, oi = oracle_build(tris, "locb")
    oh, ost, _ = oracle.trace("bvh", on, oi, tris.reshape(-1, 9), rays)
    assert np.array_equal(u32(hits), u32(oh))
    assert np.array_equal(st, ost)


@pytest.mark.parametrize("count", [3_000_000, 12_500_000])
def test_host_buffer_entry_matches_device_entry(count):
    tris = scene("incoherent_20k")
    m = rb.Mbvh.construct(gpu_build(tris, "locb"))
    rays, tmax = scenes.incoherent_rays(count, seed=9)  # 2 and 5 internal chunks
    dev, _ = m.intersect(to_cuda(rays))
    host = m.intersect_host(rays)
    assert np.array_equal(u32(host), u32(dev.cpu().numpy()))
    dev_a, _ = m.intersect(to_cuda(rays), t_max=to_cuda(tmax), any_hit=True)
    host_a = m.intersect_host(rays, t_max=tmax, any_hit=True)
    assert np.array_equal(u32(host_a), u32(dev_a.cpu().numpy()))


def test_pinned_host_buffers_are_traced_in_place():
    # page-locked host buffers: the traversal reads rays and writes hits in
    # host memory directly; mixed (pinned rays, pageable hits) takes the
    # staged copies; both equal the device entry
    tris = scene("incoherent_20k")
    m = rb.Mbvh.construct(gpu_build(tris, "locb"))
    rays, tmax = scenes.incoherent_rays(2_000_000, seed=19)
    lib = _ffi.load()
    h_rays = torch.from_numpy(rays).pin_memory()
    h_tmax = torch.from_numpy(tmax).pin_memory()
    for any_hit in (False, True):
        dev, _ = m.intersect(to_cuda(rays), t_max=to_cuda(tmax) if any_hit else None, any_hit=any_hit)
        want = u32(dev.cpu().numpy())
        flags = _ffi.TRACE_ANY_HIT if any_hit else 0
        tptr = ctypes.c_void_p(h_tmax.data_ptr()) if any_hit else None
        h_hits = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory()
        assert lib.rtbvh_intersect_mbvh_batch(m.handle, ctypes.c_void_p(h_rays.data_ptr()), tptr, len(rays),
                                              ctypes.c_void_p(h_hits.data_ptr()), flags) == 0
        assert np.array_equal(u32(h_hits.numpy()), want)
        pageable = np.empty((len(rays), 4), np.float32)
        assert lib.rtbvh_intersect_mbvh_batch(m.handle, ctypes.c_void_p(h_rays.data_ptr()), tptr, len(rays),
                                              pageable.ctypes.data_as(ctypes.c_void_p), flags) == 0
        assert np.array_equal(u32(pageable), want)


def test_legacy_c_abi_roundtrip(lib):
    # create_bvh / create_mbvh / intersect_mbvh / free_* with host inputs,
    # as a C caller of the reference uses them
    tris = scene("teapot")
    a, c = oracle.triangle_prep(tris)
    c4 = np.zeros((len(c), 4), np.float32)
    c4[:, :3] = c
    out = _ffi.RTBvh()
    for stride, cc in ((12, c), (16, c4)):
        cc = np.ascontiguousarray(cc)
        rc = lib.create_bvh(a.ctypes.data_as(ctypes.POINTER(_ffi.RTAabb)), len(a),
                            cc.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), stride, 1, 0, ctypes.byref(out))
        assert rc == 0
        on, oi = oracle.build(a, c, "locb")
        assert out.node_count == len(on) and out.index_count == len(oi)
        nodes = np.ctypeslib.as_array(ctypes.cast(out.nodes, ctypes.POINTER(ctypes.c_float)), (out.node_count * 8,))
        assert np.array_equal(u32(nodes.reshape(-1, 8)), u32(on))
        mo = _ffi.RTMbvh()
        assert lib.create_mbvh(out, ctypes.byref(mo)) == 0
        mn = np.ctypeslib.as_array(ctypes.cast(mo.nodes, ctypes.POINTER(ctypes.c_float)), (mo.node_count * 32,))
        assert np.array_equal(u32(mn.reshape(-1, 32)), u32(oracle.mbvh(on)))
        lib.free_mbvh(mo)
        lib.free_bvh(out)


def test_legacy_create_bvh_without_aabbs(lib):
    # aabbs NULL: the boxes are the points themselves (rtbvh_ffi/src/lib.rs:396-422)
    pts = np.random.default_rng(1).uniform(-1, 1, size=(5000, 3)).astype(np.float32)
    out = _ffi.RTBvh()
    rc = lib.create_bvh(None, len(pts), pts.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 12, 1, 0,
                        ctypes.byref(out))
    assert rc == 0
    a = np.zeros((len(pts), 8), np.float32)
    a[:, 0:3] = pts
    a[:, 4:7] = pts
    on, oi = oracle.build(a, pts, "locb")
    nodes = np.ctypeslib.as_array(ctypes.cast(out.nodes, ctypes.POINTER(ctypes.c_float)), (out.node_count * 8,))
    assert np.array_equal(u32(nodes.reshape(-1, 8)), u32(on))
    lib.free_bvh(out)


def test_refit_bounds_bit_exact():
    tris = scene("incoherent_20k")
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    before = g.nodes()
    moved = (tris + np.random.default_rng(2).normal(scale=1e-3, size=tris.shape)).astype(np.float32)
    g.refit(triangles=to_cuda(moved), mbvh=m)
    after = g.nodes()
    # topology is kept ...
    assert np.array_equal(u32(after)[:, [3, 7]], u32(before)[:, [3, 7]])
    # ... and the boxes equal the reference's refit bit for bit
    a2, _ = oracle.triangle_prep(moved)
    ref = oracle.refit(before, g.indices(), a2)
    cols = [0, 1, 2, 4, 5, 6]
    assert np.array_equal(u32(after)[:, cols], u32(ref)[:, cols])
    # the re-collapsed MBVH equals the collapse of the refitted tree
    assert np.array_equal(u32(m.quad_nodes()), u32(oracle.mbvh(after)))
    # and tracing the moved triangles matches the oracle
    rays, _ = scenes.incoherent_rays(8192, seed=4)
    hits, _ = m.intersect(to_cuda(rays))
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(after), g.indices(), moved.reshape(-1, 9), rays)
    assert np.array_equal(u32(hits.cpu().numpy()), u32(oh))


def test_morton_order_1m_is_a_stable_sort():
    tris = scenes.incoherent(1_000_000, seed=2)
    g = rb.Builder(primitives=rb.Triangles(to_cuda(tris))).construct_locally_ordered_clustered(host_mirror=True)
    a, c = oracle.triangle_prep(tris)
    codes, idx = oracle.morton_codes(a, c)
    gi = g.indices()
    assert np.array_equal(gi, idx)
    assert (np.diff(codes[gi].astype(np.int64)) >= 0).all()


def test_locb_1m_bit_exact_and_valid():
    tris = scenes.incoherent(1_000_000, seed=2)
    g = gpu_build(tris, "locb")
    nodes = g.nodes()
    assert len(nodes) == 2 * len(tris) - 1
    assert g.validate(len(tris))
    on, oi = oracle_build(tris, "locb")
    assert np.array_equal(u32(nodes), u32(on))
    m = rb.Mbvh.construct(g)
    assert np.array_equal(u32(m.quad_nodes()), u32(oracle.mbvh(on)))


def test_sorted_large_batch_matches_oracle():
    # with RTBVH_TRACE_REORDER rays are traced in (origin, direction)-sorted
    # order; each ray's result and counts must be unchanged
    tris = scene("incoherent_300k")
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    rays, tmax = scenes.incoherent_rays(1_000_000, seed=31)
    hits, st = m.intersect(to_cuda(rays), stats=True, reorder=True)
    hits, st = hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)
    plain, _ = m.intersect(to_cuda(rays))
    assert np.array_equal(u32(hits), u32(plain.cpu().numpy()))
    on, oi = oracle_build(tris, "locb")
    om = oracle.mbvh(on)
    pick = np.random.default_rng(3).choice(len(rays), 20000, replace=False)
    oh, ost, _ = oracle.trace("mbvh", om, oi, tris.reshape(-1, 9), rays[pick])
    assert np.array_equal(u32(hits[pick]), u32(oh))
    assert np.array_equal(st[pick], ost)
    ha, sta = m.intersect(to_cuda(rays), t_max=to_cuda(tmax), any_hit=True, stats=True, reorder=True)
    oha, osta, _ = oracle.trace("mbvh", om, oi, tris.reshape(-1, 9), rays[pick], t_max=tmax[pick], any_hit=True)
    assert np.array_equal(u32(ha.cpu().numpy()[pick]), u32(oha))
    assert np.array_equal(sta.cpu().numpy().view(np.uint32)[pick], osta)


def test_hit_t_error_against_fp64():
    """States the error of the kernel's hit t against Möller-Trumbore in
    float64 on the same triangle (incoherent 300k scene, 200k rays): the
    single-precision test of the reference, evaluated without contraction,
    stays within a few ulps of the exact value except on grazing hits."""
    tris = scene("incoherent_300k")
    rays, _ = scenes.incoherent_rays(200_000, seed=31)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    h, _ = m.intersect(to_cuda(rays))
    h = h.cpu().numpy()
    prim = np.ascontiguousarray(h[:, 3]).view(np.int32)
    ok = prim >= 0
    assert ok.sum() > 10_000
    t = tris[prim[ok]].astype(np.float64)
    r = rays[ok].astype(np.float64)
    e1, e2 = t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]
    q = np.cross(r[:, :3] - t[:, 0], e1)
    t64 = np.einsum("ij,ij->i", e2, q) / np.einsum("ij,ij->i", e1, np.cross(r[:, 3:], e2))
    rel = np.abs(h[ok, 0] - t64) / np.abs(t64)
    print(f"hit t vs FP64: median {np.median(rel):.3g}, p99 {np.quantile(rel, 0.99):.3g}, max {rel.max():.3g}")
    assert np.median(rel) < 2e-7
    assert np.quantile(rel, 0.99) < 2e-6
    assert rel.max() < 1e-4


@pytest.mark.parametrize("name", SCENES)
@pytest.mark.parametrize("kind", ["locb", "sah"])
def test_compact_nodes_same_nearest_hit(name, kind):
    """Default closest hit (64-byte compact quad nodes) against the oracle's
    traversal of the exact nodes, and against the exact-node GPU path."""
    tris = scene(name)
    g = gpu_build(tris, kind)
    m = rb.Mbvh.construct(g)
    rays, _ = rays_for(name, count=65536)
    hits = m.intersect(to_cuda(rays))[0].cpu().numpy()
    exact = m.intersect(to_cuda(rays), exact_nodes=True)[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    assert_same_nearest(hits, exact, tris, rays)
    if kind == "locb":
        on, oi = oracle_build(tris, "locb")
        oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays, stats=False)
        assert_same_nearest(hits, oh, tris, rays)
    assert (rb.hit_prims(hits) >= 0).sum() > 0


@pytest.mark.parametrize("name", ["incoherent_20k", "sphere"])
@pytest.mark.parametrize("kind", ["locb", "sah"])
def test_compact_nodes_rays_from_inside_the_scene(name, kind):
    """Rays that start inside the scene: the compact walk skips slot boxes
    that lie behind the origin, which the reference's test keeps. Origins
    uniform in the scene box with uniform directions, and secondary rays
    leaving the primary hit points 1e-4 off the surface in random
    directions (some back into the surface), against the exact-node walk and
    the oracle."""
    tris = scene(name)
    g = gpu_build(tris, kind)
    m = rb.Mbvh.construct(g)
    rng = np.random.default_rng(21)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    n = 32768
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    inside = np.concatenate([o, d / np.linalg.norm(d, axis=1, keepdims=True)], 1).astype(np.float32)
    prim_rays, _ = rays_for(name, count=n)
    ph = m.intersect(to_cuda(prim_rays))[0].cpu().numpy()
    hit = rb.hit_prims(ph) >= 0
    p = prim_rays[hit, :3].astype(np.float64) + prim_rays[hit, 3:] * ph[hit, :1]
    tri = tris[rb.hit_prims(ph)[hit]].astype(np.float64)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm *= -np.sign(np.einsum("ij,ij->i", nrm, prim_rays[hit, 3:]))[:, None]
    sd = rng.normal(size=p.shape)
    sd /= np.linalg.norm(sd, axis=1, keepdims=True)
    second = np.concatenate([p + 1e-4 * nrm, sd], 1).astype(np.float32)
    rays = np.concatenate([inside, second])
    hits = m.intersect(to_cuda(rays))[0].cpu().numpy()
    exact = m.intersect(to_cuda(rays), exact_nodes=True)[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    assert_same_nearest(hits, exact, tris, rays)
    on, oi = oracle_build(tris, kind)
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays, stats=False)
    assert_same_nearest(hits, oh, tris, rays)
    assert (rb.hit_prims(hits) >= 0).sum() > len(rays) // 20


def test_handed_on_pass_with_far_triangles_and_inside_origins():
    """A binned-SAH tree (its rays that hit escaped triangles are handed to
    the exact walk, which skips subtrees by their triangle boxes) where some
    triangles lie far beyond the compact range: their subtree boxes are the
    infinite box and must never be skipped. Rays start inside the scene box
    (the skip applies to them) or far outside it (it does not). Handed-on
    rays get the exact walk's hits bit for bit; all rays the oracle's
    nearest hit."""
    tris = scene("incoherent_20k").copy()
    far = np.random.default_rng(6).choice(len(tris), 50, replace=False)
    tris[far] *= np.float32(1e19)
    g = gpu_build(tris, "sah")
    m = rb.Mbvh.construct(g)
    rng = np.random.default_rng(23)
    n = 65536
    o = rng.uniform(0.0, 1.0, size=(n, 3))
    o[:256] = rng.uniform(-1e3, 1e3, size=(256, 3))  # beyond the compact range: exact walk, no skip
    d = rng.normal(size=(n, 3))
    rays = np.concatenate([o, d / np.linalg.norm(d, axis=1, keepdims=True)], 1).astype(np.float32)
    d_rays = to_cuda(rays)
    hits, ws = m.intersect(d_rays, walk_stats=True)
    hits, ws = hits.cpu().numpy(), ws.cpu().numpy()
    exact = m.intersect(d_rays, exact_nodes=True)[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    handed = ws[:, 2] != 0
    assert handed.sum() >= 256
    assert np.array_equal(u32(hits[handed]), u32(exact[handed]))
    assert_same_nearest(hits, exact, tris, rays)
    on, oi = oracle_build(tris, "sah")
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays, stats=False)
    assert_same_nearest(hits, oh, tris, rays)
    assert (rb.hit_prims(hits) >= 0).sum() > n // 20


def test_compact_nodes_out_of_range_values():
    """Triangles far outside the quantisable range put their quad nodes on
    the exact path; rays with huge origins trace the exact nodes entirely.
    Results equal the exact-node traversal."""
    tris = scene("incoherent_20k").copy()
    far = np.random.default_rng(5).choice(len(tris), 50, replace=False)
    tris[far] *= np.float32(1e19)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    rays, _ = rays_for("incoherent_20k", count=65536)
    rays = rays.copy()
    rays[:100, :3] = np.float32(2e18)  # beyond the compact path's range
    rays[:100, 3:] = -rays[:100, :3] / np.linalg.norm(rays[:100, :3], axis=1, keepdims=True)
    hits = m.intersect(to_cuda(rays))[0].cpu().numpy()
    exact = m.intersect(to_cuda(rays), exact_nodes=True)[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    assert_same_nearest(hits, exact, tris, rays)
    on, oi = oracle_build(tris, "locb")
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays, stats=False)
    assert_same_nearest(hits, oh, tris, rays)


def _decode_axis(lo, e, word):
    step = np.float64(2.0) ** (int(e) - 127)
    return np.array([np.float64(lo) + ((int(word) >> (8 * i)) & 0xff) * step for i in range(4)])


@pytest.mark.parametrize("name", ["teapot", "incoherent_20k"])
def test_traversal_tree_boxes_contain_and_cover(name):
    """The closest-hit traversal tree: each compact slot box contains its
    exact box, each exact slot box contains its subtree, and every
    primitive slot is in exactly one leaf."""
    tris = scene(name)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    ex, cp = m.traversal_tree()
    assert len(ex) > 0 and len(ex) == len(cp)
    exi = ex.view(np.int32)
    seen = np.zeros(len(tris), np.int32)
    for k in range(len(ex)):
        lo = cp[k, 0:3].view(np.float32)
        exps = int(cp[k, 3])
        assert exps >> 24 == 0
        for ax, (wl, wh) in enumerate(((cp[k, 4], cp[k, 5]), (cp[k, 6], cp[k, 7]), (cp[k, 8], cp[k, 9]))):
            e = (exps >> (8 * ax)) & 0xff
            dl, dh = _decode_axis(lo[ax], e, wl), _decode_axis(lo[ax], e, wh)
            assert (dl <= ex[k, 8 * ax:8 * ax + 4].astype(np.float64)).all()
            assert (dh >= ex[k, 8 * ax + 4:8 * ax + 8].astype(np.float64)).all()
        for i in range(4):
            ch, cnt = exi[k, 24 + i], exi[k, 28 + i]
            if cnt >= 0:
                seen[ch:ch + cnt] += 1
            elif ch >= 0:
                # child node's slots lie inside this slot's box
                for ax in range(3):
                    assert ex[ch, 8 * ax:8 * ax + 4].min() >= ex[k, 8 * ax + i]
                    assert ex[ch, 8 * ax + 4:8 * ax + 8].max() <= ex[k, 8 * ax + 4 + i]
    assert (seen == 1).all()


def _covering_nodes(nodes, idx, tris):
    """The BVH2 with every box replaced by its triangles' vertex box grown
    by 1e-4 (boxes that contain their subtrees, as Bvh::refit from the
    triangles gives leaves), for the true nearest hits."""
    ni, nf = nodes.view(np.int32), nodes.view(np.float32)
    cnt, lf = ni[:, 3], ni[:, 7]
    vmin, vmax = tris.min(axis=1), tris.max(axis=1)
    lo = np.full((len(nodes), 3), np.inf, np.float32)
    hi = np.full((len(nodes), 3), -np.inf, np.float32)
    order, k = [0], 0
    while k < len(order):
        x = order[k]
        k += 1
        if cnt[x] < 0 and lf[x] >= 0:
            order += [lf[x], lf[x] + 1]
    for x in reversed(order):
        if cnt[x] >= 0:
            ids = idx[lf[x]:lf[x] + cnt[x]]
            lo[x], hi[x] = vmin[ids].min(0), vmax[ids].max(0)
        else:
            lo[x] = np.minimum(lo[lf[x]], lo[lf[x] + 1])
            hi[x] = np.maximum(hi[lf[x]], hi[lf[x] + 1])
    out = nodes.copy()
    of = out.view(np.float32)
    of[:, 0:3], of[:, 4:7] = lo - np.float32(1e-4), hi + np.float32(1e-4)
    return out


def _escaped(m):
    """Escape flags of an Mbvh's leaf-ordered triangle records (the flags
    word of each 64-byte record, 1 = escaped)."""
    view = _ffi.RTGpuView()
    assert m._lib.rtbvh_gpu_view(m.handle.id, 1, ctypes.byref(view)) == 0
    recs = rb.device_copy(view.leaf_triangles, (view.index_count, 16))
    return recs.view(np.uint32)[:, 7] != 0


def _escaped_reference(nodes, idx, tris):
    """The escape flags restated: a triangle is escaped when its vertex box
    grown by 1e-4 does not lie inside every slot box the reference's Mbvh
    tests on the way to its leaf (src/mbvh_node.rs:297-411: the boxes of the
    BVH2 nodes at even depth >= 2 on the way down; a leaf at depth 1 sits in
    a slot with the root's box)."""
    ni, nf = nodes.view(np.int32), nodes.view(np.float32)
    cnt, lf = ni[:, 3], ni[:, 7]
    big = np.float32(3e38)
    out = np.zeros(len(idx), bool)
    stack = [(0, 0, np.full(3, -big, np.float32), np.full(3, big, np.float32))]
    e = np.float32(1e-4)
    while stack:
        x, d, lo, hi = stack.pop()
        if d % 2 == 0 and d >= 2:
            lo, hi = np.maximum(lo, nf[x, 0:3]), np.minimum(hi, nf[x, 4:7])
        if cnt[x] >= 0 and d <= 1:
            lo, hi = np.maximum(lo, nf[0, 0:3]), np.minimum(hi, nf[0, 4:7])
        if cnt[x] >= 0:
            ids = idx[lf[x]:lf[x] + cnt[x]]
            t = tris[ids]
            inside = (lo <= t.min(axis=1) - e).all(axis=1) & (hi >= t.max(axis=1) + e).all(axis=1)
            out[lf[x]:lf[x] + cnt[x]] = ~inside
        elif lf[x] >= 0:
            stack += [(lf[x], d + 1, lo, hi), (lf[x] + 1, d + 1, lo, hi)]
    return out


def test_gated_sah_tree_reproduces_the_reference_walk():
    """A binned-SAH tree's boxes can miss primitives (the reference sizes a
    left child's box from bins [0, best_splits[axis].count),
    src/builders/binned_sah.rs:236-256), so the reference's walk misses
    some hits. Its traversal tree (boxes from the triangles) flags the
    triangles outside those boxes (escaped); the default walk must give the
    reference's nearest hit on every ray of the full 1024 x 1024 camera,
    including the rays whose reference hit is not the true nearest one; the
    escape flags equal their restatement."""
    tris = scenes.sphere()
    rays = scenes.camera_rays(1024, 1024)
    g = gpu_build(tris, "sah")
    m = rb.Mbvh.construct(g)
    ex, cp = m.traversal_tree()
    assert len(ex) > 0
    esc = _escaped(m)
    assert esc.any()
    assert np.array_equal(esc, _escaped_reference(g.nodes(), g.indices(), tris))
    d_rays = to_cuda(rays)
    hits = m.intersect(d_rays)[0].cpu().numpy()
    exact = m.intersect(d_rays, exact_nodes=True)[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    nodes, idx = g.nodes(), g.indices()
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(nodes), idx, tris.reshape(-1, 9), rays, stats=False)
    assert np.array_equal(u32(exact), u32(oh))
    true_h, _, _ = oracle.trace("mbvh", oracle.mbvh(_covering_nodes(nodes, idx, tris)), idx, tris.reshape(-1, 9),
                                rays, stats=False)
    quirk = u32(oh[:, 0]) != u32(true_h[:, 0])
    assert quirk.sum() > 100, "the scene should hold rays the reference's boxes make miss"
    assert np.array_equal(u32(hits[quirk, 0]), u32(oh[quirk, 0]))
    assert_same_nearest(hits, oh, tris, rays, max_tie_frac=1e-3)


@pytest.mark.parametrize("name,kind", [("sphere", "sah"), ("incoherent_20k", "sah"), ("teapot", "sah")])
def test_gated_tree_boxes_contain_their_triangles(name, kind):
    """Every slot box of a gated traversal tree contains the triangles below
    it, and every primitive slot is in exactly one leaf."""
    tris = scene(name)
    g = gpu_build(tris, kind)
    m = rb.Mbvh.construct(g)
    ex, cp = m.traversal_tree()
    assert len(ex) > 0
    idx = g.indices()
    vmin, vmax = tris.min(axis=1), tris.max(axis=1)
    exi = ex.view(np.int32)
    seen = np.zeros(len(tris), np.int32)
    for k in range(len(ex)):
        for i in range(4):
            ch, cnt = exi[k, 24 + i], exi[k, 28 + i]
            lo = np.array([ex[k, 8 * ax + i] for ax in range(3)])
            hi = np.array([ex[k, 8 * ax + 4 + i] for ax in range(3)])
            if cnt >= 0:
                seen[ch:ch + cnt] += 1
                if cnt:
                    ids = idx[ch:ch + cnt]
                    assert (lo <= vmin[ids].min(0)).all() and (hi >= vmax[ids].max(0)).all()
            elif ch >= 0:
                for ax in range(3):
                    assert ex[ch, 8 * ax:8 * ax + 4].min() >= lo[ax]
                    assert ex[ch, 8 * ax + 4:8 * ax + 8].max() <= hi[ax]
    assert (seen == 1).all()


def test_moved_triangles_keep_the_reference_hits():
    """Triangles attached after the build that leave their boxes: the
    reference's walk over the unchanged boxes misses some of their hits;
    the default walk (traversal tree rebuilt from the attached triangles,
    escaped triangles flagged) gives the reference's nearest hit."""
    tris = scene("incoherent_20k")
    moved = tris + np.random.default_rng(58).normal(scale=2e-3, size=tris.shape).astype(np.float32)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    assert not _escaped(m).any()
    m.attach_triangles(to_cuda(moved))
    esc = _escaped(m)
    assert esc.any()
    on, oi = oracle_build(tris, "locb")
    assert np.array_equal(esc, _escaped_reference(on, oi, moved))
    rays, _ = rays_for("incoherent_20k", count=65536)
    hits = m.intersect(to_cuda(rays))[0].cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, moved.reshape(-1, 9), rays, stats=False)
    true_h, _, _ = oracle.trace("mbvh", oracle.mbvh(_covering_nodes(on, oi, moved)), oi, moved.reshape(-1, 9), rays,
                                stats=False)
    assert (u32(oh[:, 0]) != u32(true_h[:, 0])).sum() > 0
    assert_same_nearest(hits, oh, moved, rays)
    # the same triangles again: nothing escapes
    m.attach_triangles(to_cuda(tris))
    assert not _escaped(m).any()



@pytest.mark.parametrize("name,kind", [("incoherent_300k", "locb"), ("sphere", "sah")])
def test_walk_stats_of_the_compact_walk(name, kind):
    """RTBVH_TRACE_WALK_STATS: the default walk's own per-ray counts. The
    hits equal the call without the flag bit for bit; every ray taken by the
    compact walk visits the root, every reported hit of that walk comes from
    a triangle test; rays handed on to the exact walk are flagged (none on an
    LOCB tree, some on the binned-SAH sphere whose boxes miss triangles); on
    the LOCB tree the walk visits fewer nodes and tests fewer triangles than
    the reference's iterator (RTBVH_TRACE_STATS) on average."""
    tris = scene(name)
    m = rb.Mbvh.construct(gpu_build(tris, kind))
    rays = scenes.camera_rays(1024, 1024) if name == "sphere" else rays_for(name, count=262144)[0]
    d_rays = to_cuda(rays)
    plain = m.intersect(d_rays)[0].cpu().numpy()
    hits, ws = m.intersect(d_rays, walk_stats=True)
    hits, ws = hits.cpu().numpy(), ws.cpu().numpy()
    assert m.status() == rb.ResultCode.Ok
    assert np.array_equal(u32(hits), u32(plain))
    own = ws[:, 2] == 0
    assert set(np.unique(ws[:, 2]).tolist()) <= {0, 1}
    assert (ws[own, 0] >= 1).all()
    hit = rb.hit_prims(hits) >= 0
    assert (ws[own & hit, 1] >= 1).all()
    handed = int((~own).sum())
    if kind == "locb":
        assert handed == 0
    else:
        assert 0 < handed < len(rays) // 50
        # the pass over handed-on rays skips subtrees without a hit but keeps
        # the reference's order: its hits are the exact walk's, bit for bit
        exact = m.intersect(d_rays, exact_nodes=True)[0].cpu().numpy()
        assert np.array_equal(u32(hits[~own]), u32(exact[~own]))
    if kind == "locb":
        # the traversal tree of an LOCB build is the tighter one
        _, ref = m.intersect(d_rays, stats=True)
        ref = ref.cpu().numpy()
        assert ws[:, 0].mean() < ref[:, 0].mean()
        assert ws[:, 1].mean() < ref[:, 1].mean()
    lib = _ffi.load()
    st = torch.empty((len(rays), 3), dtype=torch.int32, device="cuda")
    h = torch.empty((len(rays), 4), dtype=torch.float32, device="cuda")
    for extra in (_ffi.TRACE_STATS, _ffi.TRACE_ANY_HIT, _ffi.TRACE_EXACT_NODES, _ffi.TRACE_REORDER):
        rc = lib.rtbvh_gpu_intersect_mbvh(m.handle, ctypes.c_void_p(d_rays.data_ptr()), None, len(rays),
                                          ctypes.c_void_p(h.data_ptr()), _ffi.TRACE_WALK_STATS | extra,
                                          ctypes.c_void_p(st.data_ptr()), None)
        assert rc == rb.ResultCode.InvalidArgument
    rc = lib.rtbvh_gpu_intersect_mbvh(m.handle, ctypes.c_void_p(d_rays.data_ptr()), None, len(rays),
                                      ctypes.c_void_p(h.data_ptr()), _ffi.TRACE_WALK_STATS, None, None)
    assert rc == rb.ResultCode.Error
