"""GPU spatial-split SAH build (src/builders/spatial_sah.rs) against the
oracle's restatement: node arrays and the full prim_indices vector bit for
bit, for the reference as written and with every correction, then
traversal, refit and the on-disk format over the built trees."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import _ffi, scenes
from gpu_helpers import scene, to_cuda, u32

pytestmark = pytest.mark.gpu

FIXES = [0, oracle.SPATIAL_FIX_ALL]


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


def _quad():
    v = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    return v[np.array([[0, 1, 2], [0, 2, 3]])]


def _grid(k=24):
    # axis-aligned unit squares on a plane: many equal centres (sort ties)
    out = []
    for i in range(k):
        for j in range(k):
            a, b, c, d = (i, j, 0), (i + 1, j, 0), (i + 1, j + 1, 0), (i, j + 1, 0)
            out += [[a, b, c], [a, c, d]]
    return np.asarray(out, np.float32) / k


SCENES = {
    "quad": _quad,
    "teapot": lambda: scene("teapot"),
    "sphere_1600": lambda: scenes.sphere(40, 20),
    "incoherent_5k": lambda: scenes.incoherent(5000, seed=1),
    "slivers_2k": lambda: scenes.slivers(2000, seed=5, length=0.5),
    "grid": _grid,
}


def gpu_spatial(tris, fixes, ppl=None):
    b = rb.Builder(primitives=rb.Triangles(to_cuda(tris)), primitives_per_leaf=ppl)
    return b.construct_spatial_sah(fixes=fixes)


@pytest.mark.parametrize("fixes", FIXES)
@pytest.mark.parametrize("name", list(SCENES))
def test_build_matches_oracle(name, fixes):
    tris = SCENES[name]()
    g = gpu_spatial(tris, fixes)
    on, oi = oracle.build_spatial(tris, fixes=fixes)
    assert g.build_type() == rb.BuildType.Spatial
    assert np.array_equal(u32(g.nodes()), u32(on)), f"{name}: nodes differ"
    assert np.array_equal(g.indices(), oi), f"{name}: prim_indices differ"
    assert g.validate(len(tris)) == oracle.validate(on, oi, len(tris))


@pytest.mark.parametrize("ppl", [2, 4, 16])
def test_leaf_sizes_match_oracle(ppl):
    tris = scenes.slivers(1500, seed=6, length=0.3)
    for fixes in FIXES:
        g = gpu_spatial(tris, fixes, ppl)
        on, oi = oracle.build_spatial(tris, prims_per_leaf=ppl, fixes=fixes)
        assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi)


def test_each_correction_alone_matches_oracle():
    tris = scenes.slivers(1200, seed=7, length=0.6)
    for bit in (1, 2, 4, 8, 16):
        g = gpu_spatial(tris, bit)
        on, oi = oracle.build_spatial(tris, fixes=bit)
        assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi), bit


def test_large_tasks_above_the_shared_memory_tile():
    # root and upper tasks sort through the merge passes (more than 2048 refs)
    tris = scenes.incoherent(40000, seed=9)
    for fixes in FIXES:
        g = gpu_spatial(tris, fixes)
        on, oi = oracle.build_spatial(tris, fixes=fixes)
        assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi)


def test_ffi_entry_with_strided_host_inputs():
    # create_spatial_Bvh (rtbvh_ffi/src/lib.rs:345-389): vec4 vertices
    # (vertex_stride 16, triangle_stride 48), vec4 centres, aabbs from the
    # wrapper's Primitive::aabb
    tris = scenes.slivers(800, seed=8, length=0.4)
    n = len(tris)
    v4 = np.zeros((n, 3, 4), np.float32)
    v4[:, :, :3] = tris
    a, c = oracle.triangle_prep(tris)
    c4 = np.zeros((n, 4), np.float32)
    c4[:, :3] = c
    lib = _ffi.load()
    out = _ffi.RTBvh()
    fp = ctypes.POINTER(ctypes.c_float)
    rc = lib.create_spatial_Bvh(None, n, c4.ctypes.data_as(fp), 16, v4.ctypes.data_as(fp), 16, 48, 1,
                                ctypes.byref(out))
    assert rc == _ffi.ResultCode.Ok
    bvh = rb.Bvh(out, rb.BuildType.Spatial, n)
    on, oi = oracle.build_spatial(tris, aabbs=a, centers=c, fixes=0)
    assert np.array_equal(u32(bvh.nodes()), u32(on)) and np.array_equal(bvh.indices(), oi)
    # the same with explicit boxes
    out2 = _ffi.RTBvh()
    rc = lib.create_spatial_Bvh(a.ctypes.data_as(ctypes.POINTER(_ffi.RTAabb)), n, c4.ctypes.data_as(fp), 16,
                                v4.ctypes.data_as(fp), 16, 48, 1, ctypes.byref(out2))
    assert rc == _ffi.ResultCode.Ok
    assert np.array_equal(u32(rb.Bvh(out2, rb.BuildType.Spatial, n).nodes()), u32(on))


@pytest.mark.parametrize("fixes", FIXES)
def test_traversal_over_spatial_trees(fixes):
    tris = scenes.slivers(2000, seed=5, length=0.5)
    rays, tmax = scenes.incoherent_rays(8192, seed=10)
    g = gpu_spatial(tris, fixes)
    m = rb.Mbvh.construct(g)
    on, oi = oracle.build_spatial(tris, fixes=fixes)
    om = oracle.mbvh(on)
    dr = to_cuda(rays)
    for structure, nodes, s in (("bvh", on, g), ("mbvh", om, m)):
        h, _ = s.intersect(dr)
        oh, _, bad = oracle.trace(structure, nodes, oi, tris, rays)
        assert not bad
        assert np.array_equal(u32(h.cpu().numpy()), u32(oh)), structure
    hx, _ = m.intersect(dr, exact_nodes=True)
    oh, _, _ = oracle.trace("mbvh", om, oi, tris, rays)
    assert np.array_equal(u32(hx.cpu().numpy()), u32(oh))
    ha, _ = m.intersect(dr, t_max=to_cuda(tmax), any_hit=True)
    oa, _, _ = oracle.trace("mbvh", om, oi, tris, rays, t_max=tmax, any_hit=True)
    assert np.array_equal(u32(ha.cpu().numpy())[:, 3] != 0xFFFFFFFF, u32(oa)[:, 3] != 0xFFFFFFFF)


def test_corrected_tree_finds_the_nearest_hit():
    # every primitive referenced: closest hits equal a brute-force search
    tris = scenes.slivers(600, seed=11, length=0.5)
    rays, _ = scenes.incoherent_rays(2048, seed=12)
    g = gpu_spatial(tris, oracle.SPATIAL_FIX_ALL)
    h, _ = rb.Mbvh.construct(g).intersect(to_cuda(rays))
    # brute force with the same triangle test: a one-leaf tree over all primitives
    root = oracle.union_of_list(scenes.triangle_aabbs(tris)).copy()
    root.view(np.int32)[3] = len(tris)
    root.view(np.int32)[7] = 0
    hb, _, _ = oracle.trace("bvh", root[None, :], np.arange(len(tris), dtype=np.uint32), tris, rays)
    hit = u32(hb)[:, 3] != 0xFFFFFFFF
    assert hit.sum() > 100
    got = h.cpu().numpy()
    assert np.array_equal(u32(got)[:, 3] != 0xFFFFFFFF, hit)
    assert np.array_equal(u32(got[hit, 0]), u32(hb[hit, 0]))


@pytest.mark.parametrize("fixes", FIXES)
def test_refit_and_bytes(fixes, tmp_path):
    tris = scenes.slivers(1500, seed=13, length=0.4)
    g = gpu_spatial(tris, fixes)
    on, oi = oracle.build_spatial(tris, fixes=fixes)
    moved = tris + np.random.default_rng(14).normal(scale=1e-3, size=tris.shape).astype(np.float32)
    g.refit(triangles=to_cuda(moved))
    torch.cuda.synchronize()
    # boxes as the reference's Bvh::refit computes them; the topology words,
    # which the reference overwrites with 0, are kept
    want = oracle.refit(on, oi, scenes.triangle_aabbs(moved))
    cols = [0, 1, 2, 4, 5, 6]
    assert np.array_equal(u32(g.nodes())[:, cols], u32(want)[:, cols])
    assert np.array_equal(u32(g.nodes())[:, [3, 7]], u32(on)[:, [3, 7]])
    data = g.to_bytes()
    assert data[-4:] == (3).to_bytes(4, "little")
    g2 = rb.Bvh.from_bytes(data)
    assert g2.build_type() == rb.BuildType.Spatial
    assert np.array_equal(u32(g2.nodes()), u32(g.nodes())) and np.array_equal(g2.indices(), g.indices())
    g2.attach_triangles(to_cuda(moved))
    rays, _ = scenes.incoherent_rays(4096, seed=15)
    dr = to_cuda(rays)
    h1, _ = g.intersect(dr)
    h2, _ = g2.intersect(dr)
    assert torch.equal(h1.view(torch.int32), h2.view(torch.int32))


def test_panicking_inputs_return_error():
    # inputs on which the reference's equal-count fallback panics (the
    # oracle raises): the as-written build returns Error, the corrected
    # builds match the oracle
    for seed, n in ((32, 40), (87, 40), (261, 120)):
        tris = scenes.plane_slivers(n, seed)
        with pytest.raises(rb.RtbvhError) as e:
            gpu_spatial(tris, 0)
        assert e.value.code == rb.ResultCode.Error
        for fixes in (oracle.SPATIAL_FIX_FALLBACK, oracle.SPATIAL_FIX_ALL):
            g = gpu_spatial(tris, fixes)
            on, oi = oracle.build_spatial(tris, fixes=fixes)
            assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi)
    # seeds of the same family where the reference does not panic
    for seed in (1, 2, 3):
        tris = scenes.plane_slivers(40, seed)
        g = gpu_spatial(tris, 0)
        on, oi = oracle.build_spatial(tris, fixes=0)
        assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi)


def _degenerate(kind):
    t = scenes.incoherent(50, seed=3)
    if kind == "identical_64":
        return np.tile(t[:1], (64, 1, 1))
    if kind == "collinear":
        return np.stack([t[:, 0], t[:, 1], t[:, 0] + 2 * (t[:, 1] - t[:, 0])], 1).astype(np.float32)
    if kind == "single":
        return t[:1].copy()
    return np.repeat(t[:, :1], 3, axis=1).astype(np.float32)  # all three vertices equal


@pytest.mark.parametrize("fixes", FIXES)
@pytest.mark.parametrize("kind", ["identical_64", "collinear", "single", "points"])
def test_degenerate_inputs(kind, fixes):
    tris = _degenerate(kind)
    try:
        on, oi = oracle.build_spatial(tris, fixes=fixes)
    except oracle.OracleError:
        with pytest.raises(rb.RtbvhError) as e:
            gpu_spatial(tris, fixes)
        assert e.value.code == rb.ResultCode.Error
        return
    g = gpu_spatial(tris, fixes)
    assert np.array_equal(u32(g.nodes()), u32(on)) and np.array_equal(g.indices(), oi)


def test_argument_errors():
    lib = _ffi.load()
    out = _ffi.RTBvh()
    v = to_cuda(scenes.slivers(10, seed=1))
    p = ctypes.c_void_p(v.data_ptr())
    assert lib.rtbvh_gpu_create_spatial_bvh(p, 0, None, None, 0, 1, 0, 0, None, ctypes.byref(out)) == \
        _ffi.ResultCode.NoPrimitives
    assert lib.rtbvh_gpu_create_spatial_bvh(p, 10, None, None, 0, 1, 64, 0, None, ctypes.byref(out)) == \
        _ffi.ResultCode.InvalidArgument
    assert lib.rtbvh_gpu_create_spatial_bvh(None, 10, None, None, 0, 1, 0, 0, None, ctypes.byref(out)) == \
        _ffi.ResultCode.Error
    with pytest.raises(TypeError):
        rb.Builder(primitives=rb.Points(np.zeros((4, 3), np.float32))).construct_spatial_sah()
