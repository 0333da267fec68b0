"""The oracle against the reference's own known-answer tests (CPU only)."""
import numpy as np
import pytest

import oracle
from rtbvh_gb300 import scenes


def test_morton_split_known_answers(golden):
    # src/morton.rs:109-115
    for v, want in golden["known"]["morton_split"]["cases"]:
        assert oracle.morton_split(v) == want


def spread3(v):
    v = (v | (v << 16)) & 0x030000FF
    v = (v | (v << 8)) & 0x0300F00F
    v = (v | (v << 4)) & 0x030C30C3
    v = (v | (v << 2)) & 0x09249249
    return v


def test_morton_split_is_the_three_way_spread():
    # the device kernel uses the closed form; the reference's loop must agree on the whole 10-bit grid
    for v in range(1024):
        assert oracle.morton_split(v) == spread3(v)


def test_prefix_sum(golden):
    k = golden["known"]["prefix_sum"]
    total, out = oracle.prefix_sum(k["input"])
    assert list(out) == k["output"] and total == k["output"][-1]
    total0, _ = oracle.prefix_sum([])
    assert total0 == 0  # count == 0 returns first[0]


def test_abi_sizes(golden):
    k = golden["known"]["abi_sizes"]
    L = oracle.lib()
    assert L.ror_abi_sizes(0) == k["RTAabb"]
    assert L.ror_abi_sizes(1) == k["RTBvhNode"]
    assert L.ror_abi_sizes(2) == k["RTMbvhNode"]


def quad_tris(golden):
    k = golden["known"]["two_triangle_quad"]
    v = np.asarray(k["vertices"], np.float32)
    return v[np.asarray(k["triangles"])]


@pytest.mark.parametrize("bt", ["sah", "locb"])
def test_two_triangle_quad_builds(golden, bt):
    # src/lib.rs:66-124
    tris = quad_tris(golden)
    nodes, idx = oracle.build(scenes.triangle_aabbs(tris), scenes.triangle_centers(tris), bt)
    assert len(nodes) >= 1 and sorted(idx) == [0, 1]


def test_no_primitives():
    # src/lib.rs:28-38
    with pytest.raises(oracle.OracleError):
        oracle.build(np.zeros((0, 8), np.float32), np.zeros((0, 3), np.float32), "sah")


def test_single_degenerate_triangle():
    # src/lib.rs:40-49: one all-zero triangle builds
    tris = np.zeros((1, 3, 3), np.float32)
    nodes, idx = oracle.build(scenes.triangle_aabbs(tris), scenes.triangle_centers(tris), "sah")
    assert len(nodes) == 1 and list(idx) == [0]


def test_five_triangles_all_leaf_sizes(golden):
    # src/lib.rs:246-311: binned SAH with leaf sizes 1..10 then Mbvh::from
    tris = np.asarray(golden["known"]["five_triangles"]["triangles"], np.float32)
    a, c = scenes.triangle_aabbs(tris), scenes.triangle_centers(tris)
    for ppl in golden["known"]["five_triangles"]["leaf_sizes"]:
        nodes, idx = oracle.build(a, c, "sah", prims_per_leaf=ppl)
        m = oracle.mbvh(nodes)
        assert len(m) >= 1
        assert oracle.validate(nodes, idx, 5)


@pytest.mark.parametrize("bt", ["sah", "locb"])
def test_teapot_structure(golden, bt):
    # src/builders/binned_sah.rs:407-458, src/builders/locb.rs:336-388
    tris = golden["teapot"]
    n = len(tris)
    assert n == golden["known"]["teapot_structure"]["prim_count"]
    nodes, idx = oracle.build(scenes.triangle_aabbs(tris), scenes.triangle_centers(tris), bt)
    assert n <= len(nodes) <= 2 * n
    root = nodes[0]
    assert (root[0:3] <= root[4:7]).all()
    assert oracle.validate(nodes, idx, n)
    v = tris.reshape(-1, 3)
    assert ((v > root[0:3]) & (v < root[4:7])).all()


def test_quad_hit_at_t_one(golden):
    # rtbvh_ffi/src/lib.rs:945-1019: ray from the origin along +z hits the quad at z = 1
    k = golden["known"]["quad_hit"]
    v = np.asarray(k["vertices"], np.float32).reshape(2, 3, 3)
    a = scenes.triangle_aabbs(v)
    centers = ((a[:, 0:3] + a[:, 4:7]) * np.float32(0.5)).astype(np.float32)
    nodes, idx = oracle.build(a, centers, "sah")
    m = oracle.mbvh(nodes)
    ray = np.asarray([k["origin"] + k["direction"]], np.float32)
    for structure, nd in (("bvh", nodes), ("mbvh", m)):
        hits, _, bad = oracle.trace(structure, nd, idx, v.reshape(-1, 9), ray, t_max=[k["t_in"]],
                                    t_min_tri=k["callback_t_min"])
        assert bad == 0
        assert abs(hits[0, 0] - k["t_expected"]) < np.finfo(np.float32).eps


def test_mbvh_preorder_numbering_matches_dfs_counts(golden):
    # structural property used by the GPU collapse: quad nodes are the interior
    # BVH2 nodes at even depth, numbered in pre-order
    tris = golden["teapot"]
    nodes, idx = oracle.build(scenes.triangle_aabbs(tris), scenes.triangle_centers(tris), "locb")
    m = oracle.mbvh(nodes)
    ints = nodes.view(np.int32)
    even_interior = 0
    stack = [(0, 0)]
    while stack:
        c, d = stack.pop()
        if ints[c, 3] < 0:
            if d % 2 == 0:
                even_interior += 1
            lf = ints[c, 7]
            stack += [(lf, d + 1), (lf + 1, d + 1)]
    assert len(m) == even_interior


def test_refit_overwrites_topology_like_the_reference(golden):
    # src/bvh.rs:176-205 assigns a fresh Aabb (extras 0) to every node
    tris = golden["teapot"][:200]
    a, c = scenes.triangle_aabbs(tris), scenes.triangle_centers(tris)
    nodes, idx = oracle.build(a, c, "locb")
    r = oracle.refit(nodes, idx, a)
    assert (r.view(np.int32)[:, [3, 7]] == 0).all()
    assert (r[0, 0:3] <= nodes[0, 0:3]).all()


def test_traversal_oracle_matches_brute_force():
    tris = scenes.incoherent(3000, seed=5)
    rays, _ = scenes.incoherent_rays(2000, seed=6)
    a, c = scenes.triangle_aabbs(tris), scenes.triangle_centers(tris)
    nodes, idx = oracle.build(a, c, "locb")
    m = oracle.mbvh(nodes)
    hits, st, bad = oracle.trace("mbvh", m, idx, tris.reshape(-1, 9), rays)
    assert bad == 0
    # brute force with the same triangle test: a one-leaf "BVH" over all prims
    root = oracle.union_of_list(a).copy()
    rv = root.view(np.int32)
    rv[3] = len(tris)
    rv[7] = 0
    bh, _, _ = oracle.trace("bvh", root[None, :], np.arange(len(tris), dtype=np.uint32), tris.reshape(-1, 9), rays)
    np.testing.assert_array_equal(hits[:, 0], bh[:, 0])
    both = oracle.hit_prims(hits) >= 0
    assert both.sum() > 20


@pytest.mark.parametrize("structure,builder", [("mbvh", "locb"), ("bvh", "sah"), ("mbvh", "sah"), ("bvh", "locb")])
def test_packet_oracle_matches_brute_force(structure, builder):
    # packets (src/iter_indices.rs:110-414) must find, per lane, the nearest
    # triangle the packet test (src/builders/spatial_sah.rs:165-244) accepts
    tris = scenes.incoherent(2000, seed=15)
    rays, _ = scenes.incoherent_rays(1600, seed=16)
    a, c = scenes.triangle_aabbs(tris), scenes.triangle_centers(tris)
    nodes, idx = oracle.build(a, c, builder)
    st_nodes = oracle.mbvh(nodes) if structure == "mbvh" else nodes
    hits, st, bad = oracle.trace_packets(structure, st_nodes, idx, tris.reshape(-1, 9), rays)
    assert bad == 0
    root = oracle.union_of_list(a).copy()
    rv = root.view(np.int32)
    rv[3] = len(tris)
    rv[7] = 0
    bh, _, _ = oracle.trace_packets("bvh", root[None, :], np.arange(len(tris), dtype=np.uint32),
                                    tris.reshape(-1, 9), rays)
    np.testing.assert_array_equal(hits[:, 0], bh[:, 0])
    assert (oracle.hit_prims(hits) >= 0).sum() > 20
    # every packet walks at least the root
    assert (st[:, 0] >= 1).all() if structure == "mbvh" else True


def test_packet_oracle_nan_lane_skips_bvh_packet():
    # BvhPacketIndexIterator::new (src/iter_indices.rs:122-143): any NaN lane -> no traversal
    tris = scenes.incoherent(500, seed=17)
    rays, _ = scenes.incoherent_rays(8, seed=18)
    rays[1, 4] = np.nan
    a, c = scenes.triangle_aabbs(tris), scenes.triangle_centers(tris)
    nodes, idx = oracle.build(a, c, "locb")
    hits, st, _ = oracle.trace_packets("bvh", nodes, idx, tris.reshape(-1, 9), rays)
    assert (oracle.hit_prims(hits[:4]) == -1).all() and (st[0] == 0).all()
