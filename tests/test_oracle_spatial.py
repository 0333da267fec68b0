"""The oracle's restatement of the spatial-split builder
(src/builders/spatial_sah.rs) against the reference's own tests of it, and
the defects that restatement exposes (CPU only)."""
import numpy as np
import pytest

import oracle
from rtbvh_gb300 import scenes


def _quad(golden):
    k = golden["known"]["two_triangle_quad"]
    v = np.asarray(k["vertices"], np.float32)
    return v[np.asarray(k["triangles"])]


def _referenced(nodes, idx, n):
    ints = nodes.view(np.int32)
    seen = np.zeros(n, bool)
    for c in np.nonzero(ints[:, 3] >= 0)[0]:
        seen[idx[ints[c, 7]:ints[c, 7] + ints[c, 3]]] = True
    return seen


def test_max_reference_count():
    # build (:937): n + (n as f32 * 0.75) as usize
    for n in (1, 2, 3, 4, 5, 6320, 16777217):
        assert oracle.spatial_max_refs(n) == n + int(np.float32(n) * np.float32(0.75))


def test_quad_builds(golden):
    # src/lib.rs:126-154: the two-triangle quad builds
    nodes, idx = oracle.build_spatial(_quad(golden))
    assert len(nodes) >= 1 and len(idx) == oracle.spatial_max_refs(2)
    assert oracle.validate(nodes, idx, 2)


def test_no_primitives():
    # spatial_sah.rs:1040-1045 (an empty builder gives no nodes) and
    # Builder::construct_spatial_sah's NoPrimitives (src/bvh.rs:63-65)
    with pytest.raises(oracle.OracleError):
        oracle.build_spatial(np.zeros((0, 9), np.float32))


@pytest.mark.parametrize("fixes", [0, oracle.SPATIAL_FIX_ALL])
def test_teapot(golden, fixes):
    # spatial_sah.rs:1047-1052 (node count between n and 2n) and
    # test_spatial_sah_build (:1055-1092): valid bounds, every primitive
    # referenced, every vertex strictly inside the root box
    tris = golden["teapot"]
    n = len(tris)
    nodes, idx = oracle.build_spatial(tris, fixes=fixes)
    ints = nodes.view(np.int32)
    refs = int(ints[ints[:, 3] >= 0, 3].sum())
    assert n <= len(nodes) <= 2 * refs
    if fixes == 0:  # no spatial split is chosen: one reference per primitive
        assert refs == n and len(nodes) <= 2 * n
    root = nodes[0]
    assert (root[0:3] <= root[4:7]).all()
    assert oracle.validate(nodes, idx, n)
    v = tris.reshape(-1, 3)
    assert ((v > root[0:3]) & (v < root[4:7])).all()


def test_reference_as_written_loses_primitives():
    # allocate_children (:375-424) moves the right child's references by
    # left_split_count but keeps the child on the old range: when
    # 0 < left_split_count < right count, the range holds stale copies of its
    # first references and the last ones fall outside it. Random triangles
    # show it at the first split; every correction together references all.
    tris = scenes.incoherent(5000, seed=1)
    nodes, idx = oracle.build_spatial(tris, fixes=0)
    assert not oracle.validate(nodes, idx, 5000)
    assert 4000 < _referenced(nodes, idx, 5000).sum() < 5000
    only_space = oracle.build_spatial(tris, fixes=oracle.SPATIAL_FIX_SPLIT_SPACE)
    assert oracle.validate(*only_space, 5000)
    fixed = oracle.build_spatial(tris, fixes=oracle.SPATIAL_FIX_ALL)
    assert oracle.validate(*fixed, 5000)


def test_corrected_builds_split_references():
    # with every correction the builder chooses spatial splits: more leaf
    # references than primitives, each leaf box holding its fragments
    tris = scenes.slivers(500, seed=5)
    nodes, idx = oracle.build_spatial(tris, fixes=oracle.SPATIAL_FIX_ALL)
    ints = nodes.view(np.int32)
    leaves = ints[:, 3] >= 0
    refs = int(ints[leaves, 3].sum())
    assert refs > 500
    assert oracle.validate(nodes, idx, 500)
    assert (idx[refs:] == 0).all()
    for c in np.nonzero(leaves)[0]:
        for p in idx[ints[c, 7]:ints[c, 7] + ints[c, 3]]:
            # a fragment's box lies inside its triangle's box
            tb_lo, tb_hi = tris[p].min(0), tris[p].max(0)
            assert (nodes[c, 0:3] <= tb_hi).all() and (nodes[c, 4:7] >= tb_lo).all()


def test_leaf_size_and_depth():
    tris = scenes.incoherent(2000, seed=3)
    for ppl in (1, 4, 16):
        nodes, idx = oracle.build_spatial(tris, prims_per_leaf=ppl, fixes=oracle.SPATIAL_FIX_ALL)
        assert oracle.validate(nodes, idx, 2000)
    # identical triangles cannot be separated: the median fallback splits
    # them down to single references
    same = np.tile(tris[:1], (64, 1, 1))
    nodes, idx = oracle.build_spatial(same, fixes=oracle.SPATIAL_FIX_ALL)
    assert oracle.validate(nodes, idx, 64)


def test_reference_panics_in_the_equal_count_fallback():
    # :643-658: with every reference on the left and none straddling,
    # left_end = left_count / 2 ignores the task's begin; below begin the
    # next slice panics. Thin triangles on three planes reach it; the
    # corrected builder references every primitive.
    for seed, n in ((32, 40), (87, 40), (261, 120)):
        tris = scenes.plane_slivers(n, seed)
        with pytest.raises(oracle.OracleError, match="panics"):
            oracle.build_spatial(tris, fixes=0)
        oracle.build_spatial(tris, fixes=oracle.SPATIAL_FIX_FALLBACK)  # no panic
        assert oracle.validate(*oracle.build_spatial(tris, fixes=oracle.SPATIAL_FIX_ALL), n)


@pytest.mark.parametrize("fixes", [0, oracle.SPATIAL_FIX_ALL])
def test_threaded_build_equals_the_single_thread_order(golden, fixes):
    # TaskSpawner's threading (a thread per task above the threshold, here
    # also far below the reference's 1024 to run many at once), renumbered
    # afterwards: the same nodes and indices as the single-thread build
    cases = [golden["teapot"], scenes.incoherent(20000, seed=1), scenes.slivers(3000, seed=5, length=0.5)]
    for tris in cases:
        want = oracle.build_spatial(tris, fixes=fixes)
        for threshold in (8, 64, 1024):
            for _ in range(2):
                got = oracle.build_spatial(tris, fixes=fixes, spawn_threshold=threshold)
                assert np.array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
                assert np.array_equal(got[1], want[1])
