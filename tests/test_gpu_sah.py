"""GPU parity: binned SAH build against the oracle.

The reference numbers nodes in the order its worker threads allocate them
(src/builders/mod.rs:59-76), so trees are compared in a canonical form: DFS
pre-order, node boxes bit for bit, leaves as primitive sets (the reference's
Lomuto partition and this build's stable partition may order a leaf's
primitives differently). The MBVH does not depend on BVH2 numbering and is
compared as-is, bit for bit."""
import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import scenes
from gpu_helpers import canonical, gpu_build, oracle_build, rays_for, scene, to_cuda, u32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


def check_tree(tris, ppl=1, full=True):
    g = gpu_build(tris, "sah", ppl=ppl)
    on, oi = oracle_build(tris, "sah", ppl=ppl)
    gn, gi = g.nodes(), g.indices()
    assert len(gn) == len(on), "node counts differ"
    assert g.validate(len(tris))
    if full:
        assert canonical(gn, gi) == canonical(on, oi)
    m = rb.Mbvh.construct(g)
    assert np.array_equal(u32(m.quad_nodes()), u32(oracle.mbvh(on)))
    return g, m, on, oi


@pytest.mark.parametrize("name", ["teapot", "sphere", "incoherent_20k", "incoherent_300k"])
def test_sah_canonical_tree_bit_exact(name):
    check_tree(scene(name))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 33, 1023, 1024, 1025, 2048, 2049, 4100, 70000])
def test_sah_sizes(n):
    check_tree(scenes.incoherent(n, seed=300 + n))


@pytest.mark.parametrize("ppl", [2, 4, 7, 16])
def test_sah_primitives_per_leaf(ppl):
    check_tree(scenes.incoherent(50000, seed=17), ppl=ppl)


def test_sah_five_triangles_every_leaf_size(golden):
    # src/lib.rs:246-311
    tris = np.asarray(golden["known"]["five_triangles"]["triangles"], np.float32)
    for ppl in golden["known"]["five_triangles"]["leaf_sizes"]:
        check_tree(tris, ppl=ppl)


def test_sah_identical_primitives_make_one_leaf():
    t = np.tile(np.asarray([[[0.1, 0.2, 0.3], [0.4, 0.2, 0.3], [0.1, 0.6, 0.3]]], np.float32), (5000, 1, 1))
    g, _, on, _ = check_tree(t)
    assert len(on) == 1 and g.nodes().view(np.int32)[0, 3] == 5000


def test_sah_clustered_spheres():
    check_tree(scenes.clustered(200_000, n_spheres=16, seed=9))


@pytest.mark.parametrize("name", ["teapot", "sphere", "incoherent_300k"])
def test_sah_trace_matches_oracle(name):
    tris = scene(name)
    g, m, on, oi = check_tree(tris, full=False)
    rays, _ = rays_for(name)
    hits, st = m.intersect(to_cuda(rays), stats=True)
    hits, st = hits.cpu().numpy(), st.cpu().numpy().view(np.uint32)
    oh, ost, _ = oracle.trace("mbvh", oracle.mbvh(on), oi, tris.reshape(-1, 9), rays)
    # t, u, v bit for bit; the primitive id too unless two primitives of one
    # leaf tie exactly (leaf order may differ, see module docstring)
    assert np.array_equal(u32(hits[:, :3]), u32(oh[:, :3]))
    same = rb.hit_prims(hits) == oracle.hit_prims(oh)
    assert same.mean() > 0.999
    assert np.array_equal(st, ost)


def test_sah_1m_canonical():
    check_tree(scenes.incoherent(1_000_000, seed=21), full=False)


def _leaf_sets(mnodes, idx):
    """(leaf offset, count, sorted primitive ids) of every leaf slot of a
    quad-node array, as one sortable key array."""
    mi = np.ascontiguousarray(mnodes).view(np.int32)
    ch, cnt = mi[:, 24:28].ravel(), mi[:, 28:32].ravel()
    leaf = cnt >= 0
    off, c = ch[leaf].astype(np.int64), cnt[leaf].astype(np.int64)
    rid = np.repeat(np.arange(len(off)), c)
    pos = np.repeat(off, c) + (np.arange(c.sum()) - np.repeat(np.cumsum(c) - c, c))
    prims = idx[pos].astype(np.int64)
    order = np.lexsort((prims, rid))
    return off, c, prims[order]


def test_sah_above_the_cooperative_limit():
    # builds above 2^20 primitives launch the phases of each level separately
    tris = scenes.clustered(1_100_000, n_spheres=24, seed=23)
    assert len(tris) > (1 << 20)
    g, m, on, oi = check_tree(tris, full=False)
    om = oracle.mbvh(on)
    go, gc, gp = _leaf_sets(m.quad_nodes(), g.indices())
    oo, oc, op = _leaf_sets(om, oi)
    assert np.array_equal(go, oo) and np.array_equal(gc, oc) and np.array_equal(gp, op)
