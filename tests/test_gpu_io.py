"""On-disk format (the crate's serde derives in bincode 1 layout) and the
Mbvh refit: bytes against an independent encoder of that layout built from
the oracle's trees, round trips, rejection of damaged input."""
import struct

import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import scenes
from gpu_helpers import gpu_build, oracle_build, to_cuda, u32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


def _vec(records, item_bytes):
    a = np.ascontiguousarray(records)
    return struct.pack("<Q", len(a)) + a.tobytes()[: len(a) * item_bytes]


def encode_bvh(nodes, idx, build_type):
    # Bvh {nodes: Vec<BvhNode>, prim_indices: Vec<u32>, build_type: BuildType}
    return (_vec(nodes.astype(np.float32), 32) + _vec(idx.astype(np.uint32), 4) +
            struct.pack("<I", build_type))


def encode_mbvh(nodes, mnodes, idx):
    # Mbvh {nodes: Vec<BvhNode>, m_nodes: Vec<MbvhNode>, prim_indices: Vec<u32>}
    return _vec(nodes.astype(np.float32), 32) + _vec(mnodes.astype(np.float32), 128) + _vec(idx.astype(np.uint32), 4)


def test_bytes_match_the_serde_layout_of_the_oracle_tree():
    tris = scenes.incoherent(5000, seed=51)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    on, oi = oracle_build(tris, "locb")
    assert g.to_bytes() == encode_bvh(on, oi, 1)
    assert m.to_bytes() == encode_mbvh(on, oracle.mbvh(on), oi)
    s = gpu_build(tris, "sah")
    assert s.to_bytes()[-4:] == struct.pack("<I", 2)


@pytest.mark.parametrize("kind", ["locb", "sah"])
def test_round_trip_traces_the_same(kind, tmp_path):
    tris = scenes.incoherent(20000, seed=52)
    rays, _ = scenes.incoherent_rays(8192, seed=53)
    g = gpu_build(tris, kind)
    m = rb.Mbvh.construct(g)
    path = tmp_path / "m.bin"
    m.save(str(path))
    g2 = rb.Bvh.from_bytes(g.to_bytes())
    m2 = rb.Mbvh.load(str(path))
    assert np.array_equal(u32(g2.nodes()), u32(g.nodes())) and np.array_equal(g2.indices(), g.indices())
    assert np.array_equal(u32(m2.quad_nodes()), u32(m.quad_nodes())) and np.array_equal(m2.indices(), m.indices())
    assert g2.build_type() == g.build_type()
    g2.attach_triangles(to_cuda(tris))
    m2.attach_triangles(to_cuda(tris))
    dr = to_cuda(rays)
    for a, b in ((g, g2), (m, m2)):
        h1, _ = a.intersect(dr)
        h2, _ = b.intersect(dr)
        assert torch.equal(h1.view(torch.int32), h2.view(torch.int32))
    h1, _ = m.intersect(dr, exact_nodes=True)
    h2, _ = m2.intersect(dr, exact_nodes=True)
    assert torch.equal(h1.view(torch.int32), h2.view(torch.int32))
    assert m2.to_bytes() == m.to_bytes()


def _rejects(fn, data, code):
    with pytest.raises(rb.RtbvhError) as e:
        fn(data)
    assert e.value.code == code


def test_damaged_input_is_rejected():
    tris = scenes.incoherent(3000, seed=54)
    g = gpu_build(tris, "locb")
    m = rb.Mbvh.construct(g)
    b, mb = g.to_bytes(), m.to_bytes()
    IA = rb.ResultCode.InvalidArgument
    _rejects(rb.Bvh.from_bytes, b[:-1], IA)                       # truncated
    _rejects(rb.Bvh.from_bytes, b + b"\0", IA)                    # trailing bytes
    # root's child pair past the node array
    _rejects(rb.Bvh.from_bytes, b[:8 + 28] + struct.pack("<i", 2 ** 31 - 1) + b[8 + 32:], IA)
    bad_type = b[:-4] + struct.pack("<I", 7)
    _rejects(rb.Bvh.from_bytes, bad_type, IA)
    n = struct.unpack("<Q", b[:8])[0]
    idx_off = 8 + 32 * n + 8
    bad_idx = b[:idx_off] + struct.pack("<I", 10 ** 6) + b[idx_off + 4:]
    _rejects(rb.Bvh.from_bytes, bad_idx, IA)                      # index out of range
    nodes = np.frombuffer(b[8:8 + 32 * n], np.float32).reshape(-1, 8).copy()
    leaf = int(np.nonzero(nodes.view(np.int32)[:, 3] >= 0)[0][0])
    nodes.view(np.int32)[leaf, 7] = 3000                           # leaf range past the indices
    _rejects(rb.Bvh.from_bytes, b[:8] + nodes.tobytes() + b[8 + 32 * n:], IA)
    _rejects(rb.Bvh.from_bytes, struct.pack("<QQI", 0, 0, 1), rb.ResultCode.NoPrimitives)
    # an Mbvh whose quad nodes are not the collapse of its Bvh nodes
    q_off = 8 + 32 * n + 8
    q = np.frombuffer(mb[q_off:q_off + 128], np.float32).copy()
    q[0] += 1.0
    _rejects(rb.Mbvh.from_bytes, mb[:q_off] + q.tobytes() + mb[q_off + 128:], IA)
    _rejects(rb.Mbvh.from_bytes, mb[:-3], IA)


def test_mbvh_refit_equals_bvh_refit_and_recollapse():
    tris = scenes.incoherent(20000, seed=55)
    rays, _ = scenes.incoherent_rays(8192, seed=56)
    moved = tris + np.random.default_rng(57).normal(scale=2e-3, size=tris.shape).astype(np.float32)
    ga, gb = gpu_build(tris, "locb"), gpu_build(tris, "locb")
    ma, mb = rb.Mbvh.construct(ga), rb.Mbvh.construct(gb)
    before = gb.nodes()
    ga.refit(triangles=to_cuda(moved), mbvh=ma)   # Bvh refit + re-collapse
    mb.refit(triangles=to_cuda(moved))            # the Mbvh alone
    torch.cuda.synchronize()
    assert np.array_equal(u32(mb.quad_nodes()), u32(ma.quad_nodes()))
    assert np.array_equal(u32(gb.nodes()), u32(before)), "the source Bvh must stay as it was"
    dr = to_cuda(rays)
    ha, _ = ma.intersect(dr)
    hb, _ = mb.intersect(dr)
    assert torch.equal(ha.view(torch.int32), hb.view(torch.int32))
    # boxes from aabbs give the same result
    mc = rb.Mbvh.construct(gpu_build(tris, "locb"))
    mc.refit(new_aabbs=scenes.triangle_aabbs(moved))
    assert np.array_equal(u32(mc.quad_nodes()), u32(ma.quad_nodes()))
