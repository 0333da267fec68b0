"""CPU tests of the bench line's parity block: `nearest_hit_parity` counts
t mismatches, triangle mismatches, proven ties and u/v mismatches, and its
triangle test (`_mt_t32`, the reference's SpatialTriangle::intersect in
float32) reproduces the oracle's t bit for bit."""
import numpy as np

import bench
import oracle
from rtbvh_gb300 import scenes


def _scene_with_duplicates():
    """Returns (tris, rays, r0, p0): the last triangle repeats triangle p0,
    which ray r0 hits, so r0 hits both copies at the same t."""
    tris = scenes.incoherent(2000, seed=31)
    # triangles 20 times larger (the reference's triangle test rejects
    # |det| < 1e-5, which tiny triangles often fall below)
    cen = tris.mean(1, keepdims=True)
    tris = (cen + 20.0 * (tris - cen)).astype(np.float32)
    rays, _ = scenes.incoherent_rays(20000, seed=32)
    prim = np.ascontiguousarray(_oracle_hits(tris, rays)[:, 3]).view(np.int32)
    r0 = int(np.nonzero(prim >= 0)[0][0])
    p0 = int(prim[r0])
    return np.concatenate([tris, tris[p0:p0 + 1]]), rays, r0, p0


def _oracle_hits(tris, rays):
    a, c = oracle.triangle_prep(tris)
    nodes, idx = oracle.build(a, c, "locb")
    hits, _, _ = oracle.trace("mbvh", oracle.mbvh(nodes), idx, tris.reshape(-1, 9), rays, stats=False)
    return hits


def test_mt_t32_reproduces_the_oracle_t():
    tris, rays, _, _ = _scene_with_duplicates()
    hits = _oracle_hits(tris, rays)
    prim = np.ascontiguousarray(hits[:, 3]).view(np.int32)
    hit = prim >= 0
    assert hit.sum() > 1000
    t = bench._mt_t32(tris[prim[hit]], rays[hit])
    assert np.array_equal(t.astype(np.float32).view(np.uint32), hits[hit, 0].view(np.uint32))


def test_parity_counts():
    tris, rays, r0, p0 = _scene_with_duplicates()
    copy = len(tris) - 1
    ref = _oracle_hits(tris, rays)
    prim = np.ascontiguousarray(ref[:, 3]).view(np.int32)
    assert prim[r0] in (p0, copy), "ray r0 hits one of the two copies"
    same = bench.nearest_hit_parity(ref.copy(), ref, tris, rays)
    assert same == {"rays": len(rays), "t_bit_mismatch": 0, "prim_mismatch": 0, "ties_proven": 0,
                    "uv_mismatch_same_prim": 0}
    gpu = ref.copy()
    g32 = gpu.view(np.uint32)
    hit_rows = np.nonzero(prim >= 0)[0]
    # a tie: the other copy of the duplicated triangle, same t
    g32[r0, 3] = copy if prim[r0] == p0 else p0
    # a triangle that does not give the reported t
    other = hit_rows[hit_rows > r0][0]
    g32[other, 3] = (prim[other] + 1) % len(tris)
    # a t one ulp off
    r_t = hit_rows[hit_rows > other][0]
    g32[r_t, 0] += 1
    # a u one ulp off on the same triangle
    r_u = hit_rows[hit_rows > r_t][0]
    g32[r_u, 1] += 1
    got = bench.nearest_hit_parity(gpu, ref, tris, rays)
    assert got == {"rays": len(rays), "t_bit_mismatch": 1, "prim_mismatch": 2, "ties_proven": 1,
                   "uv_mismatch_same_prim": 1}
