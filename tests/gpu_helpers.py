"""Shared helpers of the GPU parity tests."""
import numpy as np
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import scenes


def u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


def to_cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_build(tris, kind, ppl=None):
    b = rb.Builder(primitives=rb.Triangles(to_cuda(tris)), primitives_per_leaf=ppl)
    return b.construct_locally_ordered_clustered() if kind == "locb" else b.construct_binned_sah()


def oracle_build(tris, kind, ppl=1):
    a, c = oracle.triangle_prep(tris)
    return oracle.build(a, c, kind, prims_per_leaf=ppl)


def canonical(nodes, idx):
    """BVH2 renumbered in DFS pre-order (children of a node allocated as an
    adjacent pair, left subtree first) with leaves as sorted primitive sets,
    so trees from differently ordered builders compare equal."""
    ints = np.ascontiguousarray(nodes).view(np.int32)
    out_boxes, out_kind = [], []
    if len(nodes) == 0:
        return out_boxes, out_kind
    order = []
    stack = [0]
    while stack:
        c = stack.pop()
        order.append(c)
        if ints[c, 3] < 0 and ints[c, 7] >= 0:
            lf = ints[c, 7]
            stack += [lf + 1, lf]
    for c in order:
        box = tuple(u32(nodes[c, [0, 1, 2, 4, 5, 6]]).tolist())
        if ints[c, 3] >= 0:
            lf, cnt = ints[c, 7], ints[c, 3]
            kind = ("leaf", tuple(sorted(idx[lf:lf + cnt].tolist())))
        else:
            kind = ("node",)
        out_boxes.append(box)
        out_kind.append(kind)
    return out_boxes, out_kind


def scene(name):
    if name == "teapot":
        import os
        return np.load(os.path.join(os.path.dirname(__file__), "golden", "teapot_tris.npy"))
    if name == "sphere":
        return scenes.sphere()
    if name.startswith("incoherent_"):
        n = int(name.split("_")[1].replace("k", "000"))
        return scenes.incoherent(n, seed=7)
    raise KeyError(name)


def rays_for(name, count=16384):
    if name in ("teapot",):
        return scenes.camera_rays(128, 128, eye=(0.0, 1.5, 8.0), fov_deg=40.0), None
    if name == "sphere":
        return scenes.camera_rays(128, 128), None
    r, tmax = scenes.incoherent_rays(count, seed=8)
    return r, tmax


def _mt_t(tri, ray):
    """The reference's triangle test in float32 (no contraction) for one
    triangle and ray; t or None."""
    f32 = np.float32
    v0, v1, v2 = (tri[k].astype(f32) for k in range(3))
    o, d = ray[:3].astype(f32), ray[3:].astype(f32)
    e1, e2 = v1 - v0, v2 - v0
    h = np.array([d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0], d[0] * e2[1] - e2[0] * d[1]], f32)
    det = f32(f32(e1[0] * h[0]) + f32(e1[1] * h[1])) + f32(e1[2] * h[2])
    if -1e-5 < det < 1e-5:
        return None
    f = f32(1.0) / det
    s = o - v0
    q = np.array([s[1] * e1[2] - e1[1] * s[2], s[2] * e1[0] - e1[2] * s[0], s[0] * e1[1] - e1[0] * s[1]], f32)
    return f * (f32(f32(e2[0] * q[0]) + f32(e2[1] * q[1])) + f32(e2[2] * q[2]))


def assert_same_nearest(hits, ref, tris, rays, max_tie_frac=2e-3):
    """Same nearest hit as `ref`: t bit-identical on every ray; the triangle
    (and its u, v) identical unless the reported one is hit at exactly the
    same t (a tie, which the compact-node traversal may resolve differently)."""
    bad_t = np.nonzero(u32(hits[:, 0]) != u32(ref[:, 0]))[0]
    assert len(bad_t) == 0, f"t differs on {len(bad_t)} rays, e.g. {[(int(r), hits[r].tolist(), ref[r].tolist()) for r in bad_t[:4]]}"
    p, q = rb.hit_prims(hits), rb.hit_prims(ref)
    diff = np.nonzero(p != q)[0]
    for r in diff:
        assert p[r] >= 0 and q[r] >= 0
        t = _mt_t(tris[p[r]], rays[r])
        assert t is not None and np.float32(t).view(np.uint32) == hits[r, 0].view(np.uint32), f"ray {r}: not a tie"
    same = p == q
    assert np.array_equal(u32(hits[same]), u32(ref[same]))
    assert len(diff) <= max(1, int(max_tie_frac * len(hits))), f"{len(diff)} ties"
