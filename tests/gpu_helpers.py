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
