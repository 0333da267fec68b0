"""Differentiable closest-hit ray cast (torch.autograd harness over the C ABI).

Forward: the MBVH traversal with the fused triangle test returns t, u, v and
the hit primitive id per ray (rtbvh_gpu_intersect_mbvh). Backward: the
hand-written kernel behind rtbvh_gpu_intersect_backward maps the upstream
(dL/dt, dL/du, dL/dv) to dL/dvertices (summed per triangle in a fixed order,
so repeated runs give identical bits) and dL/d(ray origin, direction). The
BVH walk is an index selection: hit ids are stored, not re-traversed.
"""
import ctypes

import torch

from . import _ffi
from .api import Mbvh, _ptr, _stream, check


class _RayCast(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertices, rays, mbvh):
        hits, _ = mbvh.intersect(rays.detach())
        ctx.save_for_backward(vertices.detach(), rays.detach(), hits)
        prim = hits[:, 3].contiguous().view(torch.int32)
        ctx.mark_non_differentiable(prim)
        return hits[:, 0].clone(), hits[:, 1].clone(), hits[:, 2].clone(), prim

    @staticmethod
    def backward(ctx, gt, gu, gv, _gprim):
        vertices, rays, hits = ctx.saved_tensors
        R = rays.shape[0]
        z = torch.zeros(R, dtype=torch.float32, device=rays.device)
        g = torch.stack([gt if gt is not None else z, gu if gu is not None else z, gv if gv is not None else z],
                        dim=1).contiguous()
        gvert = torch.empty_like(vertices)
        grays = torch.empty_like(rays) if ctx.needs_input_grad[1] else None
        intersect_backward(vertices, rays, hits, g, gvert, grays)
        return gvert if ctx.needs_input_grad[0] else None, grays, None


def intersect_backward(vertices, rays, hits, grad_tuv, grad_vertices, grad_rays=None, stream=None):
    """Raw backward call: fills grad_vertices (n, 3, 3) and grad_rays (R, 6)."""
    lib = _ffi.load()
    n = vertices.reshape(-1, 9).shape[0]
    R = rays.reshape(-1, 6).shape[0]
    check(lib.rtbvh_gpu_intersect_backward(_ptr(vertices), n, _ptr(rays), _ptr(hits), _ptr(grad_tuv), R,
                                           _ptr(grad_vertices), _ptr(grad_rays) if grad_rays is not None else None,
                                           _stream(stream)), "intersect_backward")


def ray_cast(mbvh: Mbvh, vertices: torch.Tensor, rays: torch.Tensor):
    """Closest hits of `rays` (R, 6) against the triangles `vertices` (n, 3, 3)
    that `mbvh` was built over. Returns t, u, v (differentiable w.r.t.
    vertices and rays) and the int32 primitive id (-1: miss)."""
    return _RayCast.apply(vertices, rays, mbvh)


def step_and_refit(bvh, mbvh, vertices, grad_vertices, lr=1e-3, stream=None):
    """One vertex step v <- v - lr * dL/dv, then the GPU refit of the BVH
    (Bvh::refit boxes) and the re-collapse of the MBVH over the new vertices."""
    with torch.no_grad():
        vertices.sub_(lr * grad_vertices)
    bvh.refit(triangles=vertices, mbvh=mbvh, stream=stream)
    return vertices
