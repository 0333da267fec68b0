"""Differentiable closest-hit ray cast on the full differentiable workload
(200,000-triangle sphere, 2048 x 2048 camera): the hand-written backward
kernel against an FP64 analytic gradient and FP64 central finite
differences (h = 1e-4) on 4,096 rays sampled from the camera; determinism of
the per-triangle sums; the autograd harness; one vertex step followed by the
GPU refit."""
import os

import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import diff, scenes
from gpu_helpers import assert_same_nearest, to_cuda, u32

pytestmark = pytest.mark.gpu


def mt64(v0, v1, v2, o, d):
    """Möller-Trumbore (t, u, v) in float64, no acceptance tests (the hit
    primitive is fixed)."""
    e1, e2 = v1 - v0, v2 - v0
    h = np.cross(d, e2)
    a = np.einsum("...i,...i", e1, h)
    f = 1.0 / a
    s = o - v0
    u = f * np.einsum("...i,...i", s, h)
    q = np.cross(s, e1)
    v = f * np.einsum("...i,...i", d, q)
    t = f * np.einsum("...i,...i", e2, q)
    return t, u, v


def analytic64(tri, ray, g):
    """Per-ray FP64 gradients: (dv (R,3,3), dray (R,6))."""
    v0, v1, v2 = tri[:, 0], tri[:, 1], tri[:, 2]
    o, d = ray[:, :3], ray[:, 3:]
    t, u, v = mt64(v0, v1, v2, o, d)
    e1, e2 = v1 - v0, v2 - v0
    h = np.cross(d, e2)
    f = 1.0 / np.einsum("...i,...i", e1, h)
    lam = f[:, None] * (g[:, 0:1] * np.cross(e1, e2) + g[:, 1:2] * h + g[:, 2:3] * np.cross(e1, d))
    dv = np.stack([-(1 - u - v)[:, None] * lam, -u[:, None] * lam, -v[:, None] * lam], axis=1)
    dray = np.concatenate([lam, t[:, None] * lam], axis=1)
    return dv, dray


@pytest.fixture(scope="module")
def setup(lib):
    torch.cuda.set_device(0)
    tris = scenes.sphere_fast(500, 200, radius=1.0, noise=0.05, seed=5)  # 200,000 triangles
    rays = scenes.camera_rays(2048, 2048, eye=(0.0, 0.0, 3.0), fov_deg=45.0)  # 4,194,304 rays
    bvh = rb.Builder(primitives=rb.Triangles(to_cuda(tris))).construct_binned_sah()
    mbvh = rb.Mbvh.construct(bvh)
    d_rays = to_cuda(rays)
    hits, _ = mbvh.intersect(d_rays)
    g = np.random.default_rng(7).normal(size=(len(rays), 3)).astype(np.float32)
    return tris, rays, bvh, mbvh, d_rays, hits, g


def run_backward(tris, d_rays, hits, g):
    verts = to_cuda(tris)
    gv = torch.empty_like(verts)
    gr = torch.empty_like(d_rays)
    diff.intersect_backward(verts, d_rays, hits, to_cuda(g), gv, gr)
    torch.cuda.synchronize()
    return gv.cpu().numpy(), gr.cpu().numpy()


def test_backward_matches_fp64_analytic(setup):
    tris, rays, bvh, mbvh, d_rays, hits, g = setup
    gv, gr = run_backward(tris, d_rays, hits, g)
    h = hits.cpu().numpy()
    prim = rb.hit_prims(h)
    hit = prim >= 0
    assert hit.sum() > 50000
    t64 = tris.astype(np.float64)
    dv, dray = analytic64(t64[prim[hit]], rays[hit].astype(np.float64), g[hit].astype(np.float64))
    ref_v = np.zeros(t64.shape, np.float64)
    np.add.at(ref_v, prim[hit], dv)
    rel_v = np.linalg.norm(gv - ref_v) / np.linalg.norm(ref_v)
    rel_r = np.linalg.norm(gr[hit] - dray) / np.linalg.norm(dray)
    assert rel_v <= 1e-4, rel_v
    assert rel_r <= 1e-4, rel_r
    assert (gr[~hit] == 0).all()
    never = np.ones(len(tris), bool)
    never[prim[hit]] = False
    assert (gv[never] == 0).all()


def test_backward_matches_fp64_finite_differences(setup):
    """Central differences with h = 1e-4 on 4,096 sampled rays. The triangles
    are ~0.01 across, so a 1e-4 step is a 1 % perturbation and the FD value
    itself carries O(h^2) truncation error; the GPU gradient is held to the
    Richardson-extrapolated FD (h, h/2: O(h^4)) at 1e-4, and must be as close
    to the plain h = 1e-4 FD as the exact FP64 gradient is."""
    tris, rays, bvh, mbvh, d_rays, hits, g = setup
    h = hits.cpu().numpy()
    prim = rb.hit_prims(h)
    hit_idx = np.nonzero(prim >= 0)[0]
    pick = np.random.default_rng(8).choice(hit_idx, 4096, replace=False)
    g_s = np.zeros_like(g)
    g_s[pick] = g[pick]
    gv, gr = run_backward(tris, d_rays, hits, g_s)
    t64, r64, g64 = tris.astype(np.float64), rays.astype(np.float64), g_s.astype(np.float64)
    p = prim[pick]
    touched = np.unique(p)

    def loss(tri, ray, gg):
        t, u, v = mt64(tri[:, 0], tri[:, 1], tri[:, 2], ray[:, :3], ray[:, 3:])
        return gg[:, 0] * t + gg[:, 1] * u + gg[:, 2] * v

    def fd(step):
        fd_r = np.zeros((len(pick), 6))
        for k in range(6):
            rp, rm = r64[pick].copy(), r64[pick].copy()
            rp[:, k] += step
            rm[:, k] -= step
            fd_r[:, k] = (loss(t64[p], rp, g64[pick]) - loss(t64[p], rm, g64[pick])) / (2 * step)
        fd_v = np.zeros((len(tris), 3, 3))
        for a in range(3):
            for k in range(3):
                tp, tm = t64[p].copy(), t64[p].copy()
                tp[:, a, k] += step
                tm[:, a, k] -= step
                contrib = (loss(tp, r64[pick], g64[pick]) - loss(tm, r64[pick], g64[pick])) / (2 * step)
                np.add.at(fd_v[:, a, k], p, contrib)
        return fd_v[touched], fd_r

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    fv1, fr1 = fd(1e-4)
    fv2, fr2 = fd(5e-5)
    fv_rich, fr_rich = (4 * fv2 - fv1) / 3, (4 * fr2 - fr1) / 3
    assert rel(gv[touched], fv_rich) <= 1e-4, rel(gv[touched], fv_rich)
    assert rel(gr[pick], fr_rich) <= 1e-4, rel(gr[pick], fr_rich)
    # against the plain h = 1e-4 differences: no worse than the exact gradient
    dv, dray = analytic64(t64[p], r64[pick], g64[pick])
    exact_v = np.zeros((len(tris), 3, 3))
    np.add.at(exact_v, p, dv)
    assert rel(gv[touched], fv1) <= rel(exact_v[touched], fv1) + 1e-4
    assert rel(gr[pick], fr1) <= rel(dray, fr1) + 1e-4


def test_backward_is_deterministic(setup):
    tris, rays, bvh, mbvh, d_rays, hits, g = setup
    a = run_backward(tris, d_rays, hits, g)
    b = run_backward(tris, d_rays, hits, g)
    assert np.array_equal(u32(a[0]), u32(b[0])) and np.array_equal(u32(a[1]), u32(b[1]))


def test_autograd_harness_matches_raw_call(setup):
    tris, rays, bvh, mbvh, d_rays, hits, g = setup
    verts = to_cuda(tris).requires_grad_(True)
    r = d_rays.clone().requires_grad_(True)
    t, u, v, prim = diff.ray_cast(mbvh, verts, r)
    assert torch.equal(prim.cpu(), torch.from_numpy(rb.hit_prims(hits.cpu().numpy()).copy()))
    gg = to_cuda(g)
    loss = (t * gg[:, 0] * (prim >= 0)).sum() + (u * gg[:, 1]).sum() + (v * gg[:, 2]).sum()
    loss.backward()
    g_eff = g.copy()
    g_eff[rb.hit_prims(hits.cpu().numpy()) < 0, 0] = 0
    gv, gr = run_backward(tris, d_rays, hits, g_eff)
    assert np.array_equal(u32(verts.grad.cpu().numpy()), u32(gv))
    assert np.array_equal(u32(r.grad.cpu().numpy()), u32(gr))


def test_vertex_step_then_gpu_refit(setup):
    tris, rays, bvh0, mbvh0, d_rays, hits0, g = setup
    bvh = rb.Builder(primitives=rb.Triangles(to_cuda(tris))).construct_binned_sah()
    mbvh = rb.Mbvh.construct(bvh)
    verts = to_cuda(tris)
    hits, _ = mbvh.intersect(d_rays)
    gv = torch.empty_like(verts)
    diff.intersect_backward(verts, d_rays, hits, to_cuda(g), gv, None)
    diff.step_and_refit(bvh, mbvh, verts, gv, lr=1e-3)
    torch.cuda.synchronize()
    moved = verts.cpu().numpy()
    assert not np.array_equal(moved, tris)
    nodes = bvh.nodes()
    a2, _ = oracle.triangle_prep(moved)
    ref = oracle.refit(nodes, bvh.indices(), a2)
    cols = [0, 1, 2, 4, 5, 6]
    assert np.array_equal(u32(nodes)[:, cols], u32(ref)[:, cols])
    h2, _ = mbvh.intersect(d_rays)
    # every 16th ray against the oracle (the stepped triangles overlap a lot,
    # which makes the CPU walk slow)
    sub = slice(0, None, 16)
    oh, _, _ = oracle.trace("mbvh", oracle.mbvh(nodes), bvh.indices(), moved.reshape(-1, 9), rays[sub],
                            threads=os.cpu_count() or 1, stats=False)
    # the refitted tree is nested, so closest hit runs on the traversal tree:
    # the same nearest hit as the reference's traversal, ties aside
    assert_same_nearest(h2.cpu().numpy()[sub], oh, moved, rays[sub])
