"""GPU candidate lists (the device form of the reference's callback
iteration, rtbvh_ffi/src/lib.rs:551-581 / 700-731) against the oracle's
restatement of MbvhIndexIterator / BvhIndexIterator with a callback that
leaves t unchanged: the same primitive ids in the same order, the same
counts."""
import numpy as np
import pytest
import torch

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import scenes
from gpu_helpers import gpu_build, oracle_build, rays_for, scene, to_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _device(lib):
    torch.cuda.set_device(0)
    yield
    torch.cuda.synchronize()


def _gpu(structure, rays, t_max=None, max_per_ray=512):
    c, n = structure.candidates(to_cuda(rays), t_max=None if t_max is None else to_cuda(t_max),
                                max_per_ray=max_per_ray)
    torch.cuda.synchronize()
    assert structure.status() == rb.ResultCode.Ok
    return c.cpu().numpy().view(np.uint32), n.cpu().numpy().view(np.uint32)


def _same_lists(gc, gn, oc, on, m):
    assert np.array_equal(gn, on), "counts differ"
    for r in np.nonzero(gn)[0]:
        k = min(int(gn[r]), m)
        assert np.array_equal(gc[r, :k], oc[r, :k]), f"ray {r}: lists differ"


@pytest.mark.parametrize("name", ["teapot", "sphere", "incoherent_20k"])
@pytest.mark.parametrize("kind", ["mbvh", "bvh"])
def test_candidates_locb_match_oracle(name, kind):
    tris = scene(name)
    g = gpu_build(tris, "locb")
    rays, _ = rays_for(name, count=4096)
    on, oi = oracle_build(tris, "locb")
    s, nodes = (rb.Mbvh.construct(g), oracle.mbvh(on)) if kind == "mbvh" else (g, on)
    gc, gn = _gpu(s, rays)
    oc, onn = oracle.candidates(kind, nodes, oi, rays, max_per_ray=512)
    _same_lists(gc, gn, oc, onn, 512)
    assert gn.sum() > 0


def test_candidates_sah_mbvh_and_t_bound():
    tris = scenes.incoherent(20000, seed=41)
    rays, tmax = scenes.incoherent_rays(4096, seed=42)
    g = gpu_build(tris, "sah")
    m = rb.Mbvh.construct(g)
    on, oi = oracle_build(tris, "sah")
    om = oracle.mbvh(on)
    for t in (None, tmax):
        gc, gn = _gpu(m, rays, t_max=t)
        oc, onn = oracle.candidates("mbvh", om, oi, rays, t_max=t, max_per_ray=512)
        _same_lists(gc, gn, oc, onn, 512)
    # a shorter t culls: never more candidates than without a bound
    _, n_all = _gpu(m, rays)
    _, n_cut = _gpu(m, rays, t_max=tmax)
    assert (n_cut <= n_all).all() and n_cut.sum() < n_all.sum()


def test_candidates_sah_bvh_same_sets():
    # breadth-first numbering and stable leaf order: the same primitives per
    # ray, possibly in another order inside a leaf
    tris = scenes.incoherent(20000, seed=43)
    rays, _ = scenes.incoherent_rays(2048, seed=44)
    g = gpu_build(tris, "sah")
    gc, gn = _gpu(g, rays)
    on, oi = oracle_build(tris, "sah")
    oc, onn = oracle.candidates("bvh", on, oi, rays, max_per_ray=512)
    assert np.array_equal(gn, onn)
    for r in np.nonzero(gn)[0]:
        k = int(gn[r])
        assert sorted(gc[r, :k].tolist()) == sorted(oc[r, :k].tolist())


def test_candidates_truncation_and_count_only():
    tris = scene("incoherent_20k")
    m = rb.Mbvh.construct(gpu_build(tris, "locb"))
    rays, _ = rays_for("incoherent_20k", count=4096)
    full_c, full_n = _gpu(m, rays, max_per_ray=512)
    cut_c, cut_n = _gpu(m, rays, max_per_ray=2)
    assert np.array_equal(full_n, cut_n) and (full_n > 2).any()
    for r in range(len(rays)):
        k = min(int(full_n[r]), 2)
        assert np.array_equal(cut_c[r, :k], full_c[r, :k])
    c0, n0 = m.candidates(to_cuda(rays), max_per_ray=0)
    assert c0 is None and np.array_equal(n0.cpu().numpy().view(np.uint32), full_n)


def test_candidates_drive_a_custom_primitive():
    # spheres: the library knows only their boxes; the caller's own test over
    # the candidate lists finds the same nearest sphere as a brute-force test
    rng = np.random.default_rng(45)
    n = 3000
    centers = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    radii = rng.uniform(0.002, 0.02, size=n).astype(np.float32)
    aabbs = np.zeros((n, 8), np.float32)
    aabbs[:, 0:3] = centers - radii[:, None]
    aabbs[:, 4:7] = centers + radii[:, None]
    bvh = rb.Builder(aabbs=aabbs, primitives=rb.Points(centers)).construct_locally_ordered_clustered()
    m = rb.Mbvh.construct(bvh)
    rays, _ = scenes.incoherent_rays(8192, seed=46)
    cands, counts = m.candidates(to_cuda(rays), max_per_ray=256)
    counts = counts.long()
    assert int(counts.max()) <= 256
    dc, dr = to_cuda(centers).double(), to_cuda(radii).double()
    r = to_cuda(rays).double()
    o, d = r[:, None, :3], r[:, None, 3:]

    def sphere_t(idx):
        oc = o - dc[idx]
        b = (oc * d).sum(-1)
        cc = (oc * oc).sum(-1) - dr[idx] ** 2
        dd = (d * d).sum(-1)
        disc = b * b - dd * cc
        t = (-b - torch.sqrt(disc.clamp(min=0))) / dd
        return torch.where((disc >= 0) & (t > 1e-4), t, torch.full_like(t, float("inf")))

    # entries past counts[r] are not written by the library: replace them
    # before they are used as indices
    valid = torch.arange(cands.shape[1], device="cuda")[None, :] < counts[:, None]
    cl = torch.where(valid, cands.long(), torch.zeros_like(cands, dtype=torch.long))
    assert int(cl.min()) >= 0 and int(cl.max()) < n
    t_c = torch.where(valid, sphere_t(cl), torch.full_like(cl, float("inf"), dtype=torch.float64))
    best_c, arg_c = t_c.min(1)
    id_c = torch.gather(cl, 1, arg_c[:, None])[:, 0]
    t_b = sphere_t(torch.arange(n, device="cuda")[None, :].expand(len(rays), n))
    best_b, id_b = t_b.min(1)
    hit = torch.isfinite(best_b)
    assert int(hit.sum()) > 50
    assert torch.equal(torch.isfinite(best_c), hit)
    assert torch.equal(id_c[hit], id_b[hit])
