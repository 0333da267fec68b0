"""Seeded synthetic scenes and ray sets for the benchmark workloads.

All geometry is produced in float64 with numpy's PCG64 generator and rounded
once to float32, so a scene is a pure function of its parameters and seed.
Triangles are returned as ``(n, 3, 3)`` float32 arrays (v0, v1, v2) and rays
as ``(R, 6)`` float32 arrays (origin, direction).

Workloads (sizes as used by the benchmark and the tests):

* ``sphere``      -- closed lat-long sphere, 80x40 cells x 2 = 6,400 triangles,
                     radius 1, per-grid-vertex radial noise +-5 %; pole
                     triangles are degenerate (the pole vertex is shared).
* ``camera_rays`` -- pinhole camera on +z looking at the origin, pixel centres.
* ``incoherent``  -- n triangles with centroids uniform in the unit cube and
                     vertices at centroid + unit direction x log-normal length
                     (median 0.005, sigma 0.5).
* ``incoherent_rays`` -- origins uniform on a radius-2 sphere around the cube
                     centre, directions towards uniform points in the cube;
                     any-hit t_max = 0.5 x distance to that point.
* ``clustered``   -- spheres with log-uniform radii and Gaussian-mixture centres.
"""
import math

import numpy as np


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def sphere(n_lon=80, n_lat=40, radius=1.0, noise=0.05, seed=1, center=(0.0, 0.0, 0.0)):
    rng = _rng(seed)
    # grid vertices (n_lat - 1) interior rows x n_lon plus two shared poles
    rows = n_lat - 1
    fac = rng.uniform(1.0 - noise, 1.0 + noise, size=(rows, n_lon))
    pole_fac = rng.uniform(1.0 - noise, 1.0 + noise, size=2)
    theta = np.pi * (np.arange(1, n_lat) / n_lat)  # polar angle of the interior rows
    phi = 2.0 * np.pi * (np.arange(n_lon) / n_lon)
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    sp, cp = np.sin(phi)[None, :], np.cos(phi)[None, :]
    r = radius * fac
    grid = np.stack([r * st * cp, r * st * sp, r * ct * np.ones_like(cp)], axis=-1)  # (rows, n_lon, 3)
    north = np.array([0.0, 0.0, radius * pole_fac[0]])
    south = np.array([0.0, 0.0, -radius * pole_fac[1]])
    c = np.asarray(center, dtype=np.float64)

    def vert(i, j):
        # latitude index i in [0, n_lat], longitude j (wraps)
        j = j % n_lon
        if i == 0:
            return north
        if i == n_lat:
            return south
        return grid[i - 1, j]

    tris = np.empty((n_lat * n_lon * 2, 3, 3), dtype=np.float64)
    k = 0
    for i in range(n_lat):
        for j in range(n_lon):
            a, b = vert(i, j), vert(i, j + 1)
            d, e = vert(i + 1, j), vert(i + 1, j + 1)
            tris[k] = (a, d, e)
            tris[k + 1] = (a, e, b)
            k += 2
    return (tris + c).astype(np.float32)


def sphere_fast(n_lon, n_lat, radius=1.0, noise=0.05, seed=1, center=(0.0, 0.0, 0.0)):
    """Vectorised ``sphere`` for large tessellations (same construction)."""
    rng = _rng(seed)
    rows = n_lat - 1
    fac = rng.uniform(1.0 - noise, 1.0 + noise, size=(rows, n_lon))
    pole_fac = rng.uniform(1.0 - noise, 1.0 + noise, size=2)
    theta = np.pi * (np.arange(1, n_lat) / n_lat)
    phi = 2.0 * np.pi * (np.arange(n_lon) / n_lon)
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    sp, cp = np.sin(phi)[None, :], np.cos(phi)[None, :]
    r = radius * fac
    grid = np.stack([r * st * cp, r * st * sp, r * ct * np.ones_like(cp)], axis=-1)
    allv = np.empty((n_lat + 1, n_lon, 3), dtype=np.float64)
    allv[0] = (0.0, 0.0, radius * pole_fac[0])
    allv[n_lat] = (0.0, 0.0, -radius * pole_fac[1])
    allv[1:n_lat] = grid
    i = np.arange(n_lat)[:, None]
    j = np.arange(n_lon)[None, :]
    j1 = (j + 1) % n_lon
    a = allv[i, j]
    b = allv[i, j1]
    d = allv[i + 1, j]
    e = allv[i + 1, j1]
    t0 = np.stack([a, d, e], axis=-2)
    t1 = np.stack([a, e, b], axis=-2)
    tris = np.stack([t0, t1], axis=2).reshape(-1, 3, 3)
    return (tris + np.asarray(center, dtype=np.float64)).astype(np.float32)


def camera_rays(width=1024, height=1024, eye=(0.0, 0.0, 3.0), fov_deg=45.0):
    """Pinhole camera at ``eye`` looking at the origin (towards -z), y up."""
    tan_half = math.tan(math.radians(fov_deg) * 0.5)
    aspect = width / height
    xs = ((np.arange(width) + 0.5) / width * 2.0 - 1.0) * tan_half * aspect
    ys = (1.0 - (np.arange(height) + 0.5) / height * 2.0) * tan_half
    dx = np.broadcast_to(xs[None, :], (height, width))
    dy = np.broadcast_to(ys[:, None], (height, width))
    dz = -np.ones((height, width))
    d = np.stack([dx, dy, dz], axis=-1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(np.asarray(eye, dtype=np.float64), d.shape)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def incoherent(n, seed=2, median=0.005, sigma=0.5):
    rng = _rng(seed)
    c = rng.uniform(0.0, 1.0, size=(n, 1, 3))
    dirs = rng.normal(size=(n, 3, 3))
    dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
    length = rng.lognormal(mean=math.log(median), sigma=sigma, size=(n, 3, 1))
    return (c + dirs * length).astype(np.float32)


def slivers(n, seed=5, length=1.0, width=0.01):
    """Long thin triangles in random directions from points in the unit
    cube: their boxes overlap heavily, the case spatial splits are for."""
    rng = _rng(seed)
    a = rng.uniform(0.0, 1.0, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    e = rng.normal(size=(n, 3))
    e -= (e * d).sum(1, keepdims=True) * d
    e /= np.linalg.norm(e, axis=1, keepdims=True)
    return np.stack([a, a + length * d, a + 0.5 * length * d + width * e], axis=1).astype(np.float32)


def plane_slivers(n, seed=32):
    """Thin triangles stretched along x, lying on the planes y = 0, 1/3 and
    2/3: spatial splits along y find no straddlers, the case of the spatial
    builder's equal-count fallback."""
    rng = _rng(seed)
    a = rng.uniform(0.0, 1.0, size=(n, 3))
    a[:, 1] = rng.integers(0, 3, n) / 3.0
    b = a.copy()
    b[:, 0] += rng.uniform(0.3, 1.0, n)
    c = a.copy()
    c[:, 2] += 0.01
    return np.stack([a, b, c], axis=1).astype(np.float32)


def incoherent_rays(count, seed=3, center=(0.5, 0.5, 0.5), radius=2.0, lo=0.0, hi=1.0):
    """Returns (rays (R,6) float32, any-hit t_max (R,) float32)."""
    rng = _rng(seed)
    u = rng.normal(size=(count, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    o = np.asarray(center, dtype=np.float64) + radius * u
    target = rng.uniform(lo, hi, size=(count, 3))
    d = target - o
    dist = np.linalg.norm(d, axis=1)
    d /= dist[:, None]
    rays = np.concatenate([o, d], axis=1).astype(np.float32)
    return rays, (0.5 * dist).astype(np.float32)


def clustered(total_tris, n_spheres=64, seed=4):
    """Spheres with radii log-uniform in [0.01, 0.2] and centres from a
    4-component Gaussian mixture clipped to [-1, 1]^3; each sphere's triangle
    count is proportional to its area (r^2), summing to about ``total_tris``."""
    rng = _rng(seed)
    radii = np.exp(rng.uniform(math.log(0.01), math.log(0.2), size=n_spheres))
    means = rng.uniform(-0.6, 0.6, size=(4, 3))
    comp = rng.integers(0, 4, size=n_spheres)
    centres = np.clip(means[comp] + rng.normal(scale=0.25, size=(n_spheres, 3)), -1.0, 1.0)
    w = radii ** 2
    counts = np.maximum(8, np.round(total_tris * w / w.sum())).astype(np.int64)
    parts = []
    for s in range(n_spheres):
        cells = max(4, int(counts[s] // 2))
        n_lat = max(2, int(round(math.sqrt(cells / 2.0))))
        n_lon = max(3, int(round(cells / n_lat)))
        parts.append(sphere_fast(n_lon, n_lat, radius=float(radii[s]), noise=0.05, seed=seed * 1000 + s,
                                 center=tuple(centres[s])))
    return np.concatenate(parts, axis=0)


def triangle_aabbs(tris):
    """RTAabb records (n, 8) float32 of triangles, as the shared crate's
    Triangle::aabb (grow over the three vertices, no offset); the int fields
    are zero."""
    t = np.asarray(tris, dtype=np.float32)
    out = np.zeros((len(t), 8), dtype=np.float32)
    out[:, 0:3] = t.min(axis=1)
    out[:, 4:7] = t.max(axis=1)
    return out


def triangle_centers(tris):
    """((v0 + v1) + v2) * (1/3) in float32, as the shared crate's Triangle::center."""
    t = np.asarray(tris, dtype=np.float32)
    s = (t[:, 0] + t[:, 1]) + t[:, 2]
    return (s * np.float32(1.0 / 3.0)).astype(np.float32)
