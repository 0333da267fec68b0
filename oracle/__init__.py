"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a C++ restatement of meirbon/rtbvh's CPU build and traversal
(see ``rtbvh_oracle.cpp`` for the per-function reference citations). It is the
parity checker of the CUDA implementation and the timed CPU baseline; the
product package never imports it.
"""
import ctypes
import os

import numpy as np

from . import buildlib as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        f32p = ctypes.POINTER(ctypes.c_float)
        L.ror_abi_sizes.argtypes = [ctypes.c_int32]
        L.ror_abi_sizes.restype = ctypes.c_int32
        L.ror_morton_split.argtypes = [ctypes.c_uint32]
        L.ror_morton_split.restype = ctypes.c_uint32
        L.ror_prefix_sum_u32.argtypes = [u32p, ctypes.c_size_t, u32p]
        L.ror_prefix_sum_u32.restype = ctypes.c_uint32
        L.ror_triangle_prep.argtypes = [f32p, ctypes.c_size_t, f32p, f32p]
        L.ror_triangle_prep.restype = None
        L.ror_union_of_list.argtypes = [f32p, ctypes.c_size_t, f32p]
        L.ror_union_of_list.restype = None
        L.ror_morton_codes.argtypes = [f32p, f32p, ctypes.c_size_t, u32p, u32p]
        L.ror_morton_codes.restype = None
        L.ror_build.argtypes = [f32p, f32p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int32,
                                ctypes.c_size_t, ctypes.c_uint32, f32p, u32p]
        L.ror_build.restype = ctypes.c_int64
        L.ror_spatial_max_refs.argtypes = [ctypes.c_size_t]
        L.ror_spatial_max_refs.restype = ctypes.c_uint64
        L.ror_build_spatial.argtypes = [f32p, f32p, f32p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32,
                                        ctypes.c_size_t, f32p, ctypes.c_size_t, u32p, ctypes.c_size_t]
        L.ror_build_spatial.restype = ctypes.c_int64
        L.ror_mbvh.argtypes = [f32p, ctypes.c_size_t, f32p]
        L.ror_mbvh.restype = ctypes.c_int64
        L.ror_refit.argtypes = [f32p, ctypes.c_size_t, u32p, f32p, ctypes.c_size_t]
        L.ror_refit.restype = None
        L.ror_validate.argtypes = [f32p, ctypes.c_size_t, u32p, ctypes.c_size_t]
        L.ror_validate.restype = ctypes.c_int32
        L.ror_trace.argtypes = [ctypes.c_int32, f32p, ctypes.c_size_t, u32p, f32p, f32p, ctypes.c_size_t,
                                f32p, ctypes.c_float, ctypes.c_int32, f32p, u32p, ctypes.c_uint32]
        L.ror_trace.restype = ctypes.c_int64
        L.ror_trace_packets.argtypes = [ctypes.c_int32, f32p, ctypes.c_size_t, u32p, f32p,
                                        ctypes.POINTER(f32p), f32p, ctypes.c_size_t, ctypes.c_float,
                                        f32p, u32p, ctypes.c_uint32]
        L.ror_trace_packets.restype = ctypes.c_int64
        L.ror_candidates.argtypes = [ctypes.c_int32, f32p, ctypes.c_size_t, u32p, f32p, ctypes.c_size_t, f32p,
                                     ctypes.c_uint32, u32p, u32p]
        L.ror_candidates.restype = ctypes.c_int64
        _lib = L
    return _lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _u(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def morton_split(v: int) -> int:
    return int(lib().ror_morton_split(v))


def prefix_sum(values):
    a = _c(values, np.uint32)
    out = np.zeros(max(len(a), 1), np.uint32)
    if len(a) == 0:
        a = np.zeros(1, np.uint32)
        total = lib().ror_prefix_sum_u32(_u(a), 0, _u(out))
        return total, out[:0]
    total = lib().ror_prefix_sum_u32(_u(a), len(a), _u(out))
    return int(total), out


def triangle_prep(tris):
    """(aabbs (n,8), centers (n,3)) of triangles as the shared crate computes them."""
    t = _c(tris, np.float32).reshape(-1, 9)
    n = len(t)
    a = np.zeros((n, 8), np.float32)
    c = np.zeros((n, 3), np.float32)
    if n:
        lib().ror_triangle_prep(_f(t), n, _f(a), _f(c))
    return a, c


def union_of_list(aabbs):
    a = _c(aabbs, np.float32).reshape(-1, 8)
    out = np.zeros(8, np.float32)
    lib().ror_union_of_list(_f(a), len(a), _f(out))
    return out


def morton_codes(aabbs, centers):
    a = _c(aabbs, np.float32).reshape(-1, 8)
    c = _c(centers, np.float32).reshape(-1, 3)
    n = len(a)
    codes = np.zeros(n, np.uint32)
    idx = np.zeros(n, np.uint32)
    lib().ror_morton_codes(_f(a), _f(c), n, _u(codes), _u(idx))
    return codes, idx


class OracleError(RuntimeError):
    pass


def build(aabbs, centers, build_type: str, prims_per_leaf: int = 1, spawn_threshold: int = 0, threads: int = 1):
    """Returns (nodes (m,8) float32, prim_indices (n,) uint32)."""
    a = _c(aabbs, np.float32).reshape(-1, 8)
    c = _c(centers, np.float32).reshape(-1, 3)
    n = len(a)
    if n == 0:
        raise OracleError("NoPrimitives")
    nodes = np.zeros((2 * n - 1, 8), np.float32)
    idx = np.zeros(n, np.uint32)
    bt = {"locb": 0, "sah": 1}[build_type]
    m = lib().ror_build(_f(a), _f(c), n, prims_per_leaf, bt, spawn_threshold, threads, _f(nodes), _u(idx))
    if m < 0:
        raise OracleError(f"build failed ({m})")
    return nodes[:m].copy(), idx


# Corrections of the reference's spatial-split builder (bit flags, 0 = as
# written); rtbvh_oracle.cpp SpatialFix says what each one changes.
SPATIAL_FIX_CLIP = 1
SPATIAL_FIX_EXIT_BIN = 2
SPATIAL_FIX_SWEEP_BOX = 4
SPATIAL_FIX_SPLIT_SPACE = 8
SPATIAL_FIX_FALLBACK = 16
SPATIAL_FIX_ALL = 31


def spatial_max_refs(n: int) -> int:
    return int(lib().ror_spatial_max_refs(n))


def build_spatial(tris, aabbs=None, centers=None, prims_per_leaf: int = 1, fixes: int = 0, spawn_threshold: int = 0):
    """Spatial-split SAH build (src/builders/spatial_sah.rs). Returns (nodes
    (m,8) float32, prim_indices (max_refs,) uint32, the reference's full
    index vector). Raises OracleError where the reference panics.
    spawn_threshold > 0 runs the reference's threading (1024 in the
    reference) with the same output."""
    t = _c(tris, np.float32).reshape(-1, 9)
    n = len(t)
    if n == 0:
        raise OracleError("NoPrimitives")
    if aabbs is None or centers is None:
        pa, pc = triangle_prep(t)
        aabbs = pa if aabbs is None else aabbs
        centers = pc if centers is None else centers
    a = _c(aabbs, np.float32).reshape(-1, 8)
    c = _c(centers, np.float32).reshape(-1, 3)
    mr = spatial_max_refs(n)
    nodes = np.zeros((2 * mr + 1, 8), np.float32)
    idx = np.zeros(mr, np.uint32)
    m = lib().ror_build_spatial(_f(a), _f(c), _f(t), n, prims_per_leaf, fixes, spawn_threshold, _f(nodes), len(nodes),
                                _u(idx), len(idx))
    if m == -3:
        raise OracleError("the reference panics on this input")
    if m < 0:
        raise OracleError(f"build failed ({m})")
    return nodes[:m].copy(), idx


def mbvh(nodes):
    nd = _c(nodes, np.float32).reshape(-1, 8)
    out = np.zeros((max(len(nd), 1), 32), np.float32)
    k = lib().ror_mbvh(_f(nd), len(nd), _f(out))
    return out[:k].copy()


def refit(nodes, prim_indices, new_aabbs):
    nd = _c(nodes, np.float32).reshape(-1, 8).copy()
    idx = _c(prim_indices, np.uint32)
    na = _c(new_aabbs, np.float32).reshape(-1, 8)
    lib().ror_refit(_f(nd), len(nd), _u(idx), _f(na), len(na))
    return nd


def validate(nodes, prim_indices, prim_count):
    nd = _c(nodes, np.float32).reshape(-1, 8)
    idx = _c(prim_indices, np.uint32)
    return bool(lib().ror_validate(_f(nd), len(nd), _u(idx), prim_count))


def trace(structure: str, nodes, prim_indices, tris, rays, t_max=None, t_min_tri=1e-4, any_hit=False,
          threads: int = 1, stats: bool = True):
    """Returns (hits (R,4) float32 [t,u,v,prim bits], stats (R,3) uint32 or None, overflows)."""
    st = {"mbvh": 0, "bvh": 1}[structure]
    nd = _c(nodes, np.float32).reshape(-1, 32 if st == 0 else 8)
    idx = _c(prim_indices, np.uint32)
    tr = _c(tris, np.float32).reshape(-1, 9)
    ry = _c(rays, np.float32).reshape(-1, 6)
    R = len(ry)
    hits = np.zeros((R, 4), np.float32)
    sts = np.zeros((R, 3), np.uint32) if stats else None
    tm = None
    if t_max is not None:
        tm = _c(np.broadcast_to(np.asarray(t_max, np.float32), (R,)), np.float32)
    bad = lib().ror_trace(st, _f(nd), len(nd), _u(idx), _f(tr), _f(ry), R,
                          _f(tm) if tm is not None else None, float(t_min_tri), int(bool(any_hit)),
                          _f(hits), _u(sts) if sts is not None else None, threads)
    return hits, sts, int(bad)


def trace_packets(structure: str, nodes, prim_indices, tris, rays, t=None, t_min_tri=1e-4, threads: int = 1):
    """Packet traversal; packet p = rays 4p..4p+3 (len(rays) must be a multiple of 4).

    Returns (hits (R,4) float32 [t,u,v,prim bits], stats (P,3) uint32, overflows).
    """
    st = {"mbvh": 0, "bvh": 1}[structure]
    nd = _c(nodes, np.float32).reshape(-1, 32 if st == 0 else 8)
    idx = _c(prim_indices, np.uint32)
    tr = _c(tris, np.float32).reshape(-1, 9)
    ry = _c(rays, np.float32).reshape(-1, 6)
    R = len(ry)
    if R % 4:
        raise ValueError("packet traversal needs a multiple of 4 rays")
    P = R // 4
    soa = [np.ascontiguousarray(ry[:, k]) for k in range(6)]
    tt = np.full(R, 1e34, np.float32) if t is None else _c(np.broadcast_to(np.asarray(t, np.float32), (R,)),
                                                            np.float32).copy()
    arr = (ctypes.POINTER(ctypes.c_float) * 6)(*[_f(a) for a in soa])
    hits = np.zeros((R, 4), np.float32)
    sts = np.zeros((P, 3), np.uint32)
    bad = lib().ror_trace_packets(st, _f(nd), len(nd), _u(idx), _f(tr), arr, _f(tt), P, float(t_min_tri),
                                  _f(hits), _u(sts), threads)
    return hits, sts, int(bad)


def candidates(structure: str, nodes, prim_indices, rays, t_max=None, max_per_ray: int = 64):
    """Primitive ids the reference's index iterator yields per ray when the
    callback leaves t unchanged, in yield order.

    Returns (cands (R, max_per_ray) uint32, counts (R,) uint32 full yield counts).
    """
    st = {"mbvh": 0, "bvh": 1}[structure]
    nd = _c(nodes, np.float32).reshape(-1, 32 if st == 0 else 8)
    idx = _c(prim_indices, np.uint32)
    ry = _c(rays, np.float32).reshape(-1, 6)
    R = len(ry)
    tm = None
    if t_max is not None:
        tm = _c(np.broadcast_to(np.asarray(t_max, np.float32), (R,)), np.float32)
    cands = np.zeros((R, max(int(max_per_ray), 1)), np.uint32)
    counts = np.zeros(R, np.uint32)
    lib().ror_candidates(st, _f(nd), len(nd), _u(idx), _f(ry), R, _f(tm) if tm is not None else None,
                         int(max_per_ray), _u(cands), _u(counts))
    return cands[:, :max_per_ray], counts


def hit_prims(hits):
    return np.ascontiguousarray(hits[:, 3]).view(np.int32)
