"""Python mirror of the reference crate's public API for the BVH path.

Names and error behaviour follow the Rust crate:

* ``Builder(aabbs, primitives, primitives_per_leaf)`` with
  ``construct_binned_sah()`` / ``construct_locally_ordered_clustered()``
  (src/bvh.rs:49-138), raising ``BuildError`` with the reference's two
  variants (src/bvh.rs:26-29);
* ``Bvh`` (src/bvh.rs:143-284) and ``Mbvh`` (src/bvh.rs:320-444) with
  ``nodes()``, ``indices()``, ``quad_nodes()``, ``prim_count()``,
  ``refit()``, ``validate()`` and ``Mbvh.construct(bvh)`` / ``Mbvh.from_bvh``
  (``From<Bvh> for Mbvh``, src/bvh.rs:446-450).

Builds and traversal run in the CUDA library through its C ABI; device
memory, streams and the autograd harness use PyTorch. Primitives are
``Triangles`` (the shared crate's Triangle: v0, v1, v2) or ``Points`` (the
FFI's Vector3/Vector4 primitives, rtbvh_ffi/src/lib.rs:391-422).
"""
import ctypes
import enum

import numpy as np
import torch

from . import _ffi
from ._ffi import BvhType, ResultCode, RtbvhError, check


class BuildType(enum.IntEnum):
    """src/bvh.rs:18-23"""
    None_ = 0
    LocallyOrderedClustered = 1
    BinnedSAH = 2
    Spatial = 3


class BuildError(Exception):
    """src/bvh.rs:26-46: NoPrimitives | InequalAabbsAndPrimitives(aabbs, prims)."""

    def __init__(self, kind, aabbs=None, prims=None):
        self.kind = kind
        self.counts = (aabbs, prims)
        if kind == "NoPrimitives":
            msg = "No primitives supplied"
        else:
            msg = f"#Aabbs({aabbs}) != #Primitives({prims})"
        super().__init__(msg)

    def __eq__(self, other):
        return isinstance(other, BuildError) and (self.kind, self.counts) == (other.kind, other.counts)

    def __hash__(self):
        return hash((self.kind, self.counts))

    @classmethod
    def NoPrimitives(cls):
        return cls("NoPrimitives")

    @classmethod
    def InequalAabbsAndPrimitives(cls, aabbs, prims):
        return cls("InequalAabbsAndPrimitives", aabbs, prims)


def _stream(stream=None):
    if stream is None:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, torch.cuda.Stream):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def _cuda_f32(x, shape_last=None):
    t = torch.as_tensor(x)
    if t.dtype != torch.float32:
        t = t.to(torch.float32)
    if not t.is_cuda:
        t = t.cuda()
    t = t.contiguous()
    if shape_last is not None:
        t = t.reshape(-1, shape_last)
    return t


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Triangles:
    """Triangle primitives: (n, 3, 3) float32 vertices (v0, v1, v2). Their
    aabb/center are the shared crate's Triangle::aabb / Triangle::center."""

    def __init__(self, vertices):
        self.vertices = _cuda_f32(vertices).reshape(-1, 3, 3)

    def __len__(self):
        return self.vertices.shape[0]


class Points:
    """Point primitives (centre = the point, box = the degenerate point box)."""

    def __init__(self, centers):
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float32))
        if c.ndim != 2 or c.shape[1] not in (3, 4):
            raise ValueError("centers must be (n, 3) or (n, 4)")
        self.centers = c

    def __len__(self):
        return self.centers.shape[0]


def _aabbs_array(aabbs):
    a = np.ascontiguousarray(np.asarray(aabbs, dtype=np.float32))
    return a.reshape(-1, 8)


class Bvh:
    """A library-owned BVH (handle + device arrays)."""

    def __init__(self, handle, build_type, prim_count):
        self._h = handle
        self._build_type = build_type
        self._n = prim_count
        self._lib = _ffi.load()

    @property
    def handle(self):
        return self._h

    def build_type(self):
        return self._build_type

    def prim_count(self):
        return self._n

    def nodes(self):
        """(node_count, 8) float32 copy of the nodes (RTBvhNode layout)."""
        h = self._h
        if h.node_count == 0:
            return np.zeros((0, 8), np.float32)
        if not h.nodes:
            raise RtbvhError(ResultCode.Error, "nodes are device-only")
        buf = ctypes.cast(h.nodes, ctypes.POINTER(ctypes.c_float * (8 * h.node_count))).contents
        return np.frombuffer(buf, dtype=np.float32).reshape(-1, 8).copy()

    def indices(self):
        h = self._h
        if h.index_count == 0:
            return np.zeros(0, np.uint32)
        buf = ctypes.cast(h.indices, ctypes.POINTER(ctypes.c_uint32 * h.index_count)).contents
        return np.frombuffer(buf, dtype=np.uint32).copy()

    def refit(self, new_aabbs=None, triangles=None, mbvh=None, stream=None):
        """Bvh::refit (src/bvh.rs:176-205) on the GPU from new primitive boxes
        or new triangle vertices; optionally re-collapses ``mbvh`` from it."""
        if (new_aabbs is None) == (triangles is None):
            raise ValueError("give exactly one of new_aabbs / triangles")
        mid = mbvh.handle.id if mbvh is not None else 0xFFFFFFFF
        if triangles is not None:
            v = triangles.vertices if isinstance(triangles, Triangles) else _cuda_f32(triangles)
            check(self._lib.rtbvh_gpu_refit(self._h.id, _ptr(v), None, mid, _stream(stream)), "refit")
        else:
            a = _cuda_f32(_aabbs_array(new_aabbs))
            check(self._lib.rtbvh_gpu_refit(self._h.id, None, _ptr(a), mid, _stream(stream)), "refit")
        # the host mirror was refreshed in place; the handle stays valid

    def validate(self, prim_count):
        """Bvh::validate (src/bvh.rs:230-244): every primitive referenced."""
        nodes = self.nodes()
        idx = self.indices()
        ints = nodes.view(np.int32)
        seen = np.zeros(prim_count, bool)
        stack = [0] if len(nodes) else []
        while stack:
            c = stack.pop()
            cnt, lf = int(ints[c, 3]), int(ints[c, 7])
            if lf < 0:
                continue
            if cnt >= 0:
                seen[idx[lf:lf + cnt]] = True
            else:
                stack += [lf, lf + 1]
        return bool(seen.all())

    def bounds(self):
        n = self.nodes()
        return n[0].copy() if len(n) else None

    def intersect(self, rays, t_max=None, any_hit=False, stats=False, stream=None):
        """GPU BvhIndexIterator + triangle test for a batch of rays."""
        return _trace(self._lib.rtbvh_gpu_intersect_bvh, self._h, rays, t_max, any_hit, stats, stream)

    def intersect_packets(self, rays, t=None, stats=False, stream=None):
        """GPU BvhPacketIndexIterator + packet triangle test; packet p is
        rays 4p..4p+3. Returns (hits (R,4) CUDA tensor [t, u, v, prim bits],
        stats (P,3) int32 or None)."""
        return _trace_packets(self._lib.rtbvh_gpu_intersect_bvh_packets, self._h, rays, t, stats, stream)

    def candidates(self, rays, t_max=None, max_per_ray=64, stream=None):
        """Primitive ids BvhIndexIterator yields per ray (callback leaving t
        unchanged), in order: (cands (R, max_per_ray) int32 CUDA tensor,
        counts (R,) int32 -- full yield counts, may exceed max_per_ray)."""
        return _candidates(self._lib.rtbvh_gpu_bvh_candidates, self._h, rays, t_max, max_per_ray, stream)

    def attach_triangles(self, vertices, stream=None):
        """Device triangles (n, 3, 3) for the GPU traces of a structure that
        has none (e.g. one loaded with from_bytes)."""
        v = _cuda_f32(vertices)
        check(self._lib.rtbvh_gpu_set_triangles(self._h.id, 0, _ptr(v), v.numel() // 9, _stream(stream)),
              "set_triangles")

    def to_bytes(self):
        """The crate's serde form of the Bvh in bincode 1 layout (see rtbvh.h)."""
        return _serialize(self._lib.rtbvh_serialize_bvh, self._h)

    @classmethod
    def from_bytes(cls, data, host_mirror=True, stream=None):
        lib = _ffi.load()
        out = _ffi.RTBvh()
        buf = bytes(data)
        flags = 0 if host_mirror else _ffi.FLAG_NO_HOST_MIRROR
        check(lib.rtbvh_deserialize_bvh(buf, len(buf), flags, _stream(stream), ctypes.byref(out)), "deserialize_bvh")
        build_type = BuildType(int.from_bytes(buf[-4:], "little"))
        return cls(out, build_type, out.index_count)

    def save(self, path):
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def load(cls, path, host_mirror=True):
        with open(path, "rb") as f:
            return cls.from_bytes(f.read(), host_mirror=host_mirror)

    def status(self):
        return ResultCode(self._lib.rtbvh_gpu_status(self._h.id, 0))

    def __del__(self):
        try:
            self._lib.free_bvh(self._h)
        except Exception:
            pass


class Mbvh:
    """A library-owned 4-wide MBVH."""

    def __init__(self, handle, prim_count, source):
        self._h = handle
        self._n = prim_count
        self._source = source  # keeps the Bvh (and its triangles) alive
        self._lib = _ffi.load()

    @classmethod
    def construct(cls, bvh: Bvh, stream=None, host_mirror=True):
        """Mbvh::construct (src/bvh.rs:381-404) on the GPU."""
        lib = _ffi.load()
        out = _ffi.RTMbvh()
        flags = 0 if host_mirror else _ffi.FLAG_NO_HOST_MIRROR
        check(lib.rtbvh_gpu_create_mbvh(bvh.handle, flags, _stream(stream), ctypes.byref(out)), "create_mbvh")
        return cls(out, bvh.prim_count(), bvh)

    from_bvh = construct

    @property
    def handle(self):
        return self._h

    def prim_count(self):
        return self._n

    def quad_nodes(self):
        """(node_count, 32) float32 copy (RTMbvhNode layout)."""
        h = self._h
        if h.node_count == 0:
            return np.zeros((0, 32), np.float32)
        if not h.nodes:
            raise RtbvhError(ResultCode.Error, "nodes are device-only")
        buf = ctypes.cast(h.nodes, ctypes.POINTER(ctypes.c_float * (32 * h.node_count))).contents
        return np.frombuffer(buf, dtype=np.float32).reshape(-1, 32).copy()

    def indices(self):
        h = self._h
        if h.index_count == 0:
            return np.zeros(0, np.uint32)
        buf = ctypes.cast(h.indices, ctypes.POINTER(ctypes.c_uint32 * h.index_count)).contents
        return np.frombuffer(buf, dtype=np.uint32).copy()

    def intersect(self, rays, t_max=None, any_hit=False, stats=False, stream=None, reorder=False,
                  exact_nodes=False, walk_stats=False):
        """GPU MbvhIndexIterator + triangle test for a batch of rays.
        rays: (R, 6) float32 (CUDA tensor or array). Returns (hits (R,4)
        float32 CUDA tensor [t, u, v, prim bits], stats (R,3) int32 or None).
        reorder: trace in (origin, direction)-sorted order (same results).
        exact_nodes: closest hit over the exact 128-byte quad nodes in the
        reference's visit order (default: compact nodes, same nearest hit,
        either triangle where two are hit at exactly the same t).
        walk_stats: closest hit of the default walk with its own per-ray
        counts as stats: traversal-tree node visits, triangle tests, 1 if
        the ray was handed on to the exact walk."""
        return _trace(self._lib.rtbvh_gpu_intersect_mbvh, self._h, rays, t_max, any_hit, stats, stream, reorder,
                      exact_nodes, walk_stats)

    def intersect_packets(self, rays, t=None, stats=False, stream=None):
        """GPU MbvhPacketIndexIterator + packet triangle test (the reference's
        RayPacket4 path); packet p is rays 4p..4p+3 of the (R, 6) rays, R a
        multiple of 4. Returns (hits (R,4) CUDA tensor [t, u, v, prim bits],
        stats (P,3) int32 [node tests, triangle tests, max stack] or None)."""
        return _trace_packets(self._lib.rtbvh_gpu_intersect_mbvh_packets, self._h, rays, t, stats, stream)

    def candidates(self, rays, t_max=None, max_per_ray=64, stream=None):
        """Primitive ids MbvhIndexIterator yields per ray when the callback
        leaves t unchanged, in yield order -- the device form of
        intersect_mbvh with a user callback, for primitives tested by the
        caller (see Bvh.candidates for the return values)."""
        return _candidates(self._lib.rtbvh_gpu_mbvh_candidates, self._h, rays, t_max, max_per_ray, stream)

    def refit(self, new_aabbs=None, triangles=None, stream=None):
        """Refits the Mbvh's own copy of its Bvh nodes (Bvh::refit's
        arithmetic) and collapses the quad nodes again; the source Bvh is
        left as it was."""
        if (new_aabbs is None) == (triangles is None):
            raise ValueError("give exactly one of new_aabbs / triangles")
        if triangles is not None:
            v = triangles.vertices if isinstance(triangles, Triangles) else _cuda_f32(triangles)
            check(self._lib.rtbvh_gpu_refit_mbvh(self._h.id, _ptr(v), None, _stream(stream)), "refit_mbvh")
        else:
            a = _cuda_f32(_aabbs_array(new_aabbs))
            check(self._lib.rtbvh_gpu_refit_mbvh(self._h.id, None, _ptr(a), _stream(stream)), "refit_mbvh")

    def attach_triangles(self, vertices, stream=None):
        """Device triangles (n, 3, 3) for the GPU traces (see Bvh.attach_triangles)."""
        v = _cuda_f32(vertices)
        check(self._lib.rtbvh_gpu_set_triangles(self._h.id, 1, _ptr(v), v.numel() // 9, _stream(stream)),
              "set_triangles")

    def to_bytes(self):
        """The crate's serde form of the Mbvh in bincode 1 layout (see rtbvh.h)."""
        return _serialize(self._lib.rtbvh_serialize_mbvh, self._h)

    @classmethod
    def from_bytes(cls, data, host_mirror=True, stream=None):
        lib = _ffi.load()
        out = _ffi.RTMbvh()
        buf = bytes(data)
        flags = 0 if host_mirror else _ffi.FLAG_NO_HOST_MIRROR
        check(lib.rtbvh_deserialize_mbvh(buf, len(buf), flags, _stream(stream), ctypes.byref(out)),
              "deserialize_mbvh")
        return cls(out, out.index_count, None)

    def save(self, path):
        with open(path, "wb") as f:
            f.write(self.to_bytes())

    @classmethod
    def load(cls, path, host_mirror=True):
        with open(path, "rb") as f:
            return cls.from_bytes(f.read(), host_mirror=host_mirror)

    def traversal_tree(self):
        """(exact (count, 32) float32 quad records, compact (count, 16) uint32
        records) of the closest-hit traversal tree, copied to the host."""
        ex, cp, cnt = _ffi._vp(), _ffi._vp(), _ffi._u32()
        check(self._lib.rtbvh_gpu_traversal_tree(self._h, ctypes.byref(ex), ctypes.byref(cp), ctypes.byref(cnt)),
              "traversal_tree")
        n = cnt.value
        if n == 0:
            return np.zeros((0, 32), np.float32), np.zeros((0, 16), np.uint32)
        return device_copy(ex.value, (n, 32)), device_copy(cp.value, (n, 16), np.uint32)

    def intersect_host(self, rays, t_max=None, any_hit=False):
        """Same, with host (numpy) rays and hits, copies included
        (rtbvh_intersect_mbvh_batch)."""
        r = np.ascontiguousarray(np.asarray(rays, np.float32).reshape(-1, 6))
        tm = None if t_max is None else np.ascontiguousarray(np.asarray(t_max, np.float32).reshape(-1))
        hits = np.empty((len(r), 4), np.float32)
        flags = _ffi.TRACE_ANY_HIT if any_hit else 0
        check(self._lib.rtbvh_intersect_mbvh_batch(
            self._h, r.ctypes.data_as(ctypes.c_void_p), tm.ctypes.data_as(ctypes.c_void_p) if tm is not None else None,
            len(r), hits.ctypes.data_as(ctypes.c_void_p), flags), "intersect_mbvh_batch")
        return hits

    def status(self):
        return ResultCode(self._lib.rtbvh_gpu_status(self._h.id, 1))

    def __del__(self):
        try:
            self._lib.free_mbvh(self._h)
        except Exception:
            pass


def _trace(fn, handle, rays, t_max, any_hit, stats, stream, reorder=False, exact_nodes=False, walk_stats=False):
    r = _cuda_f32(rays, 6)
    n = r.shape[0]
    tm = _cuda_f32(t_max).reshape(-1) if t_max is not None else None
    hits = torch.empty((n, 4), dtype=torch.float32, device=r.device)
    st = torch.empty((n, 3), dtype=torch.int32, device=r.device) if (stats or walk_stats) else None
    flags = (_ffi.TRACE_ANY_HIT if any_hit else 0) | (_ffi.TRACE_STATS if stats else 0)
    flags |= _ffi.TRACE_REORDER if reorder else 0
    flags |= _ffi.TRACE_EXACT_NODES if exact_nodes else 0
    flags |= _ffi.TRACE_WALK_STATS if walk_stats else 0
    check(fn(handle, _ptr(r), _ptr(tm), n, _ptr(hits), flags, _ptr(st), _stream(stream)), "intersect")
    return hits, st


def _trace_packets(fn, handle, rays, t, stats, stream):
    r = _cuda_f32(rays, 6)
    n = r.shape[0]
    if n % 4:
        raise ValueError("packet traversal needs a multiple of 4 rays")
    soa = r.t().contiguous()  # (6, R): origin x, y, z, direction x, y, z
    tt = (torch.full((n,), 1e34, dtype=torch.float32, device=r.device) if t is None
          else _cuda_f32(t).reshape(-1).expand(n).contiguous().clone())
    hits = torch.empty((n, 4), dtype=torch.float32, device=r.device)
    st = torch.empty((n // 4, 3), dtype=torch.int32, device=r.device) if stats else None
    flags = _ffi.TRACE_STATS if stats else 0
    ptrs = [ctypes.c_void_p(soa[k].data_ptr()) for k in range(6)]
    check(fn(handle, *ptrs, _ptr(tt), n // 4, _ptr(hits), flags, _ptr(st), _stream(stream)), "intersect_packets")
    return hits, st


def _serialize(fn, handle):
    size = ctypes.c_size_t(0)
    check(fn(handle, None, 0, ctypes.byref(size)), "serialize")
    buf = ctypes.create_string_buffer(size.value)
    check(fn(handle, buf, size.value, ctypes.byref(size)), "serialize")
    return buf.raw[:size.value]


def _candidates(fn, handle, rays, t_max, max_per_ray, stream):
    r = _cuda_f32(rays, 6)
    n = r.shape[0]
    tm = _cuda_f32(t_max).reshape(-1) if t_max is not None else None
    m = int(max_per_ray)
    cands = torch.empty((n, max(m, 1)), dtype=torch.int32, device=r.device) if m > 0 else None
    counts = torch.empty((n,), dtype=torch.int32, device=r.device)
    check(fn(handle, _ptr(r), _ptr(tm), n, m, _ptr(cands), _ptr(counts), _stream(stream)), "candidates")
    return (cands[:, :m] if cands is not None else None), counts


class Builder:
    """src/bvh.rs:49-56: {aabbs: Option<&[Aabb]>, primitives, primitives_per_leaf}."""

    def __init__(self, aabbs=None, primitives=None, primitives_per_leaf=None):
        self.aabbs = aabbs
        self.primitives = primitives
        self.primitives_per_leaf = primitives_per_leaf

    def construct_binned_sah(self, stream=None, host_mirror=True) -> Bvh:
        return self._construct(BvhType.BinnedSAH, stream, host_mirror)

    def construct_locally_ordered_clustered(self, stream=None, host_mirror=True) -> Bvh:
        return self._construct(BvhType.LocallyOrderedClustered, stream, host_mirror)

    def construct_spatial_sah(self, stream=None, host_mirror=True, fixes=0) -> Bvh:
        """Builder::construct_spatial_sah (src/bvh.rs:59-85) on the GPU;
        primitives must be Triangles. ``fixes`` (SPATIAL_FIX_* bits of
        ``rtbvh_gb300._ffi``) corrects defects of the reference builder;
        0 reproduces it as written, which on many inputs leaves some
        primitives out of every leaf."""
        prims = self.primitives
        n = 0 if prims is None else len(prims)
        if n == 0:
            raise BuildError.NoPrimitives()
        if not isinstance(prims, Triangles):
            raise TypeError("the spatial-split builder needs Triangles (SpatialTriangle)")
        aabbs = None if self.aabbs is None else _aabbs_array(self.aabbs)
        if aabbs is not None and len(aabbs) != n:
            raise BuildError.InequalAabbsAndPrimitives(len(aabbs), n)
        a = _cuda_f32(aabbs) if aabbs is not None else None
        lib = _ffi.load()
        out = _ffi.RTBvh()
        flags = 0 if host_mirror else _ffi.FLAG_NO_HOST_MIRROR
        check(lib.rtbvh_gpu_create_spatial_bvh(_ptr(prims.vertices), n, _ptr(a), None, 0,
                                               int(self.primitives_per_leaf or 0), int(fixes), flags,
                                               _stream(stream), ctypes.byref(out)), "create_spatial_bvh")
        return Bvh(out, BuildType.Spatial, n)

    def _construct(self, bvh_type, stream, host_mirror):
        prims = self.primitives
        n = 0 if prims is None else len(prims)
        if n == 0:
            raise BuildError.NoPrimitives()
        aabbs = None if self.aabbs is None else _aabbs_array(self.aabbs)
        if aabbs is not None and len(aabbs) != n:
            raise BuildError.InequalAabbsAndPrimitives(len(aabbs), n)
        ppl = int(self.primitives_per_leaf or 0)
        lib = _ffi.load()
        out = _ffi.RTBvh()
        flags = 0 if host_mirror else _ffi.FLAG_NO_HOST_MIRROR
        s = _stream(stream)
        build_type = BuildType.BinnedSAH if bvh_type == BvhType.BinnedSAH else BuildType.LocallyOrderedClustered
        if isinstance(prims, Triangles):
            if aabbs is None:
                rc = lib.rtbvh_gpu_create_bvh_from_triangles(_ptr(prims.vertices), n, ppl, int(bvh_type), flags, s,
                                                             ctypes.byref(out))
                check(rc, "create_bvh_from_triangles")
            else:
                v = prims.vertices
                centers = ((v[:, 0] + v[:, 1]) + v[:, 2]) * torch.tensor(1.0 / 3.0, dtype=torch.float32)
                centers = centers.contiguous()
                a = _cuda_f32(aabbs)
                rc = lib.rtbvh_gpu_create_bvh(_ptr(a), n, _ptr(centers), 12, ppl, int(bvh_type), flags, s,
                                              ctypes.byref(out))
                check(rc, "create_bvh")
                check(lib.rtbvh_gpu_set_triangles(out.id, 0, _ptr(v), n, s), "set_triangles")
        elif isinstance(prims, Points):
            c = prims.centers
            aptr = None
            if aabbs is not None:
                aptr = aabbs.ctypes.data_as(ctypes.POINTER(_ffi.RTAabb))
            rc = lib.create_bvh(aptr, n, c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), c.shape[1] * 4, ppl,
                                int(bvh_type), ctypes.byref(out))
            check(rc, "create_bvh")
        else:
            raise TypeError("primitives must be Triangles or Points")
        return Bvh(out, build_type, n)


class Batch:
    """Many meshes built and traced together (rtbvh_gpu_batch_*): mesh m owns
    triangles [prim_offsets[m], prim_offsets[m + 1]) of `vertices` and rays
    [ray_offsets[m], ray_offsets[m + 1]) of `rays`. The whole build + trace
    is captured in a CUDA graph at construction; run() replays it. The
    vertex/ray tensors are bound by address: change their contents in place."""

    def __init__(self, vertices, prim_offsets, rays, ray_offsets, t_max=None, any_hit=False, stream=None):
        self._lib = _ffi.load()
        self.vertices = _cuda_f32(vertices).reshape(-1, 3, 3)
        self.rays = _cuda_f32(rays, 6)
        self.t_max = _cuda_f32(t_max).reshape(-1) if t_max is not None else None
        self.prim_offsets = np.ascontiguousarray(np.asarray(prim_offsets, dtype=np.uint32))
        self.ray_offsets = np.ascontiguousarray(np.asarray(ray_offsets, dtype=np.uint32))
        self.mesh_count = len(self.prim_offsets) - 1
        self.hits = torch.empty((self.rays.shape[0], 4), dtype=torch.float32, device=self.rays.device)
        self._b = _ffi.RTBatch()
        flags = _ffi.TRACE_ANY_HIT if any_hit else 0
        check(self._lib.rtbvh_gpu_batch_create(
            _ptr(self.vertices), self.prim_offsets.ctypes.data_as(ctypes.c_void_p), self.mesh_count,
            _ptr(self.rays), _ptr(self.t_max), self.ray_offsets.ctypes.data_as(ctypes.c_void_p), _ptr(self.hits),
            flags, _stream(stream), ctypes.byref(self._b)), "batch_create")

    def run(self, graph=True, stream=None):
        fn = self._lib.rtbvh_gpu_batch_run if graph else self._lib.rtbvh_gpu_batch_run_uncaptured
        check(fn(self._b, _stream(stream)), "batch_run")
        return self.hits

    def tune(self, stream=None):
        """Times candidate launch parameters on this batch (the pipeline runs
        several times), keeps the fastest and re-captures the graph. Returns
        the chosen values and the measured build + trace time."""
        t = _ffi.RTBatchTuning()
        check(self._lib.rtbvh_gpu_batch_tune(self._b, _stream(stream), ctypes.byref(t)), "batch_tune")
        return {"trace_blocks_per_sm": t.trace_blocks_per_sm, "trace_ray_batch": t.trace_ray_batch,
                "cluster_min_prims": t.cluster_min_prims, "trace_stack": t.trace_stack,
                "pipeline_ms": t.pipeline_ms}

    @property
    def tuning(self):
        t = _ffi.RTBatchTuning()
        check(self._lib.rtbvh_gpu_batch_get_tuning(self._b, ctypes.byref(t)), "batch_get_tuning")
        return {"trace_blocks_per_sm": t.trace_blocks_per_sm, "trace_ray_batch": t.trace_ray_batch,
                "cluster_min_prims": t.cluster_min_prims, "trace_stack": t.trace_stack}

    def set_tuning(self, trace_blocks_per_sm=0, trace_ray_batch=0, cluster_min_prims=0, trace_stack=0, stream=None):
        t = _ffi.RTBatchTuning(trace_blocks_per_sm, trace_ray_batch, cluster_min_prims, 0.0, trace_stack)
        check(self._lib.rtbvh_gpu_batch_set_tuning(self._b, ctypes.byref(t), _stream(stream)), "batch_set_tuning")

    def view(self):
        v = _ffi.RTGpuBatchView()
        check(self._lib.rtbvh_gpu_batch_view(self._b, ctypes.byref(v)), "batch_view")
        return v

    def status(self):
        return ResultCode(self._lib.rtbvh_gpu_batch_status(self._b))

    def __del__(self):
        try:
            self._lib.rtbvh_gpu_batch_free(self._b)
        except Exception:
            pass


class DeviceArray:
    """Zero-copy view of library-owned device memory (for torch.as_tensor).
    torch accepts only writable views; callers must not write through it."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3}


def device_copy(ptr, shape, dtype=np.float32):
    """Host numpy copy of library-owned device memory (4-byte element types)."""
    dtype = np.dtype(dtype)
    if dtype.itemsize != 4:
        raise ValueError("device_copy handles 4-byte element types")
    t = torch.as_tensor(DeviceArray(ptr, shape, "<i4"), device="cuda")
    return t.clone().cpu().numpy().view(dtype)


def hit_prims(hits):
    """int32 primitive ids of a (R, 4) hits array/tensor (-1: miss)."""
    if isinstance(hits, torch.Tensor):
        return hits[:, 3].contiguous().view(torch.int32)
    return np.ascontiguousarray(hits[:, 3]).view(np.int32)
