"""The C-ABI library without a GPU: it loads, exports every declared symbol,
keeps the reference's layouts, and its host-side entry points behave like
rtbvh_ffi (argument checks, result codes, callback traversal)."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
import rtbvh_gb300 as rb
from rtbvh_gb300 import _ffi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "rtbvh.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^(?:ResultCode|void|const\s+char\s*\*)\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "create_bvh" in names and "rtbvh_gpu_intersect_mbvh" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_ffi.SIGNATURES), "ctypes signatures out of sync with include/rtbvh.h"


def test_alias_library_name_exists(lib):
    # C users of the reference link librtbvh_rs (rtbvh_ffi/Cargo.toml [lib] name)
    assert os.path.exists(os.path.join(ROOT, "rtbvh_gb300", "_lib", "librtbvh_rs.so"))


def test_struct_layouts(golden):
    # rtbvh_ffi/src/lib.rs:855-866
    k = golden["known"]["abi_sizes"]
    assert ctypes.sizeof(_ffi.RTAabb) == k["RTAabb"]
    assert ctypes.sizeof(_ffi.RTBvhNode) == k["RTBvhNode"]
    assert ctypes.sizeof(_ffi.RTMbvhNode) == k["RTMbvhNode"]
    assert ctypes.sizeof(_ffi.RTBvh) == 32 and ctypes.sizeof(_ffi.RTMbvh) == 32


def test_result_code_and_type_values(golden):
    for name, v in golden["known"]["result_codes"].items():
        if name != "source":
            assert int(_ffi.ResultCode[name]) == v
    for name, v in golden["known"]["bvh_type"].items():
        if name != "source":
            assert int(_ffi.BvhType[name]) == v


def test_create_bvh_argument_errors(lib):
    # rtbvh_ffi/src/lib.rs:437-449 and the create_delete test (:868-904)
    out = _ffi.RTBvh()
    centers = np.zeros((27, 4), np.float32)
    cp = centers.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.create_bvh(None, 27, None, 16, 1, 1, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_bvh(None, 27, cp, 16, 1, 1, None) == _ffi.ResultCode.Error
    for stride in (8, 13, 20):  # the reference aborts; this library reports Error
        assert lib.create_bvh(None, 27, cp, stride, 1, 1, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_bvh(None, 0, cp, 16, 1, 1, ctypes.byref(out)) == _ffi.ResultCode.NoPrimitives
    # create_spatial_Bvh (rtbvh_ffi/src/lib.rs:345-389): no vertices, no
    # centres (the wrapper dereferences both), a stride that is not a
    # multiple of 4 (assert_eq! in the reference), no primitives
    vp = np.zeros((27, 3, 4), np.float32).ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.create_spatial_Bvh(None, 27, cp, 16, None, 0, 0, 1, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_spatial_Bvh(None, 27, None, 16, vp, 16, 48, 1, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_spatial_Bvh(None, 27, cp, 14, vp, 16, 48, 1, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_spatial_Bvh(None, 27, cp, 16, vp, 16, 48, 1, None) == _ffi.ResultCode.Error
    assert lib.create_spatial_Bvh(None, 0, cp, 16, vp, 16, 48, 1, ctypes.byref(out)) == _ffi.ResultCode.NoPrimitives
    assert lib.rtbvh_gpu_create_spatial_bvh(None, 0, None, None, 0, 1, 0, 0, None,
                                            ctypes.byref(out)) == _ffi.ResultCode.NoPrimitives


def test_create_mbvh_and_refit_null_checks(lib):
    empty = _ffi.RTBvh()
    out = _ffi.RTMbvh()
    assert lib.create_mbvh(empty, ctypes.byref(out)) == _ffi.ResultCode.Error
    assert lib.create_mbvh(empty, None) == _ffi.ResultCode.Error
    assert lib.refit(None, empty) == _ffi.ResultCode.Error


def test_free_unknown_ids_do_not_crash(lib, capfd):
    h = _ffi.RTBvh()
    h.id = 123456
    lib.free_bvh(h)
    m = _ffi.RTMbvh()
    m.id = 654321
    lib.free_mbvh(m)
    err = capfd.readouterr().err
    assert "Could not free bvh with id: 123456" in err


def test_python_builder_errors():
    # src/lib.rs:28-64
    with pytest.raises(rb.BuildError) as e:
        rb.Builder(aabbs=None, primitives=rb.Points(np.zeros((0, 3)))).construct_binned_sah()
    assert e.value == rb.BuildError.NoPrimitives()
    with pytest.raises(rb.BuildError) as e:
        rb.Builder(aabbs=np.zeros((0, 8), np.float32), primitives=rb.Points(np.zeros((1, 3)))).construct_binned_sah()
    assert e.value == rb.BuildError.InequalAabbsAndPrimitives(0, 1)
    # construct_spatial_sah (src/bvh.rs:59-85): no primitives first; the
    # builder needs SpatialTriangle primitives
    with pytest.raises(rb.BuildError) as e:
        rb.Builder(primitives=None).construct_spatial_sah()
    assert e.value == rb.BuildError.NoPrimitives()
    with pytest.raises(TypeError):
        rb.Builder(primitives=rb.Points(np.zeros((4, 3)))).construct_spatial_sah()


class _UserData(ctypes.Structure):
    pass


def mt_callback(vertices, origin, direction, t_min=np.float32(1e-5)):
    """The reference FFI test's intersect_test (rtbvh_ffi/src/lib.rs:1027-1060),
    in float32 arithmetic."""
    f32 = np.float32
    o = np.asarray(origin, f32)
    d = np.asarray(direction, f32)

    def cross(a, b):
        return np.array([a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]], f32)

    def dot(a, b):
        return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))

    @_ffi.INTERSECT_FN
    def cb(pid, tptr, _user):
        v0, v1, v2 = (np.asarray(x, f32) for x in vertices[pid])
        e1, e2 = v1 - v0, v2 - v0
        h = cross(d, e2)
        a = dot(e1, h)
        if a > f32(-1e-5) and a < f32(1e-5):
            return False
        f = f32(1.0) / a
        s = o - v0
        u = f * dot(s, h)
        if not (f32(0.0) <= u <= f32(1.0)):
            return False
        q = cross(s, e1)
        v = f * dot(d, q)
        if v < 0 or f32(u + v) > f32(1.0):
            return False
        t = f * dot(e2, q)
        if t > t_min and t < tptr[0]:
            tptr[0] = float(t)
        return False

    return cb


def host_handles(tris):
    """Bvh / Mbvh handles over oracle-built host arrays (no GPU involved)."""
    a = scenes.triangle_aabbs(tris)
    centers = ((a[:, 0:3] + a[:, 4:7]) * np.float32(0.5)).astype(np.float32)
    nodes, idx = oracle.build(a, centers, "sah")
    m = oracle.mbvh(nodes)
    keep = [np.ascontiguousarray(nodes), np.ascontiguousarray(idx), np.ascontiguousarray(m)]
    hb = _ffi.RTBvh()
    hb.node_count = len(nodes)
    hb.nodes = keep[0].ctypes.data_as(ctypes.POINTER(_ffi.RTBvhNode))
    hb.index_count = len(idx)
    hb.indices = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    hm = _ffi.RTMbvh()
    hm.node_count = len(m)
    hm.nodes = keep[2].ctypes.data_as(ctypes.POINTER(_ffi.RTMbvhNode))
    hm.index_count = len(idx)
    hm.indices = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    return hb, hm, keep


def test_host_callback_traversal_quad_hit(lib, golden):
    # rtbvh_ffi/src/lib.rs:945-1019: t == 1 through both intersect and intersect_mbvh
    k = golden["known"]["quad_hit"]
    v = np.asarray(k["vertices"], np.float32).reshape(2, 3, 3)
    hb, hm, keep = host_handles(v)
    o = np.asarray(k["origin"], np.float32)
    d = np.asarray(k["direction"], np.float32)
    cb = mt_callback(v, o, d)
    for fn, h in ((lib.intersect, hb), (lib.intersect_mbvh, hm)):
        t = ctypes.c_float(k["t_in"])
        rc = fn(h, o.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                ctypes.byref(t), None, cb)
        assert rc == _ffi.ResultCode.Ok
        assert abs(t.value - k["t_expected"]) < np.finfo(np.float32).eps


def test_host_callback_traversal_nan(lib, golden):
    v = np.asarray(golden["known"]["quad_hit"]["vertices"], np.float32).reshape(2, 3, 3)
    hb, hm, keep = host_handles(v)
    o = np.asarray([np.nan, 0, 0], np.float32)
    d = np.asarray([0, 0, 1], np.float32)
    cb = mt_callback(v, o, d)
    t = ctypes.c_float(1e26)
    for fn, h in ((lib.intersect, hb), (lib.intersect_mbvh, hm)):
        rc = fn(h, o.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                ctypes.byref(t), None, cb)
        assert rc == _ffi.ResultCode.Nan


def test_host_callback_traversal_matches_oracle_on_teapot(lib, golden):
    tris = golden["teapot"]
    hb, hm, keep = host_handles(tris)
    nodes, idx, m = keep
    rng = np.random.default_rng(0)
    rays = scenes.camera_rays(16, 16, eye=(0.0, 1.5, 8.0), fov_deg=40.0)[rng.permutation(256)[:24]]
    want, _, _ = oracle.trace("mbvh", m, idx, tris.reshape(-1, 9), rays, t_min_tri=1e-5)
    for r in range(len(rays)):
        o, d = rays[r, :3].copy(), rays[r, 3:].copy()
        cb = mt_callback(tris, o, d)
        t = ctypes.c_float(1e34)
        rc = lib.intersect_mbvh(hm, o.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(t), None, cb)
        assert rc == 0
        assert np.float32(t.value) == want[r, 0]


def test_python_flag_constants_equal_the_header():
    """The ctypes layer's flag constants are the values include/rtbvh.h
    defines (RTBVH_TRACE_* and RTBVH_FLAG_NO_HOST_MIRROR)."""
    header = open(os.path.join(os.path.dirname(__file__), "..", "include", "rtbvh.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (RTBVH_\w+) (\d+)u", header)}
    for name in ("ANY_HIT", "STATS", "REORDER", "EXACT_NODES", "WALK_STATS"):
        assert getattr(_ffi, "TRACE_" + name) == defs["RTBVH_TRACE_" + name]
    assert _ffi.FLAG_NO_HOST_MIRROR == defs["RTBVH_FLAG_NO_HOST_MIRROR"]
