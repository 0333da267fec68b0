"""ctypes binding of ``librtbvh_gb300.so`` (declarations in include/rtbvh.h).

The library is loaded from the package's ``_lib`` folder. There is no
fallback: if the compiled library is missing or fails to load, every call
raises, so a process can never silently run without the CUDA code.
"""
import ctypes
import enum
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "librtbvh_gb300.so")


class ResultCode(enum.IntEnum):
    """rtbvh_ffi/src/lib.rs:17-25, plus this library's extensions (>= 5)."""
    Ok = 0
    Error = 1
    NoPrimitives = 2
    InequalAabbsAndPrimitives = 3
    Nan = 4
    DeviceError = 5
    Timeout = 6
    StackOverflow = 7
    OutOfMemory = 8
    InvalidArgument = 9


class BvhType(enum.IntEnum):
    """rtbvh_ffi/src/lib.rs:129-133"""
    LocallyOrderedClustered = 0
    BinnedSAH = 1


FLAG_NO_HOST_MIRROR = 1
TRACE_ANY_HIT = 1
TRACE_STATS = 2
TRACE_REORDER = 4
TRACE_EXACT_NODES = 8
TRACE_WALK_STATS = 16

# RTBVH_SPATIAL_FIX_*: corrections of the reference's spatial-split builder.
SPATIAL_FIX_CLIP = 1
SPATIAL_FIX_EXIT_BIN = 2
SPATIAL_FIX_SWEEP_BOX = 4
SPATIAL_FIX_SPLIT_SPACE = 8
SPATIAL_FIX_FALLBACK = 16
SPATIAL_FIX_ALL = 31


class RTAabb(ctypes.Structure):
    _fields_ = [("min", ctypes.c_float * 3), ("count", ctypes.c_int32), ("max", ctypes.c_float * 3),
                ("left_first", ctypes.c_int32)]


class RTBvhNode(ctypes.Structure):
    _fields_ = [("aabb", RTAabb)]


class RTMbvhNode(ctypes.Structure):
    _fields_ = [("min_x", ctypes.c_float * 4), ("max_x", ctypes.c_float * 4), ("min_y", ctypes.c_float * 4),
                ("max_y", ctypes.c_float * 4), ("min_z", ctypes.c_float * 4), ("max_z", ctypes.c_float * 4),
                ("children", ctypes.c_int32 * 4), ("counts", ctypes.c_int32 * 4)]


class RTBvh(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("node_count", ctypes.c_uint32), ("nodes", ctypes.POINTER(RTBvhNode)),
                ("index_count", ctypes.c_uint32), ("indices", ctypes.POINTER(ctypes.c_uint32))]


class RTMbvh(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32), ("node_count", ctypes.c_uint32), ("nodes", ctypes.POINTER(RTMbvhNode)),
                ("index_count", ctypes.c_uint32), ("indices", ctypes.POINTER(ctypes.c_uint32))]


class RTBatch(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint32)]


class RTGpuBatchView(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("node_capacity", ctypes.c_uint32), ("indices", ctypes.c_void_p),
                ("mnodes", ctypes.c_void_p), ("mnode_base", ctypes.c_void_p), ("prim_offsets", ctypes.c_void_p),
                ("mesh_count", ctypes.c_uint32), ("leaf_triangles", ctypes.c_void_p)]


class RTBatchTuning(ctypes.Structure):
    _fields_ = [("trace_blocks_per_sm", ctypes.c_uint32), ("trace_ray_batch", ctypes.c_uint32),
                ("cluster_min_prims", ctypes.c_uint32), ("pipeline_ms", ctypes.c_float),
                ("trace_stack", ctypes.c_uint32)]


class RTGpuView(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("node_count", ctypes.c_uint32),
                ("indices", ctypes.c_void_p), ("index_count", ctypes.c_uint32),
                ("leaf_triangles", ctypes.c_void_p)]


INTERSECT_FN = ctypes.CFUNCTYPE(ctypes.c_bool, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float), ctypes.c_void_p)

# Every symbol include/rtbvh.h declares: name -> (restype, argtypes)
_fp = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u32 = ctypes.c_uint32
_rc = ctypes.c_int
SIGNATURES = {
    "create_spatial_Bvh": (_rc, [ctypes.POINTER(RTAabb), _sz, _fp, _sz, _fp, _sz, _sz, _u32, ctypes.POINTER(RTBvh)]),
    "create_bvh": (_rc, [ctypes.POINTER(RTAabb), _sz, _fp, _sz, _sz, _u32, ctypes.POINTER(RTBvh)]),
    "create_mbvh": (_rc, [RTBvh, ctypes.POINTER(RTMbvh)]),
    "refit": (_rc, [ctypes.POINTER(RTAabb), RTBvh]),
    "intersect": (_rc, [RTBvh, _fp, _fp, _fp, _vp, INTERSECT_FN]),
    "intersect_packet": (_rc, [RTBvh, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _vp, INTERSECT_FN]),
    "intersect_mbvh": (_rc, [RTMbvh, _fp, _fp, _fp, _vp, INTERSECT_FN]),
    "intersect_mbvh_packet": (_rc, [RTMbvh, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _vp, INTERSECT_FN]),
    "free_bvh": (None, [RTBvh]),
    "free_mbvh": (None, [RTMbvh]),
    "rtbvh_gpu_create_bvh_from_triangles": (_rc, [_vp, _sz, _sz, _u32, _u32, _vp, ctypes.POINTER(RTBvh)]),
    "rtbvh_gpu_create_spatial_bvh": (_rc, [_vp, _sz, _vp, _vp, _sz, _sz, _u32, _u32, _vp, ctypes.POINTER(RTBvh)]),
    "rtbvh_gpu_create_bvh": (_rc, [_vp, _sz, _vp, _sz, _sz, _u32, _u32, _vp, ctypes.POINTER(RTBvh)]),
    "rtbvh_gpu_create_mbvh": (_rc, [RTBvh, _u32, _vp, ctypes.POINTER(RTMbvh)]),
    "rtbvh_gpu_set_triangles": (_rc, [_u32, ctypes.c_int, _vp, _sz, _vp]),
    "rtbvh_gpu_intersect_mbvh": (_rc, [RTMbvh, _vp, _vp, _sz, _vp, _u32, _vp, _vp]),
    "rtbvh_gpu_intersect_bvh": (_rc, [RTBvh, _vp, _vp, _sz, _vp, _u32, _vp, _vp]),
    "rtbvh_gpu_intersect_mbvh_packets": (_rc, [RTMbvh, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _u32, _vp,
                                                _vp]),
    "rtbvh_gpu_intersect_bvh_packets": (_rc, [RTBvh, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _u32, _vp,
                                               _vp]),
    "rtbvh_gpu_mbvh_candidates": (_rc, [RTMbvh, _vp, _vp, _sz, _u32, _vp, _vp, _vp]),
    "rtbvh_gpu_bvh_candidates": (_rc, [RTBvh, _vp, _vp, _sz, _u32, _vp, _vp, _vp]),
    "rtbvh_intersect_mbvh_batch": (_rc, [RTMbvh, _vp, _vp, _sz, _vp, _u32]),
    "rtbvh_gpu_status": (_rc, [_u32, ctypes.c_int]),
    "rtbvh_gpu_view": (_rc, [_u32, ctypes.c_int, ctypes.POINTER(RTGpuView)]),
    "rtbvh_gpu_traversal_tree": (_rc, [RTMbvh, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_u32)]),
    "rtbvh_gpu_refit": (_rc, [_u32, _vp, _vp, _u32, _vp]),
    "rtbvh_gpu_refit_mbvh": (_rc, [_u32, _vp, _vp, _vp]),
    "rtbvh_serialize_bvh": (_rc, [RTBvh, _vp, _sz, ctypes.POINTER(_sz)]),
    "rtbvh_deserialize_bvh": (_rc, [_vp, _sz, _u32, _vp, ctypes.POINTER(RTBvh)]),
    "rtbvh_serialize_mbvh": (_rc, [RTMbvh, _vp, _sz, ctypes.POINTER(_sz)]),
    "rtbvh_deserialize_mbvh": (_rc, [_vp, _sz, _u32, _vp, ctypes.POINTER(RTMbvh)]),
    "rtbvh_gpu_refit_noalloc": (_rc, [_u32, _vp, _vp]),
    "rtbvh_gpu_intersect_backward": (_rc, [_vp, _sz, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "rtbvh_gpu_batch_create": (_rc, [_vp, _vp, _u32, _vp, _vp, _vp, _vp, _u32, _vp, ctypes.POINTER(RTBatch)]),
    "rtbvh_gpu_batch_run": (_rc, [RTBatch, _vp]),
    "rtbvh_gpu_batch_run_uncaptured": (_rc, [RTBatch, _vp]),
    "rtbvh_gpu_batch_view": (_rc, [RTBatch, ctypes.POINTER(RTGpuBatchView)]),
    "rtbvh_gpu_batch_status": (_rc, [RTBatch]),
    "rtbvh_gpu_batch_free": (None, [RTBatch]),
    "rtbvh_gpu_batch_tune": (_rc, [RTBatch, _vp, ctypes.POINTER(RTBatchTuning)]),
    "rtbvh_gpu_batch_get_tuning": (_rc, [RTBatch, ctypes.POINTER(RTBatchTuning)]),
    "rtbvh_gpu_batch_set_tuning": (_rc, [RTBatch, ctypes.POINTER(RTBatchTuning), _vp]),
    "rtbvh_gpu_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads (once) and returns the library with every signature bound."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"rtbvh_gb300: compiled library not found at {path}; run rtbvh_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class RtbvhError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = ResultCode(code) if code in ResultCode._value2member_map_ else code
        super().__init__(f"{what}: {self.code!r}" if what else repr(self.code))


def check(code, what=""):
    if code != ResultCode.Ok:
        raise RtbvhError(code, what)
