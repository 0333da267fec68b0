"""rtbvh_gb300 -- GB300-native BVH construction and ray traversal.

A drop-in for the BVH build + single-ray traversal path of meirbon/rtbvh:
the reference's C ABI (include/rtbvh.h, librtbvh_gb300.so) and a Python
mirror of its Builder / Bvh / Mbvh API, with every build and traversal
running as hand-written CUDA kernels for sm_103a.
"""
from ._ffi import BvhType, ResultCode, RtbvhError, load as load_library  # noqa: F401
from .api import (Batch, BuildError, BuildType, Builder, Bvh, Mbvh, Points, Triangles,  # noqa: F401
                  device_copy, hit_prims)

__all__ = ["Builder", "Bvh", "Mbvh", "Batch", "Triangles", "Points", "BuildError", "BuildType", "BvhType",
           "ResultCode", "RtbvhError", "hit_prims", "load_library"]
