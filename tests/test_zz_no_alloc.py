"""The allocation-free refit entry point, rtbvh_gpu_refit_noalloc, called
through the C ABI and checked against the regular rtbvh_gpu_refit.

It exists for callers that cannot allocate device memory while they run --
for example a per-frame animation loop that refits its BVH and must not call
cudaMalloc, which can synchronise the device or fail mid-frame. Its results
must equal the regular refit's bit for bit. Two refits in a row check that
the scratch array it shares between calls is reset properly."""
import ctypes

import numpy as np
import pytest
import torch

from rtbvh_gb300 import _ffi, scenes
from gpu_helpers import gpu_build, to_cuda, u32

pytestmark = pytest.mark.gpu


class _DeviceArray:
    """Zero-copy view of library-owned device memory for torch."""

    def __init__(self, ptr, shape, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3}


def device_nodes(lib, bvh):
    view = _ffi.RTGpuView()
    assert lib.rtbvh_gpu_view(bvh.handle.id, 0, ctypes.byref(view)) == 0
    t = torch.as_tensor(_DeviceArray(view.nodes, (view.node_count, 8)), device="cuda")
    return t.clone().cpu().numpy()


def test_refit_noalloc_matches_refit_twice_in_a_row(lib):
    torch.cuda.set_device(0)
    tris = scenes.incoherent(20000, seed=41)
    a = gpu_build(tris, "locb")
    b = gpu_build(tris, "locb")
    assert np.array_equal(u32(device_nodes(lib, a)), u32(device_nodes(lib, b)))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(5)
    for step in range(2):
        moved = (tris + rng.normal(scale=2e-3, size=tris.shape)).astype(np.float32)
        d_aabbs = to_cuda(scenes.triangle_aabbs(moved))
        ptr = ctypes.c_void_p(d_aabbs.data_ptr())
        assert lib.rtbvh_gpu_refit(a.handle.id, None, ptr, 0xFFFFFFFF, stream) == 0
        assert lib.rtbvh_gpu_refit_noalloc(b.handle.id, ptr, stream) == 0
        torch.cuda.synchronize()
        na, nb = device_nodes(lib, a), device_nodes(lib, b)
        assert np.array_equal(u32(na), u32(nb)), f"refit {step}: no-alloc result differs"
        assert not np.array_equal(u32(na), u32(device_nodes(lib, gpu_build(tris, "locb"))))


def test_refit_noalloc_rejects_trees_over_the_limit(lib):
    torch.cuda.set_device(0)
    n = 600_000  # 1,199,999 nodes > RTBVH_REFIT_NOALLOC_MAX_NODES
    tris = scenes.incoherent(n, seed=42)
    big = gpu_build(tris, "locb")
    before = device_nodes(lib, big)
    d_aabbs = to_cuda(scenes.triangle_aabbs(tris * np.float32(1.01)))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.rtbvh_gpu_refit_noalloc(big.handle.id, ctypes.c_void_p(d_aabbs.data_ptr()), stream)
    assert rc == _ffi.ResultCode.InvalidArgument
    torch.cuda.synchronize()
    assert np.array_equal(u32(device_nodes(lib, big)), u32(before))


def test_refit_noalloc_reports_bad_leaf_ranges_in_the_status(lib):
    """A leaf whose index range runs past the Bvh's index slots is skipped by
    the kernel's bounds checks, and the error shows up in rtbvh_gpu_status
    for that Bvh; a repaired tree refits cleanly again."""
    torch.cuda.set_device(0)
    tris = scenes.incoherent(5000, seed=43)
    bvh = gpu_build(tris, "locb")
    view = _ffi.RTGpuView()
    assert lib.rtbvh_gpu_view(bvh.handle.id, 0, ctypes.byref(view)) == 0
    nodes = torch.as_tensor(_DeviceArray(view.nodes, (view.node_count, 8)), device="cuda")
    ints = nodes.view(torch.int32)
    leaf = int(torch.nonzero(ints[:, 3] >= 0)[0])
    good = int(ints[leaf, 7])
    ints[leaf, 7] = view.index_count + 5  # host-side damage of the device tree: a leaf past the index slots
    torch.cuda.synchronize()
    d_aabbs = to_cuda(scenes.triangle_aabbs(tris))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.rtbvh_gpu_status(bvh.handle.id, 0) == _ffi.ResultCode.Ok
    assert lib.rtbvh_gpu_refit_noalloc(bvh.handle.id, ctypes.c_void_p(d_aabbs.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    assert lib.rtbvh_gpu_status(bvh.handle.id, 0) == _ffi.ResultCode.Error
    ints[leaf, 7] = good
    torch.cuda.synchronize()
    assert lib.rtbvh_gpu_refit_noalloc(bvh.handle.id, ctypes.c_void_p(d_aabbs.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    assert lib.rtbvh_gpu_status(bvh.handle.id, 0) == _ffi.ResultCode.Ok


def test_refit_noalloc_leaves_free_device_memory_unchanged(lib):
    """After a first call (which may load the library's code on the device),
    further calls take no device memory: the device's free memory is the same
    before and after them."""
    torch.cuda.set_device(0)
    tris = scenes.incoherent(20000, seed=44)
    bvh = gpu_build(tris, "locb")
    d_aabbs = to_cuda(scenes.triangle_aabbs(tris))
    ptr = ctypes.c_void_p(d_aabbs.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.rtbvh_gpu_refit_noalloc(bvh.handle.id, ptr, stream) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        assert lib.rtbvh_gpu_refit_noalloc(bvh.handle.id, ptr, stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert lib.rtbvh_gpu_status(bvh.handle.id, 0) == _ffi.ResultCode.Ok
