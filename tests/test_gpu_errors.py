"""Argument and device-side error reporting: every failure is a status, never a fault."""
import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu


def test_invalid_host_arguments(gpu_ctx):
    lib = gqs_ctypes.load_library()
    assert lib.gqs_sort_u32(gpu_ctx.h, None, None, 10) == 1
    assert lib.gqs_sort_u32(gpu_ctx.h, None, None, 0) == 0
    a = np.zeros(1, dtype=np.uint32)
    assert lib.gqs_sort_u32(gpu_ctx.h, a.ctypes.data, None, 1) == 0
    off = np.array([0, 10, 5], dtype=np.uint64)
    k = np.zeros(10, dtype=np.uint32)
    assert lib.gqs_sort_segments_u32(gpu_ctx.h, k.ctypes.data, 10, off.ctypes.data, 2) == 1
    off = np.array([0, 11], dtype=np.uint64)
    assert lib.gqs_sort_segments_u32(gpu_ctx.h, k.ctypes.data, 10, off.ctypes.data, 1) == 1


def test_misaligned_device_pointer_rejected(gpu_ctx):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(1024, dtype=torch.int32, device="cuda")
    assert gpu_ctx.sort_dev("u32", buf.data_ptr() + 2, None, 100, 0) == 1
    buf64 = torch.zeros(1024, dtype=torch.float64, device="cuda")
    assert gpu_ctx.sort_dev("f64", buf64.data_ptr() + 4, None, 100, 0) == 1


def test_bad_device_segment_table_reported(gpu_ctx):
    """A decreasing device segment table is caught by the seed kernel and reported."""
    torch = pytest.importorskip("torch")
    keys = torch.arange(1000, 0, -1, dtype=torch.int32, device="cuda")
    off = torch.tensor([0, 600, 400, 1000], dtype=torch.int64, device="cuda")
    rc = gpu_ctx.sort_segments_dev("u32", keys.data_ptr(), None, 1000, off.data_ptr(), 3, 0)
    assert rc == 1
    # the context stays usable
    a = gqs_ctypes.generate("u32", "uniform", 1, 50000)
    b = a.copy()
    gpu_ctx.sort(b)
    assert np.array_equal(b, np.sort(a))
