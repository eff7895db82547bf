"""GPU parity for the segmented (batched) sort: every segment equals its own std::sort."""
import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu


def check_segments(a, b, off):
    for i in range(len(off) - 1):
        s, e = int(off[i]), int(off[i + 1])
        assert np.array_equal(b[s:e], np.sort(a[s:e])), (i, s, e)


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_many_small_segments(gpu_ctx, dtype):
    off = gqs_ctypes.segment_offsets(21, 3000, 1, 3000)
    a = gqs_ctypes.generate(dtype, "uniform" if dtype != "f32" else "gaussian", 21, int(off[-1]))
    b = a.copy()
    gpu_ctx.sort_segments(b, off)
    check_segments(a, b, off)


def test_log_uniform_batch(gpu_ctx):
    off = gqs_ctypes.segment_offsets(22, 512, 32, 1 << 20)
    a = gqs_ctypes.generate("u32", "uniform", 22, int(off[-1]))
    b = a.copy()
    gpu_ctx.sort_segments(b, off)
    check_segments(a, b, off)


def test_empty_and_unit_segments(gpu_ctx):
    off = np.array([0, 0, 1, 1, 5, 5, 300, 300, 20000, 20001], dtype=np.uint64)
    a = gqs_ctypes.generate("u32", "distinct16", 23, 20001)
    b = a.copy()
    gpu_ctx.sort_segments(b, off)
    check_segments(a, b, off)


def test_segments_leave_gaps_untouched(gpu_ctx):
    """Keys outside [offsets[0], offsets[nseg]) are not part of any segment and stay put."""
    off = np.array([100, 5000, 90000], dtype=np.uint64)
    a = gqs_ctypes.generate("u32", "uniform", 24, 100000)
    b = a.copy()
    gpu_ctx.sort_segments(b, off)
    assert np.array_equal(b[:100], a[:100]) and np.array_equal(b[90000:], a[90000:])
    check_segments(a, b, off)
