"""gqs_sort_u32_noalloc: the sort for callers that cannot allocate device memory when they sort.

Such callers (hosts whose device memory all belongs to their own pool, latency-critical code
that cannot take cudaMalloc's implicit synchronisation) cannot create a gqs_ctx either, so this
entry point takes none and keeps its scratch in a static device array inside the library. The
test checks its output against the context-based gqs_sort_u32_dev, bit for bit, on two calls in
a row (the second call reuses the array the first one left behind), and that sizes beyond the
array are refused before any work. It is collected last so a stopping run has run everything
else first; it needs no earlier test and works in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20  # GQS_NOALLOC_MAX_KEYS in include/gqs.h


def test_noalloc_matches_context_sort_twice():
    torch = pytest.importorskip("torch")
    lib = gqs_ctypes.load_library()
    stream = torch.cuda.current_stream().cuda_stream
    ctx = gqs_ctypes.Context(device=0)
    try:
        for call, (dist, n, seed) in enumerate((("uniform", MAX_KEYS, 101), ("zipf", 777_777, 202))):
            a = gqs_ctypes.generate("u32", dist, seed, n)
            mine = torch.from_numpy(a.view(np.int32)).cuda()
            theirs = mine.clone()
            torch.cuda.synchronize()
            assert lib.gqs_sort_u32_noalloc(ctypes.c_void_p(mine.data_ptr()), n, ctypes.c_void_p(stream)) == 0, call
            assert ctx.sort_dev("u32", theirs.data_ptr(), None, n, stream) == 0, call
            torch.cuda.synchronize()
            assert torch.equal(mine, theirs), f"call {call}: differs from gqs_sort_u32_dev"
            assert np.array_equal(mine.cpu().numpy().view(np.uint32), np.sort(a)), call
    finally:
        ctx.close()


def test_noalloc_refuses_more_than_its_scratch():
    torch = pytest.importorskip("torch")
    lib = gqs_ctypes.load_library()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    # n is checked before the pointer is used, so a small buffer is safe here
    assert lib.gqs_sort_u32_noalloc(ctypes.c_void_p(buf.data_ptr()), MAX_KEYS + 1, None) == 1
    assert lib.gqs_sort_u32_noalloc(None, 0, None) == 0


def test_noalloc_refuses_null_and_misaligned_pointers():
    torch = pytest.importorskip("torch")
    lib = gqs_ctypes.load_library()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    # both are refused by the argument checks, before the device is touched
    assert lib.gqs_sort_u32_noalloc(None, 2, None) == 1
    assert lib.gqs_sort_u32_noalloc(ctypes.c_void_p(buf.data_ptr() + 2), 2, None) == 1
