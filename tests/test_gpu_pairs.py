"""GPU parity for the key-value sorts (gqs_sort_pairs_*): keys sorted with their values; pairs
with equal keys in ascending value order, so values 0..n-1 give numpy's stable argsort."""
import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 2, 3, 255, 256, 257, 4097, 65537, 1 << 20, (1 << 22) + 3]


@pytest.mark.parametrize("n", SIZES)
def test_u32_pairs_match_lexicographic_sort(gpu_ctx, n):
    keys = gqs_ctypes.generate("u32", "uniform", 90 + n, max(n, 1))[:n].copy()
    vals = gqs_ctypes.generate("u32", "uniform", 91 + n, max(n, 1))[:n].copy()
    order = np.lexsort((vals, keys))
    k, v = keys.copy(), vals.copy()
    gpu_ctx.sort_pairs(k, v)
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


@pytest.mark.parametrize("dtype,dist", [("u32", "distinct16"), ("u32", "zipf"), ("f32", "gaussian"),
                                        ("f32", "distinct16"), ("u32", "allequal"), ("u32", "sorted"),
                                        ("f32", "reverse")])
def test_argsort_is_stable(gpu_ctx, dtype, dist):
    keys = gqs_ctypes.generate(dtype, dist, 77, 3 * (1 << 18) + 11)
    idx = gpu_ctx.argsort(keys)
    assert np.array_equal(idx, np.argsort(keys, kind="stable").astype(np.uint32))


def test_float_pairs_keep_key_bits(gpu_ctx):
    keys = gqs_ctypes.generate("f32", "gaussian", 5, 1 << 20)
    vals = np.arange(keys.size, dtype=np.uint32)[::-1].copy()
    k, v = keys.copy(), vals.copy()
    gpu_ctx.sort_pairs(k, v)
    order = np.lexsort((vals, keys))
    assert np.array_equal(k.view(np.uint32), keys[order].view(np.uint32))
    assert np.array_equal(v, vals[order])


@pytest.mark.parametrize("dtype", ["u32", "f32"])
def test_device_pairs(gpu_ctx, dtype):
    torch = pytest.importorskip("torch")
    n = (1 << 23) + 5
    keys = gqs_ctypes.generate(dtype, "uniform" if dtype == "u32" else "gaussian", 8, n)
    vals = np.arange(n, dtype=np.uint32)
    tk = torch.from_numpy(keys.view(np.int32)).cuda()
    tv = torch.from_numpy(vals.view(np.int32)).cuda()
    s = torch.cuda.current_stream()
    assert gpu_ctx.sort_pairs_dev(dtype, tk.data_ptr(), tv.data_ptr(), n, s.cuda_stream) == 0
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(tk.cpu().numpy().view(keys.dtype).view(np.uint32), keys[order].view(np.uint32))
    assert np.array_equal(tv.cpu().numpy().view(np.uint32), order.astype(np.uint32))
    st = gpu_ctx.stats()
    assert st["status"] == 0 and st["keys"] == n
