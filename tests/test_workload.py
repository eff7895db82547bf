"""The seeded workload generators: distribution properties and determinism."""
import math

import numpy as np
import pytest

import gqs_ctypes


def test_deterministic_math_close_to_libm():
    wl = gqs_ctypes.load_workload()
    for x in [1e-300, 1e-9, 0.1, 0.5, 0.999999, 1.0, 2.0, 1234.5, 2.0 ** 20]:
        assert abs(wl.gqs_workload_det_log(x) - math.log(x)) <= 4e-16 * max(1.0, abs(math.log(x)))
    for x in [-700.0, -20.0, -1.1, 0.0, 0.3, 5.0, 14.0]:
        assert abs(wl.gqs_workload_det_exp(x) - math.exp(x)) <= 1e-15 * math.exp(x)
    for u in [0.0, 0.1, 0.25, 0.33, 0.5, 0.77, 0.999]:
        assert abs(wl.gqs_workload_det_cos2pi(u) - math.cos(2 * math.pi * u)) <= 1e-15


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_no_nan_inf_negzero(dtype):
    for dist in ["uniform", "gaussian", "sorted", "reverse", "distinct16"]:
        a = gqs_ctypes.generate(dtype, dist, 1, 200_000)
        if dtype != "u32":
            assert np.all(np.isfinite(a))
            assert not np.any(np.signbit(a) & (a == 0))


def test_distributions_u32():
    n = 1 << 18
    s = gqs_ctypes.generate("u32", "sorted", 1, n)
    assert np.all(s[1:] >= s[:-1])
    r = gqs_ctypes.generate("u32", "reverse", 1, n)
    assert np.all(r[1:] <= r[:-1])
    d = gqs_ctypes.generate("u32", "distinct16", 1, n)
    assert len(np.unique(d)) == 16
    g = gqs_ctypes.generate("u32", "gaussian", 1, n).astype(np.float64)
    assert abs(g.mean() - 2 ** 31) < 2 ** 28 * 0.02
    assert abs(g.std() - 2 ** 28) < 2 ** 28 * 0.02
    z = gqs_ctypes.generate("u32", "zipf", 1, n)
    vals, counts = np.unique(z, return_counts=True)
    assert counts.max() > n // 10  # rank 1 is heavy under s = 1.1
    k = gqs_ctypes.generate("u32", "kat", 1, n)
    assert np.array_equal(np.sort(k), np.arange(1, n + 1, dtype=np.uint32))


def test_float_configs():
    f = gqs_ctypes.generate("f32", "gaussian", 2, 1 << 18).astype(np.float64)
    assert abs(f.std() - 1000.0) < 20.0
    d = gqs_ctypes.generate("f64", "uniform", 2, 1 << 18)
    assert d.min() >= -1e9 and d.max() < 1e9


def test_segment_table_config():
    off = gqs_ctypes.segment_offsets(7, 4096, 32, 1 << 20)
    lens = np.diff(off.astype(np.int64))
    assert off[0] == 0 and np.all(lens >= 32) and np.all(lens <= 1 << 20)
    assert 2 ** 27.5 < off[-1] < 2 ** 29.5


def test_seed_changes_output():
    a = gqs_ctypes.generate("u32", "uniform", 1, 1000)
    b = gqs_ctypes.generate("u32", "uniform", 2, 1000)
    assert not np.array_equal(a, b)
