"""The CPU oracle, pinned before it is trusted.

Pins: the reference's own known-answer test (a shuffled 1..N comes back as out[i] == i + 1,
GPU-Quicksort_OpenCL_1.2/QuicksortMain.cpp:415-416 with the check at 498-516) and its verifier
std::sort (TRUST_BUT_VERIFY) on the committed golden vectors.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import gqs_ctypes
import oracle_ctypes

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]
NP = gqs_ctypes.NP_DTYPES


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
@pytest.mark.parametrize("n", [1, 2, 3, 7, 511, 512, 513, 1023, 1024, 1025, 4096, 100_003, 1 << 20])
def test_known_answer_shuffled_iota(dtype, n):
    """The reference's KAT: shuffled 1..N sorts to 1..N (exact for float up to 2^24)."""
    a = gqs_ctypes.generate(dtype, "kat", 7, n)
    st = oracle_ctypes.gpuqsort(a, threads=1)
    assert np.array_equal(a, np.arange(1, n + 1, dtype=NP[dtype]))
    if n > 1024:
        assert st["levels"] >= 1


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['dtype']}-{c['dist']}-{c['n']}")
def test_golden_vectors(case):
    a = gqs_ctypes.generate(case["dtype"], case["dist"], case["seed"], case["n"])
    assert sha(a) == case["input_sha256"], "generator drifted from the committed vector"
    b = a.copy()
    oracle_ctypes.std_sort(b)
    assert sha(b) == case["sorted_sha256"]
    c = a.copy()
    oracle_ctypes.gpuqsort(c, threads=4)
    assert sha(c) == case["sorted_sha256"], "GPUQSort restatement differs from std::sort"


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_restatement_threads_agree(dtype):
    a = gqs_ctypes.generate(dtype, "uniform" if dtype != "f32" else "gaussian", 11, 300_001)
    x, y = a.copy(), a.copy()
    s1 = oracle_ctypes.gpuqsort(x, threads=1)
    s8 = oracle_ctypes.gpuqsort(y, threads=8)
    # Block reservation order (the reference's atomics) moves keys inside children, so the
    # level count may differ between runs; the sorted output may not.
    assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
    assert s1["levels"] > 0 and s8["levels"] > 0


def test_level_structure_matches_reference_rules():
    """MAXSEQ follows optp (QuicksortMain.cpp:831-833): 256 at 2^20."""
    a = gqs_ctypes.generate("u32", "uniform", 3, 1 << 20)
    st = oracle_ctypes.gpuqsort(a, threads=8)
    assert st["maxseq"] == 256
    assert 15 <= st["levels"] <= 40
    assert st["active_keys"] > 8 * (1 << 20)


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_reference_cpu_quicksort(dtype):
    a = gqs_ctypes.generate(dtype, "uniform", 5, 200_000)
    b, c = a.copy(), a.copy()
    oracle_ctypes.cpu_quicksort(b)
    oracle_ctypes.std_sort(c)
    assert np.array_equal(b, c)


def test_parallel_sort_matches():
    a = gqs_ctypes.generate("u32", "zipf", 5, 500_000)
    b, c = a.copy(), a.copy()
    oracle_ctypes.parallel_sort(b, 4)
    oracle_ctypes.std_sort(c)
    assert np.array_equal(b, c)


def test_segmented_restatement():
    off = gqs_ctypes.segment_offsets(9, 200, 1, 5000)
    a = gqs_ctypes.generate("u32", "uniform", 9, int(off[-1]))
    b = a.copy()
    oracle_ctypes.gpuqsort_segments_u32(b, off, threads=4)
    for i in range(len(off) - 1):
        s, e = int(off[i]), int(off[i + 1])
        assert np.array_equal(b[s:e], np.sort(a[s:e]))


def test_negative_and_fractional_floats():
    """The restatement compares in T; the Full-SYCL network's `uint av, bv` would truncate these."""
    a = np.array([-1.5, 2.25, -0.75, 0.5, -1e9, 1e9, 3.0, -3.0] * 200, dtype=np.float64)
    b = a.copy()
    oracle_ctypes.gpuqsort(b)
    assert np.array_equal(b, np.sort(a))
