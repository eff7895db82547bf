"""The full-size std::sort digests (tests/golden/full_size.json) against this machine (no GPU).

The digests stand in for arrays too large to commit. Here the seeded inputs of every
configuration are regenerated and must hash as recorded (the generator is the same on every
machine), and the smallest configuration is sorted again by std::sort and by the oracle's
restatement of GPUQSort<T>, whose digests must both equal the recorded output digest.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import gqs_ctypes
import oracle_ctypes

FULL_SIZE = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "full_size.json")))


def sha(a):
    return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()


@pytest.mark.parametrize("case", FULL_SIZE["cases"], ids=lambda c: f"{c['kind']}-{c['dtype']}-{c['dist']}-{c['n']}")
def test_inputs_hash_as_recorded(case):
    if case["kind"] == "segments":
        off = gqs_ctypes.segment_offsets(case["seed"], case["segments"], case["min_len"], case["max_len"])
        assert sha(off.astype(np.uint64)) == case["offsets_sha256"]
        assert int(off[-1]) == case["n"]
        assert len(case["segment_sha256_16"]) == case["segments"]
    a = gqs_ctypes.generate(case["dtype"], case["dist"], case["seed"], case["n"])
    assert sha(a) == case["input_sha256"]


def test_smallest_configuration_sorts_to_the_recorded_digest():
    case = next(c for c in FULL_SIZE["cases"] if c["kind"] == "plain" and c["n"] == 1 << 20)
    a = gqs_ctypes.generate(case["dtype"], case["dist"], case["seed"], case["n"])
    s = a.copy()
    oracle_ctypes.std_sort(s)
    assert sha(s) == case["sorted_sha256"]
    r = a.copy()
    oracle_ctypes.gpuqsort(r, threads=4)
    assert sha(r) == case["sorted_sha256"]
    assert s[:4].tobytes().hex() == case["head"] and s[-4:].tobytes().hex() == case["tail"]
