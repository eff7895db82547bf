"""Regenerates tests/golden/full_size.json: std::sort digests of every benchmark configuration
at its real size.

The configurations are the benchmark's own (the same generators and the same seed, 20260301,
that bench.py uses on rank 0):

    2^20 uint32 uniform
    2^28 uint32: uniform, sorted, reverse, 16 distinct values, Zipf(1.1) over 2^20 ranks,
                 Gaussian(2^31, 2^28)
    2^27 float32 N(0, 1e3)
    2^26 float64 U[-1e9, 1e9]
    4096 uint32 arrays, lengths log-uniform in [32, 2^20], uniform keys, each sorted on its own

For each one the SHA-256 of the seeded input (which pins the generator on the machine that runs
the check) and of its std::sort output (the reference's verifier, TRUST_BUT_VERIFY,
GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:1120-1138) are recorded; the batched configuration
also gets a digest per segment, so that a failing segment can be named. The arrays are too
large to commit; their digests stand in for them. Takes a few minutes on 8 cores. Run from the
repository root:

    python tests/golden/make_full_size.py
"""
import concurrent.futures as cf
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "gpu-quicksort_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_lib  # noqa: E402
import gqs_ctypes  # noqa: E402
import oracle_ctypes  # noqa: E402

SEED = 20260301  # bench.py's seed (rank 0)
PLAIN = [
    ("u32", "uniform", 20),
    ("u32", "uniform", 28),
    ("u32", "sorted", 28),
    ("u32", "reverse", 28),
    ("u32", "distinct16", 28),
    ("u32", "zipf", 28),
    ("u32", "gaussian", 28),
    ("f32", "gaussian", 27),
    ("f64", "uniform", 26),
]
BATCH = {"dtype": "u32", "dist": "uniform", "segments": 4096, "min_len": 32, "max_len": 1 << 20}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()


def plain_case(dt: str, dist: str, log2n: int) -> dict:
    n = 1 << log2n
    a = gqs_ctypes.generate(dt, dist, SEED, n)
    case = {"kind": "plain", "dtype": dt, "dist": dist, "seed": SEED, "n": n, "input_sha256": sha(a)}
    oracle_ctypes.std_sort(a)
    case["sorted_sha256"] = sha(a)
    case["head"] = a[:4].tobytes().hex()
    case["tail"] = a[-4:].tobytes().hex()
    return case


def batch_case() -> dict:
    off = gqs_ctypes.segment_offsets(SEED, BATCH["segments"], BATCH["min_len"], BATCH["max_len"])
    n = int(off[-1])
    a = gqs_ctypes.generate(BATCH["dtype"], BATCH["dist"], SEED, n)
    case = dict(BATCH, kind="segments", seed=SEED, n=n, offsets_sha256=sha(off.astype(np.uint64)),
                input_sha256=sha(a))
    seg = []
    for i in range(BATCH["segments"]):
        s = a[int(off[i]):int(off[i + 1])]
        oracle_ctypes.std_sort(s)  # a view: sorted in place inside `a`
        seg.append(hashlib.sha256(memoryview(s).cast("B")).hexdigest()[:16])
    case["sorted_sha256"] = sha(a)
    case["segment_sha256_16"] = seg
    return case


def main() -> None:
    build_lib.build()
    oracle_ctypes.load()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        futs = [ex.submit(plain_case, *c) for c in PLAIN] + [ex.submit(batch_case)]
        cases = [f.result() for f in futs]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "full_size.json")
    with open(out, "w") as f:
        json.dump({"generator": "gpu-quicksort_gb300/workload/gqs_workload.cpp", "sorter": "std::sort",
                   "seed": SEED, "cases": cases}, f, indent=1)
    print(len(cases), "cases ->", out)


if __name__ == "__main__":
    main()
