"""Regenerates tests/golden/golden.json.

For every key type and configured distribution, at a few sizes, records the SHA-256 of the
seeded input (pins the generators across x86-64 and AArch64) and of its std::sort output
(the reference's verifier, TRUST_BUT_VERIFY, GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:1120-1138),
plus the first and last sorted keys. Run from the repository root:

    python tests/golden/make_golden.py
"""
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

SEED = 20260101
SIZES = [1, 2, 3, 1000, 65537, 1 << 20]
DISTS = {
    "u32": ["uniform", "sorted", "reverse", "distinct16", "zipf", "gaussian", "kat", "allequal"],
    "f32": ["gaussian", "uniform", "sorted", "reverse", "distinct16", "kat", "allequal"],
    "f64": ["uniform", "gaussian", "sorted", "reverse", "distinct16", "kat", "allequal"],
}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    build_lib.build()
    cases = []
    for dt, dists in DISTS.items():
        for dist in dists:
            for n in SIZES:
                a = gqs_ctypes.generate(dt, dist, SEED, n)
                s = a.copy()
                oracle_ctypes.std_sort(s)
                cases.append({
                    "dtype": dt, "dist": dist, "seed": SEED, "n": n,
                    "input_sha256": sha(a), "sorted_sha256": sha(s),
                    "head": [s[: min(4, n)].tobytes().hex()], "tail": [s[-min(4, n):].tobytes().hex()],
                })
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json"), "w") as f:
        json.dump({"generator": "gpu-quicksort_gb300/workload/gqs_workload.cpp", "sorter": "std::sort",
                   "cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
