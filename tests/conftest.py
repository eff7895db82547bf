"""Test configuration: the `gpu` marker, import paths, and in-tree builds.

`-m "not gpu"` tests need no GPU: the oracle against the reference's known-answer test and the
golden vectors, the workload generators, and the C ABI library's exports. `-m gpu` tests call
the CUDA sort through the C ABI and compare with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-quicksort_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    import build_lib  # gpu-quicksort_gb300/build_lib.py
    build_lib.build()
    import oracle_ctypes
    oracle_ctypes.load()
    yield


@pytest.fixture(scope="session")
def gpu_ctx():
    import gqs_ctypes
    ctx = gqs_ctypes.Context(device=0, sync=True, timing=True, timeout_ms=4000)
    yield ctx
    ctx.close()
