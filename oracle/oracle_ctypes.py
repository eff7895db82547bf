"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle (oracle/_build/liboracle.so).

Loaded by the tests, by __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline
leg. The product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None

_TAG = {np.dtype(np.uint32): "u32", np.dtype(np.float32): "f32", np.dtype(np.float64): "f64"}


class OracleStats(C.Structure):
    _fields_ = [("levels", C.c_uint64), ("active_keys", C.c_uint64), ("blocks", C.c_uint64),
                ("done_records", C.c_uint64), ("maxseq", C.c_uint64)]


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(HERE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    lib = C.CDLL(path)
    vp, sz = C.c_void_p, C.c_size_t
    for t in ("u32", "f32", "f64"):
        f = getattr(lib, f"oracle_gpuqsort_{t}")
        f.argtypes = [vp, vp, sz, C.c_int, C.POINTER(OracleStats)]
        f.restype = C.c_int
        for name in ("oracle_std_sort_", "oracle_cpu_quicksort_"):
            g = getattr(lib, name + t)
            g.argtypes = [vp, sz]
            g.restype = None
        g = getattr(lib, f"oracle_parallel_sort_{t}")
        g.argtypes = [vp, sz, C.c_int]
        g.restype = None
    lib.oracle_gpuqsort_segments_u32.argtypes = [vp, vp, vp, sz, C.c_int]
    lib.oracle_gpuqsort_segments_u32.restype = C.c_int
    _lib = lib
    return lib


def _tag(a: np.ndarray) -> str:
    assert a.flags.c_contiguous
    return _TAG[a.dtype]


def gpuqsort(a: np.ndarray, threads: int = 1) -> dict:
    """The reference's GPUQSort<T> restated on the CPU; sorts `a` in place."""
    lib = load()
    dn = np.empty_like(a)
    st = OracleStats()
    rc = getattr(lib, f"oracle_gpuqsort_{_tag(a)}")(a.ctypes.data, dn.ctypes.data, a.size, threads, C.byref(st))
    if rc != 0:
        raise ValueError("oracle_gpuqsort rejected the input")
    return {k: getattr(st, k) for k, _ in OracleStats._fields_}


def std_sort(a: np.ndarray) -> None:
    getattr(load(), f"oracle_std_sort_{_tag(a)}")(a.ctypes.data, a.size)


def parallel_sort(a: np.ndarray, threads: int) -> None:
    getattr(load(), f"oracle_parallel_sort_{_tag(a)}")(a.ctypes.data, a.size, threads)


def cpu_quicksort(a: np.ndarray) -> None:
    getattr(load(), f"oracle_cpu_quicksort_{_tag(a)}")(a.ctypes.data, a.size)


def gpuqsort_segments_u32(a: np.ndarray, offsets: np.ndarray, threads: int = 1) -> None:
    assert a.dtype == np.uint32
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    dn = np.empty_like(a)
    rc = load().oracle_gpuqsort_segments_u32(a.ctypes.data, dn.ctypes.data, off.ctypes.data, off.size - 1, threads)
    if rc != 0:
        raise ValueError("oracle rejected a segment")
