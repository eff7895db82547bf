"""ctypes binding of the gqs C ABI (include/gqs.h) and of the workload generators.

This is the binding a Python caller of the reference's GPUQSort<T> path would add: one
`ctypes.CDLL` over libgqs.so with the argument types declared once. The library is required;
there is no CPU fallback, and a missing build raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgqs.so")
WORKLOAD_PATH = os.path.join(HERE, "libgqs_workload.so")

DTYPES = {"u32": 0, "f32": 1, "f64": 2}
NP_DTYPES = {"u32": np.uint32, "f32": np.float32, "f64": np.float64}
DIST = {"uniform": 0, "sorted": 1, "reverse": 2, "distinct16": 3, "zipf": 4, "gaussian": 5, "kat": 6,
        "allequal": 7}

STATUS = {0: "GQS_OK", 1: "GQS_ERR_INVALID", 2: "GQS_ERR_CUDA", 3: "GQS_ERR_NOMEM", 4: "GQS_ERR_TIMEOUT",
          5: "GQS_ERR_CAPACITY", 6: "GQS_ERR_NO_DEVICE", 7: "GQS_ERR_INTERNAL", 8: "GQS_ERR_CANCELLED",
          9: "GQS_ERR_BOUNDS"}

# Every function include/gqs.h declares.
EXPORTS = [
    "gqs_config_default", "gqs_create", "gqs_destroy", "gqs_reserve",
    "gqs_sort_u32", "gqs_sort_f32", "gqs_sort_f64",
    "gqs_sort_u32_dev", "gqs_sort_f32_dev", "gqs_sort_f64_dev",
    "gqs_sort_segments_u32_dev", "gqs_sort_segments_f32_dev", "gqs_sort_segments_f64_dev",
    "gqs_sort_segments_u32", "gqs_sort_segments_f32", "gqs_sort_segments_f64",
    "gqs_sort_u32_noalloc", "gqs_sync", "gqs_last_stats", "gqs_last_profile", "gqs_last_levels",
    "gqs_last_phases", "gqs_variant_count", "gqs_variant_describe", "gqs_set_variant",
    "gqs_get_variant", "gqs_strerror", "gqs_version",
    "gqs_batch_create", "gqs_batch_destroy", "gqs_batch_keys", "gqs_batch_offsets", "gqs_batch_launch",
    "gqs_batch_wait", "gqs_batch_copy_in", "gqs_batch_copy_out", "gqs_batch_set_variant", "gqs_batch_get_variant", "gqs_batch_autotune",
    "gqs_srv_config_default", "gqs_srv_create", "gqs_srv_destroy", "gqs_srv_submit", "gqs_srv_wait",
    "gqs_srv_wait_any", "gqs_srv_cancel", "gqs_srv_drain", "gqs_srv_stats", "gqs_srv_now_ns",
    "gqs_selftest_stalled_queue",
    "gqs_selftest_bounds",
    "gqs_sort_pairs_u32", "gqs_sort_pairs_f32", "gqs_sort_pairs_u32_dev", "gqs_sort_pairs_f32_dev",
]


class GqsError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {STATUS.get(code, code)}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("variant", C.c_int32), ("timeout_ms", C.c_uint32), ("sync", C.c_uint32),
                ("timing", C.c_uint32), ("reserved", C.c_uint32 * 4)]


class Stats(C.Structure):
    _fields_ = [("keys", C.c_uint64), ("part_keys", C.c_uint64), ("local_keys", C.c_uint64),
                ("tiny_keys", C.c_uint64), ("fill_keys", C.c_uint64), ("chunks", C.c_uint64),
                ("algo_bytes", C.c_uint64), ("part_jobs", C.c_uint32), ("local_jobs", C.c_uint32),
                ("fill_chunks", C.c_uint32), ("max_depth", C.c_uint32), ("status", C.c_uint32),
                ("variant", C.c_uint32), ("grid", C.c_uint32), ("threads", C.c_uint32),
                ("kernel_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Level(C.Structure):
    _fields_ = [("depth", C.c_uint32), ("part_jobs", C.c_uint32), ("part_keys", C.c_uint64),
                ("local_jobs", C.c_uint32), ("reserved", C.c_uint32), ("local_keys", C.c_uint64),
                ("first_ms", C.c_double), ("last_ms", C.c_double)]


class Phases(C.Structure):
    _fields_ = [("partition_cycles", C.c_uint64), ("onchip_cycles", C.c_uint64), ("fill_cycles", C.c_uint64),
                ("total_cycles", C.c_uint64)]


class VariantDesc(C.Structure):
    _fields_ = [("threads", C.c_int32), ("tile", C.c_int32), ("chunk", C.c_int32), ("kpt", C.c_int32),
                ("stages", C.c_int32), ("tiny", C.c_int32), ("smem_bytes", C.c_uint64), ("name", C.c_char * 64)]


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("batch_keys", C.c_uint64), ("batch_segments", C.c_uint32),
                ("lanes", C.c_uint32), ("timeout_ms", C.c_uint32), ("per_request", C.c_uint32),
                ("variant", C.c_int32 * 3), ("reserved", C.c_uint32 * 4)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_uint32), ("dtype", C.c_uint32), ("n", C.c_uint64), ("t_submit_ns", C.c_uint64),
                ("t_admit_ns", C.c_uint64), ("t_launch_ns", C.c_uint64), ("t_done_ns", C.c_uint64),
                ("batch_requests", C.c_uint32), ("lane", C.c_uint32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "failed", "cancelled", "completed_keys", "batches",
                                          "max_batch_requests", "arena_bytes", "arena_used", "arena_peak",
                                          "pending", "outstanding")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
_wl = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libgqs.so and declares its signatures (raises if it was never built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or os.environ.get("GQS_LIB") or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: build it with __graft_entry__.build() "
                                "(the sort has no CPU fallback)")
    lib = C.CDLL(p)
    vp, sz, st = C.c_void_p, C.c_size_t, C.c_int
    lib.gqs_config_default.argtypes = [C.POINTER(Config)]
    lib.gqs_config_default.restype = None
    lib.gqs_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(Config)]
    lib.gqs_create.restype = st
    lib.gqs_destroy.argtypes = [vp]
    lib.gqs_destroy.restype = None
    lib.gqs_reserve.argtypes = [vp, C.c_int, sz, sz, C.c_int]
    lib.gqs_reserve.restype = st
    for t in ("u32", "f32", "f64"):
        f = getattr(lib, f"gqs_sort_{t}")
        f.argtypes = [vp, vp, vp, sz]
        f.restype = st
        f = getattr(lib, f"gqs_sort_{t}_dev")
        f.argtypes = [vp, vp, vp, sz, vp]
        f.restype = st
        f = getattr(lib, f"gqs_sort_segments_{t}_dev")
        f.argtypes = [vp, vp, vp, sz, vp, sz, vp]
        f.restype = st
        f = getattr(lib, f"gqs_sort_segments_{t}")
        f.argtypes = [vp, vp, sz, vp, sz]
        f.restype = st
    for t in ("u32", "f32"):
        f = getattr(lib, f"gqs_sort_pairs_{t}")
        f.argtypes = [vp, vp, vp, sz]
        f.restype = st
        f = getattr(lib, f"gqs_sort_pairs_{t}_dev")
        f.argtypes = [vp, vp, vp, sz, vp]
        f.restype = st
    lib.gqs_sort_u32_noalloc.argtypes = [vp, sz, vp]
    lib.gqs_sort_u32_noalloc.restype = st
    lib.gqs_sync.argtypes = [vp]
    lib.gqs_sync.restype = st
    lib.gqs_last_stats.argtypes = [vp, C.POINTER(Stats)]
    lib.gqs_last_stats.restype = st
    lib.gqs_last_profile.argtypes = [vp, C.POINTER(C.c_uint64), sz]
    lib.gqs_last_profile.restype = C.c_int
    lib.gqs_last_levels.argtypes = [vp, C.POINTER(Level), C.c_int]
    lib.gqs_last_levels.restype = C.c_int
    lib.gqs_last_phases.argtypes = [vp, C.POINTER(Phases)]
    lib.gqs_last_phases.restype = st
    lib.gqs_variant_count.argtypes = [C.c_int]
    lib.gqs_variant_count.restype = C.c_int
    lib.gqs_variant_describe.argtypes = [C.c_int, C.c_int, C.POINTER(VariantDesc)]
    lib.gqs_variant_describe.restype = st
    lib.gqs_set_variant.argtypes = [vp, C.c_int, C.c_int]
    lib.gqs_set_variant.restype = st
    lib.gqs_get_variant.argtypes = [vp, C.c_int]
    lib.gqs_get_variant.restype = C.c_int
    lib.gqs_strerror.argtypes = [C.c_int]
    lib.gqs_strerror.restype = C.c_char_p
    lib.gqs_version.argtypes = []
    lib.gqs_version.restype = C.c_int
    lib.gqs_batch_create.argtypes = [C.c_int, C.c_int, sz, sz, C.POINTER(Config), C.POINTER(vp)]
    lib.gqs_batch_create.restype = st
    lib.gqs_batch_destroy.argtypes = [vp]
    lib.gqs_batch_destroy.restype = None
    lib.gqs_batch_keys.argtypes = [vp]
    lib.gqs_batch_keys.restype = vp
    lib.gqs_batch_offsets.argtypes = [vp]
    lib.gqs_batch_offsets.restype = C.POINTER(C.c_uint64)
    lib.gqs_batch_launch.argtypes = [vp, sz, vp]
    lib.gqs_batch_launch.restype = st
    lib.gqs_batch_wait.argtypes = [vp, C.POINTER(Stats)]
    lib.gqs_batch_wait.restype = st
    lib.gqs_batch_copy_in.argtypes = [vp, vp, sz, sz]
    lib.gqs_batch_copy_in.restype = st
    lib.gqs_batch_copy_out.argtypes = [vp, vp, sz, sz]
    lib.gqs_batch_copy_out.restype = st
    lib.gqs_batch_set_variant.argtypes = [vp, C.c_int]
    lib.gqs_batch_set_variant.restype = st
    lib.gqs_batch_get_variant.argtypes = [vp]
    lib.gqs_batch_get_variant.restype = C.c_int
    lib.gqs_batch_autotune.argtypes = [vp, sz, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)]
    lib.gqs_batch_autotune.restype = st
    lib.gqs_srv_config_default.argtypes = [C.POINTER(ServerConfig)]
    lib.gqs_srv_config_default.restype = None
    lib.gqs_srv_create.argtypes = [C.c_int, C.POINTER(ServerConfig), C.POINTER(vp)]
    lib.gqs_srv_create.restype = st
    lib.gqs_srv_destroy.argtypes = [vp]
    lib.gqs_srv_destroy.restype = None
    lib.gqs_srv_submit.argtypes = [vp, C.c_int, vp, vp, sz, C.POINTER(C.c_uint64)]
    lib.gqs_srv_submit.restype = st
    lib.gqs_srv_wait.argtypes = [vp, C.c_uint64, C.POINTER(RequestInfo)]
    lib.gqs_srv_wait.restype = st
    lib.gqs_srv_wait_any.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(RequestInfo), C.c_uint32]
    lib.gqs_srv_wait_any.restype = st
    lib.gqs_srv_cancel.argtypes = [vp, C.c_uint64]
    lib.gqs_srv_cancel.restype = st
    lib.gqs_selftest_stalled_queue.argtypes = [vp, C.c_int, C.c_uint32]
    lib.gqs_selftest_stalled_queue.restype = st
    lib.gqs_selftest_bounds.argtypes = [vp, C.c_int]
    lib.gqs_selftest_bounds.restype = st
    lib.gqs_srv_drain.argtypes = [vp]
    lib.gqs_srv_drain.restype = st
    lib.gqs_srv_stats.argtypes = [vp, C.POINTER(ServerStats)]
    lib.gqs_srv_stats.restype = st
    lib.gqs_srv_now_ns.argtypes = []
    lib.gqs_srv_now_ns.restype = C.c_uint64
    if path is None:
        _lib = lib
    return lib


def _check(code: int, what: str) -> None:
    if code != 0:
        raise GqsError(code, what)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Context:
    """A gqs context on one device (the reference's OCLResources role)."""

    def __init__(self, device: int = 0, sync: bool = True, timing: bool = False, timeout_ms: int = 4000,
                 variant: int = -1):
        self.lib = load_library()
        cfg = Config()
        self.lib.gqs_config_default(C.byref(cfg))
        cfg.sync = 1 if sync else 0
        cfg.timing = 1 if timing else 0
        cfg.timeout_ms = timeout_ms
        cfg.variant = variant
        h = C.c_void_p()
        _check(self.lib.gqs_create(C.byref(h), device, C.byref(cfg)), "gqs_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gqs_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- host pointers (the reference's GPUQSort<T>(ctx, size, d, dn)) ---
    def sort(self, a: np.ndarray) -> None:
        """Sorts a contiguous numpy array of uint32/float32/float64 in place."""
        t = _np_tag(a)
        assert a.flags.c_contiguous
        _check(getattr(self.lib, f"gqs_sort_{t}")(self.h, _ptr(a), None, a.size), f"gqs_sort_{t}")

    def sort_pairs(self, keys: np.ndarray, values: np.ndarray) -> None:
        """Sorts (key, value) pairs in place by key (uint32 or float32 keys, uint32 values)."""
        t = _np_tag(keys)
        if t not in ("u32", "f32") or values.dtype != np.uint32 or values.size != keys.size:
            raise TypeError("pairs are uint32/float32 keys with uint32 values of the same length")
        assert keys.flags.c_contiguous and values.flags.c_contiguous
        _check(getattr(self.lib, f"gqs_sort_pairs_{t}")(self.h, _ptr(keys), _ptr(values), keys.size),
               f"gqs_sort_pairs_{t}")

    def argsort(self, keys: np.ndarray) -> np.ndarray:
        """Stable argsort of uint32/float32 keys (keys are left untouched)."""
        k = keys.copy()
        idx = np.arange(keys.size, dtype=np.uint32)
        self.sort_pairs(k, idx)
        return idx

    def sort_pairs_dev(self, dtype: str, keys: int, values: int, n: int, stream: int = 0) -> int:
        return getattr(self.lib, f"gqs_sort_pairs_{dtype}_dev")(self.h, keys, values, n, stream or None)

    def sort_segments(self, a: np.ndarray, offsets: np.ndarray) -> None:
        t = _np_tag(a)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        _check(getattr(self.lib, f"gqs_sort_segments_{t}")(self.h, _ptr(a), a.size, _ptr(off), off.size - 1),
               f"gqs_sort_segments_{t}")

    # --- device pointers ---
    def sort_dev(self, dtype: str, d: int, scratch: int | None, n: int, stream: int = 0) -> int:
        return getattr(self.lib, f"gqs_sort_{dtype}_dev")(self.h, d, scratch, n, stream or None)

    def sort_segments_dev(self, dtype: str, keys: int, scratch: int | None, n: int, offsets: int, nseg: int,
                          stream: int = 0) -> int:
        return getattr(self.lib, f"gqs_sort_segments_{dtype}_dev")(self.h, keys, scratch, n, offsets, nseg,
                                                                    stream or None)

    def reserve(self, dtype: str, n: int, nseg: int = 1, with_buffers: bool = False) -> None:
        _check(self.lib.gqs_reserve(self.h, DTYPES[dtype], n, nseg, 1 if with_buffers else 0), "gqs_reserve")

    def sync(self) -> int:
        return self.lib.gqs_sync(self.h)

    def stats(self) -> dict:
        s = Stats()
        code = self.lib.gqs_last_stats(self.h, C.byref(s))
        d = s.as_dict()
        d["call_status"] = code
        return d

    PROFILE_SLOTS = ["c_wait", "c_part", "c_drain", "c_lwait", "c_lcta", "c_lwarp", "c_lstore", "c_fill",
                     "p_grab", "p_empty", "p_lempty", "p_idle", "q_busy", "q_idle", "n_local", "c_total",
                     "p_issue", "n_grab", "n_lcta", "n_lwarp", "n_lbit", "n_items", "c_count", "c_leader",
                     "c_scatter", "w_slice", "n_segs", "w_bit"]

    def profile(self) -> dict:
        buf = (C.c_uint64 * 32)()
        k = self.lib.gqs_last_profile(self.h, buf, 32)
        return {name: int(buf[i]) for i, name in enumerate(self.PROFILE_SLOTS) if i < k}

    def phases(self) -> dict:
        """The last sort's split of consumer-leader cycles: partition chunks, on-chip sorts, pivot
        fills and the whole loop, with the shares of the first three."""
        ph = Phases()
        _check(self.lib.gqs_last_phases(self.h, C.byref(ph)), "gqs_last_phases")
        d = {f: int(getattr(ph, f)) for f, _ in Phases._fields_}
        tot = d["total_cycles"] or 1
        d["partition_share"] = d["partition_cycles"] / tot
        d["onchip_share"] = d["onchip_cycles"] / tot
        d["fill_share"] = d["fill_cycles"] / tot
        return d

    def set_variant(self, dtype: str, v: int) -> None:
        _check(self.lib.gqs_set_variant(self.h, DTYPES[dtype], v), "gqs_set_variant")

    def levels(self) -> list[dict]:
        """Per-level rows of the last sort (profiling library only; [] otherwise)."""
        buf = (Level * 64)()
        k = self.lib.gqs_last_levels(self.h, buf, 64)
        return [{f: getattr(buf[i], f) for f, _ in Level._fields_ if f != "reserved"} for i in range(k)]

    def selftest_bounds(self, dtype: str) -> int:
        """Sorts keys under a deliberately short index bound; a -DGQS_CHECK build reports
        GQS_ERR_BOUNDS, the product build sorts them (GQS_OK)."""
        return self.lib.gqs_selftest_bounds(self.h, DTYPES[dtype])

    def selftest_stalled_queue(self, dtype: str, timeout_ms: int) -> int:
        """Runs the kernel on a queue that can never finish; returns the status it reports."""
        return self.lib.gqs_selftest_stalled_queue(self.h, DTYPES[dtype], timeout_ms)

    def get_variant(self, dtype: str) -> int:
        return self.lib.gqs_get_variant(self.h, DTYPES[dtype])


class Batch:
    """A graph-captured batched segmented sort (gqs_batch_*): the caller fills the device key
    arena (`keys_ptr`) and the pinned segment table (`offsets`), then launches."""

    def __init__(self, dtype: str, max_keys: int, max_segments: int, device: int = 0, variant: int = -1,
                 timeout_ms: int = 4000):
        self.lib = load_library()
        self.dtype = dtype
        cfg = Config()
        self.lib.gqs_config_default(C.byref(cfg))
        cfg.variant = variant
        cfg.timeout_ms = timeout_ms
        h = C.c_void_p()
        _check(self.lib.gqs_batch_create(device, DTYPES[dtype], max_keys, max_segments, C.byref(cfg), C.byref(h)),
               "gqs_batch_create")
        self.h = h
        self.max_keys = max_keys
        self.max_segments = max_segments
        self.keys_ptr = self.lib.gqs_batch_keys(h)
        self.offsets = np.ctypeslib.as_array(self.lib.gqs_batch_offsets(h), shape=(max_segments + 1,))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.offsets = None
            self.lib.gqs_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_segments(self, offsets: np.ndarray) -> int:
        off = np.asarray(offsets, dtype=np.uint64)
        nseg = off.size - 1
        if nseg > self.max_segments:
            raise ValueError("too many segments for this batch")
        self.offsets[: nseg + 1] = off
        return nseg

    def copy_in(self, a: np.ndarray, first: int = 0) -> None:
        assert a.dtype == NP_DTYPES[self.dtype] and a.flags.c_contiguous
        _check(self.lib.gqs_batch_copy_in(self.h, _ptr(a), first, a.size), "gqs_batch_copy_in")

    def copy_out(self, a: np.ndarray, first: int = 0) -> None:
        assert a.dtype == NP_DTYPES[self.dtype] and a.flags.c_contiguous
        _check(self.lib.gqs_batch_copy_out(self.h, _ptr(a), first, a.size), "gqs_batch_copy_out")

    def launch(self, nseg: int, stream: int = 0) -> int:
        return self.lib.gqs_batch_launch(self.h, nseg, stream or None)

    def wait(self) -> tuple[int, dict]:
        s = Stats()
        code = self.lib.gqs_batch_wait(self.h, C.byref(s))
        return code, s.as_dict()

    def set_variant(self, v: int) -> None:
        _check(self.lib.gqs_batch_set_variant(self.h, v), "gqs_batch_set_variant")

    @property
    def variant(self) -> int:
        return self.lib.gqs_batch_get_variant(self.h)

    def autotune(self, nseg: int, reps: int = 3) -> tuple[int, list[float]]:
        """Times every variant on the batch as it stands; selects and returns the fastest."""
        nv = self.lib.gqs_variant_count(DTYPES[self.dtype])
        ms = (C.c_double * nv)()
        best = C.c_int(-1)
        _check(self.lib.gqs_batch_autotune(self.h, nseg, reps, ms, C.byref(best)), "gqs_batch_autotune")
        return best.value, [ms[i] for i in range(nv)]


class Server:
    """The continuous-batching sort server (gqs_srv_*)."""

    def __init__(self, device: int = 0, budget_bytes: int = 64 << 30, batch_keys: int = 1 << 27,
                 batch_segments: int = 4096, lanes: int = 3, per_request: bool = False,
                 variants: tuple[int, int, int] = (-1, -1, -1), timeout_ms: int = 4000):
        self.lib = load_library()
        cfg = ServerConfig()
        self.lib.gqs_srv_config_default(C.byref(cfg))
        cfg.budget_bytes = budget_bytes
        cfg.batch_keys = batch_keys
        cfg.batch_segments = batch_segments
        cfg.lanes = lanes
        cfg.per_request = 1 if per_request else 0
        cfg.timeout_ms = timeout_ms
        for i, v in enumerate(variants):
            cfg.variant[i] = v
        h = C.c_void_p()
        _check(self.lib.gqs_srv_create(device, C.byref(cfg), C.byref(h)), "gqs_srv_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gqs_srv_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, src: np.ndarray, out: np.ndarray | None = None) -> int:
        """Queues a sort of `src` into `out` (default: in place); both must outlive the request."""
        t = _np_tag(src)
        out = src if out is None else out
        assert out.dtype == src.dtype and out.size >= src.size and src.flags.c_contiguous and out.flags.c_contiguous
        rid = C.c_uint64()
        _check(self.lib.gqs_srv_submit(self.h, DTYPES[t], _ptr(src), _ptr(out), src.size, C.byref(rid)),
               "gqs_srv_submit")
        return rid.value

    def submit_raw(self, dtype: str, src: int, out: int, n: int) -> int:
        rid = C.c_uint64()
        _check(self.lib.gqs_srv_submit(self.h, DTYPES[dtype], src, out, n, C.byref(rid)), "gqs_srv_submit")
        return rid.value

    def wait(self, rid: int) -> tuple[int, dict]:
        info = RequestInfo()
        code = self.lib.gqs_srv_wait(self.h, rid, C.byref(info))
        return code, info.as_dict()

    def wait_any(self, timeout_ms: int = 10000) -> tuple[int, int, dict]:
        """(status, request id, info) of the next completed request; status 4 (timeout) when none."""
        rid = C.c_uint64(0)
        info = RequestInfo()
        code = self.lib.gqs_srv_wait_any(self.h, C.byref(rid), C.byref(info), timeout_ms)
        return code, rid.value, info.as_dict()

    def cancel(self, rid: int) -> int:
        return self.lib.gqs_srv_cancel(self.h, rid)

    def drain(self) -> int:
        return self.lib.gqs_srv_drain(self.h)

    def stats(self) -> dict:
        s = ServerStats()
        code = self.lib.gqs_srv_stats(self.h, C.byref(s))
        d = s.as_dict()
        d["call_status"] = code
        return d

    def now_ns(self) -> int:
        return self.lib.gqs_srv_now_ns()


def variants(dtype: str) -> list[dict]:
    lib = load_library()
    out = []
    for v in range(lib.gqs_variant_count(DTYPES[dtype])):
        d = VariantDesc()
        _check(lib.gqs_variant_describe(DTYPES[dtype], v, C.byref(d)), "gqs_variant_describe")
        out.append({"index": v, "threads": d.threads, "tile": d.tile, "chunk": d.chunk, "kpt": d.kpt,
                    "stages": d.stages, "tiny": d.tiny, "smem_bytes": d.smem_bytes, "name": d.name.decode()})
    return out


def _np_tag(a: np.ndarray) -> str:
    for t, dt in NP_DTYPES.items():
        if a.dtype == dt:
            return t
    raise TypeError(f"unsupported key dtype {a.dtype}")


# ---------------------------------------------------------------------------
# Workload generators (libgqs_workload.so)

def load_workload() -> C.CDLL:
    global _wl
    if _wl is not None:
        return _wl
    if not os.path.exists(WORKLOAD_PATH):
        raise FileNotFoundError(f"{WORKLOAD_PATH} is missing: build it with __graft_entry__.build()")
    wl = C.CDLL(WORKLOAD_PATH)
    for t in ("u32", "f32", "f64"):
        f = getattr(wl, f"gqs_workload_{t}")
        f.argtypes = [C.c_int, C.c_uint64, C.c_size_t, C.c_void_p]
        f.restype = C.c_int
    wl.gqs_workload_segments.argtypes = [C.c_uint64, C.c_size_t, C.c_uint64, C.c_uint64, C.c_void_p]
    wl.gqs_workload_segments.restype = C.c_uint64
    for name in ("gqs_workload_det_log", "gqs_workload_det_exp", "gqs_workload_det_cos2pi"):
        getattr(wl, name).argtypes = [C.c_double]
        getattr(wl, name).restype = C.c_double
    _wl = wl
    return wl


def generate(dtype: str, dist: str, seed: int, n: int, out: np.ndarray | None = None) -> np.ndarray:
    """Seeded keys of one configured distribution (identical on every platform)."""
    wl = load_workload()
    if out is None:
        out = np.empty(n, dtype=NP_DTYPES[dtype])
    assert out.dtype == NP_DTYPES[dtype] and out.size >= n and out.flags.c_contiguous
    rc = getattr(wl, f"gqs_workload_{dtype}")(DIST[dist], seed, n, _ptr(out))
    if rc != 0:
        raise ValueError(f"distribution {dist} is not defined for {dtype}")
    return out


def segment_offsets(seed: int, nseg: int, minlen: int, maxlen: int) -> np.ndarray:
    """nseg + 1 offsets with log-uniform segment lengths in [minlen, maxlen]."""
    wl = load_workload()
    off = np.empty(nseg + 1, dtype=np.uint64)
    wl.gqs_workload_segments(seed, nseg, minlen, maxlen, _ptr(off))
    return off
