"""The C ABI library loads and exports every function include/gqs.h declares (no GPU needed)."""
import ctypes
import os
import re

import gqs_ctypes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gqs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gqs_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(gqs_ctypes.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = gqs_ctypes.load_library()
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_host_only_calls():
    lib = gqs_ctypes.load_library()
    assert lib.gqs_version() >= 1
    assert lib.gqs_strerror(0) == b"ok"
    assert lib.gqs_strerror(4).startswith(b"device wait timed out")
    cfg = gqs_ctypes.Config()
    lib.gqs_config_default(ctypes.byref(cfg))
    assert cfg.variant == -1 and cfg.sync == 1 and cfg.timeout_ms == 4000
    for t in ("u32", "f32", "f64"):
        vs = gqs_ctypes.variants(t)
        assert vs and all(v["smem_bytes"] <= 232448 for v in vs)
        assert all(v["tile"] > v["tiny"] for v in vs)


def test_null_context_is_rejected():
    lib = gqs_ctypes.load_library()
    assert lib.gqs_sort_u32(None, None, None, 10) == 1
    assert lib.gqs_sort_u32_dev(None, None, None, 10, None) == 1
    assert lib.gqs_sync(None) == 1


def test_batch_and_server_need_a_gb300():
    """Without an sm_103 GPU the batch and server constructors fail with a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a GPU is present")
    lib = gqs_ctypes.load_library()
    h = ctypes.c_void_p()
    assert lib.gqs_batch_create(0, 0, 1000, 10, None, ctypes.byref(h)) == 6
    assert lib.gqs_srv_create(0, None, ctypes.byref(h)) == 6
    assert lib.gqs_batch_launch(None, 1, None) == 1
    assert lib.gqs_srv_submit(None, 0, None, None, 1, ctypes.byref(ctypes.c_uint64())) == 1
    cfg = gqs_ctypes.ServerConfig()
    lib.gqs_srv_config_default(ctypes.byref(cfg))
    assert cfg.budget_bytes == 64 << 30 and cfg.lanes == 3 and cfg.batch_segments == 4096
