"""Device bounds checks (the -DGQS_CHECK build, libgqs_check.so), the stand-in for a memory
checker on this pool: every job record, staged range and global write index is tested against
the sort's bounds, and a failed test ends the sort with GQS_ERR_BOUNDS instead of an access.

The check build runs a battery of sorts (every key type, sizes around every threshold, both
entry points, segments, key-value pairs, a graph-captured batch, the pipelined host sort) in a
child process and must report no violation and exact results; its self-test, which gives the
kernel a key-index bound shorter than the data, must report GQS_ERR_BOUNDS. The product build
compiles the checks out: the same self-test sorts normally. Every access of the self-test stays
inside its buffers whatever the build, so nothing here can fault a GPU."""
import os
import subprocess
import sys

import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-quicksort_gb300")

BATTERY = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import gqs_ctypes, torch

DISTS = {"u32": ["uniform", "sorted", "reverse", "distinct16", "zipf", "allequal"],
         "f32": ["gaussian", "distinct16", "reverse"], "f64": ["uniform", "sorted", "distinct16"]}
SIZES = [1, 2, 255, 256, 257, 2049, 4097, 6145, 8193, 12289, 16385, 100003, 1 << 20, 3000001]
checked = 0
for dtype in ("u32", "f32", "f64"):
    for v in range(len(gqs_ctypes.variants(dtype))):
        with gqs_ctypes.Context(variant=v) as ctx:
            for i, n in enumerate(SIZES):
                dist = DISTS[dtype][(i + v) % len(DISTS[dtype])]
                a = gqs_ctypes.generate(dtype, dist, 1000 * v + n, n)
                ref = np.sort(a)
                if i % 2:
                    b = a.copy()
                    ctx.sort(b)
                else:
                    d = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
                    assert ctx.sort_dev(dtype, d.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
                    b = d.cpu().numpy()
                    b = b.view(np.uint32) if dtype == "u32" else b
                assert np.array_equal(b.view(np.uint8), ref.view(np.uint8)), (dtype, v, dist, n)
                assert ctx.stats()["status"] == 0
                checked += 1
    with gqs_ctypes.Context() as ctx:
        assert ctx.selftest_bounds(dtype) == 9, "the planted bound must be reported"
        x = gqs_ctypes.generate(dtype, DISTS[dtype][0], 7, (1 << 24) + 3)  # pipelined host sort
        y = x.copy()
        ctx.sort(y)
        assert np.array_equal(y.view(np.uint8), np.sort(x).view(np.uint8))
        off = gqs_ctypes.segment_offsets(11, 300, 1, 20000)
        x = gqs_ctypes.generate(dtype, DISTS[dtype][0], 12, int(off[-1]))
        y = x.copy()
        ctx.sort_segments(y, off)
        for s, e in zip(off[:-1], off[1:]):
            assert np.array_equal(y[s:e].view(np.uint8), np.sort(x[s:e]).view(np.uint8))
        checked += 3
with gqs_ctypes.Context() as ctx:
    k = gqs_ctypes.generate("u32", "distinct16", 21, 500001)
    vals = np.arange(k.size, dtype=np.uint32)
    kk, vv = k.copy(), vals.copy()
    ctx.sort_pairs(kk, vv)
    order = np.argsort(k, kind="stable")
    assert np.array_equal(kk, k[order]) and np.array_equal(vv, vals[order])
    checked += 1
off = gqs_ctypes.segment_offsets(13, 512, 32, 1 << 16)
with gqs_ctypes.Batch("u32", int(off[-1]), 512) as b:
    x = gqs_ctypes.generate("u32", "uniform", 14, int(off[-1]))
    nseg = b.set_segments(off)
    b.copy_in(x)
    assert b.launch(nseg) == 0
    code, st = b.wait()
    assert code == 0 and st["status"] == 0
    y = np.empty_like(x)
    b.copy_out(y)
    for s, e in zip(off[:-1], off[1:]):
        assert np.array_equal(y[s:e], np.sort(x[s:e]))
    checked += 1
print("checked", checked)
"""


def test_check_build_finds_no_violation_and_reports_a_planted_one():
    import build_lib
    lib = build_lib.build(check=True)["lib"]
    env = dict(os.environ, GQS_LIB=lib)
    r = subprocess.run([sys.executable, "-c", BATTERY, PKG], env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "checked" in r.stdout


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_product_build_compiles_the_checks_out(gpu_ctx, dtype):
    assert gpu_ctx.selftest_bounds(dtype) == 0
    assert gpu_ctx.stats()["status"] == 0
