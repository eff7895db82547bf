"""The profiling flavour of the library (libgqs_prof.so): its per-level rows, the counterpart of
the reference's optional per-level timing, add up to the sort's own counters; the product
library records none."""
import os
import subprocess
import sys

import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-quicksort_gb300")

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import gqs_ctypes, torch
for dtype, dist, n in (("u32", "uniform", 1 << 24), ("u32", "distinct16", 3000001), ("f64", "uniform", 1 << 22)):
    with gqs_ctypes.Context(timing=True) as ctx:
        a = gqs_ctypes.generate(dtype, dist, 9, n)
        d = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
        assert ctx.sort_dev(dtype, d.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
        b = d.cpu().numpy()
        b = b.view(np.uint32) if dtype == "u32" else b
        assert np.array_equal(b.view(np.uint8), np.sort(a).view(np.uint8))
        st, lv = ctx.stats(), ctx.levels()
        assert lv and [r["depth"] for r in lv] == sorted(r["depth"] for r in lv)
        assert sum(r["part_keys"] for r in lv) == st["part_keys"], (lv, st)
        assert sum(r["local_keys"] for r in lv) == st["local_keys"], (lv, st)
        assert sum(r["part_jobs"] for r in lv) == st["part_jobs"], (lv, st)
        assert sum(r["local_jobs"] for r in lv) == st["local_jobs"], (lv, st)
        assert lv[0]["depth"] == 0 and lv[0]["part_jobs"] == 1 and lv[0]["part_keys"] == n
        for r in lv:
            assert 0.0 <= r["first_ms"] <= r["last_ms"], r
        print(dtype, dist, n, [(r["depth"], r["part_jobs"], r["local_jobs"], round(r["last_ms"], 3)) for r in lv])
print("levels ok")
"""


def test_profiling_library_levels_add_up():
    import build_lib
    lib = build_lib.build(profile=True)["lib"]
    env = dict(os.environ, GQS_LIB=lib)
    r = subprocess.run([sys.executable, "-c", CHILD, PKG], env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "levels ok" in r.stdout


def test_product_library_records_no_levels(gpu_ctx):
    a = gqs_ctypes.generate("u32", "uniform", 3, 1 << 20)
    b = a.copy()
    gpu_ctx.sort(b)
    assert np.array_equal(b, np.sort(a))
    assert gpu_ctx.levels() == []
