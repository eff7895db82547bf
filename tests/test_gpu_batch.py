"""GPU parity for the graph-captured batch (gqs_batch_*): every segment of every replay equals
its own sort, for every kernel variant, and the autotuner picks a variant that runs."""
import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

DIST = {"u32": "uniform", "f32": "gaussian", "f64": "uniform"}


def check_segments(a, b, off, what=None):
    for i in range(len(off) - 1):
        s, e = int(off[i]), int(off[i + 1])
        assert np.array_equal(b[s:e], np.sort(a[s:e])), (what, i, s, e)


def run_batch(batch, a, off):
    nseg = batch.set_segments(off)
    batch.copy_in(a)
    assert batch.launch(nseg) == 0
    code, st = batch.wait()
    assert code == 0, st
    b = np.empty_like(a)
    batch.copy_out(b)
    return b, st


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_batch_matches_per_segment_sort(dtype):
    off = gqs_ctypes.segment_offsets(31, 3000, 1, 5000)
    a = gqs_ctypes.generate(dtype, DIST[dtype], 31, int(off[-1]))
    with gqs_ctypes.Batch(dtype, int(off[-1]), 4096) as batch:
        b, st = run_batch(batch, a, off)
        assert st["keys"] == int(off[-1]) and st["kernel_ms"] > 0
    check_segments(a, b, off)


def test_one_graph_replays_batches_of_any_shape():
    """The segment table is data: one captured graph sorts differently shaped batches."""
    with gqs_ctypes.Batch("u32", 1 << 21, 2048) as batch:
        for seed, nseg, lo, hi in [(41, 2000, 1, 1000), (42, 7, 1000, 1 << 18), (43, 1, 1 << 20, 1 << 20),
                                   (44, 512, 32, 4096), (45, 0, 1, 1)]:
            off = gqs_ctypes.segment_offsets(seed, nseg, lo, hi) if nseg else np.zeros(1, np.uint64)
            a = gqs_ctypes.generate("u32", "uniform", seed, max(1, int(off[-1])))[: int(off[-1])]
            if a.size == 0:
                assert batch.set_segments(off) == 0
                assert batch.launch(0) == 0 and batch.wait()[0] == 0
                continue
            b, _ = run_batch(batch, a, off)
            check_segments(a, b, off)


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_every_variant_in_a_batch(dtype):
    off = gqs_ctypes.segment_offsets(51, 300, 16, 1 << 16)
    a = gqs_ctypes.generate(dtype, DIST[dtype], 51, int(off[-1]))
    with gqs_ctypes.Batch(dtype, int(off[-1]), 512) as batch:
        for v in range(len(gqs_ctypes.variants(dtype))):
            batch.set_variant(v)
            b, st = run_batch(batch, a, off)
            assert st["variant"] == v
            check_segments(a, b, off, f"variant {v}")


@pytest.mark.parametrize("dtype", ["u32", "f64"])
def test_autotune_picks_a_running_variant(dtype):
    off = gqs_ctypes.segment_offsets(61, 1000, 32, 1 << 17)
    a = gqs_ctypes.generate(dtype, DIST[dtype], 61, int(off[-1]))
    with gqs_ctypes.Batch(dtype, int(off[-1]), 1024) as batch:
        nseg = batch.set_segments(off)
        batch.copy_in(a)
        best, ms = batch.autotune(nseg, reps=2)
        assert 0 <= best < len(ms) and ms[best] > 0
        assert ms[best] == min(m for m in ms if m >= 0)
        assert batch.variant == best
        b = np.empty_like(a)
        batch.copy_out(b)  # left sorted by the chosen variant
        check_segments(a, b, off)
        b2, st = run_batch(batch, a, off)
        assert st["variant"] == best
        assert np.array_equal(b, b2)


def test_bad_tables_are_rejected_before_launch():
    with gqs_ctypes.Batch("u32", 1000, 8) as batch:
        batch.offsets[:3] = [0, 10, 5]  # decreasing
        assert batch.launch(2) == 1
        batch.offsets[:3] = [0, 10, 1001]  # past the arena
        assert batch.launch(2) == 1
        assert batch.launch(9) == 1  # more segments than the batch holds
        batch.offsets[:3] = [0, 10, 20]
        batch.copy_in(np.arange(20, 0, -1, dtype=np.uint32))
        assert batch.launch(2) == 0 and batch.wait()[0] == 0
