"""Failure detection without a GPU fault: bounded device waits that run out end the kernel with
a status and leave the context usable; allocation failures, over-budget requests and
cancellations come back as statuses. Nothing here faults, traps or hangs a GPU."""
import time

import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

DIST = {"u32": "uniform", "f32": "gaussian", "f64": "uniform"}


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_stalled_queue_times_out_and_context_recovers(dtype):
    """A queue that claims a key but holds no work: every role waits for progress that never
    comes, the waits end after the limit with GQS_ERR_TIMEOUT, and the next sort is exact."""
    with gqs_ctypes.Context(timeout_ms=4000) as ctx:
        t0 = time.perf_counter()
        st = ctx.selftest_stalled_queue(dtype, 200)
        dt = time.perf_counter() - t0
        assert st == 4, gqs_ctypes.STATUS.get(st, st)
        assert 0.15 < dt < 5.0, dt
        assert ctx.stats()["status"] == 4
        x = gqs_ctypes.generate(dtype, DIST[dtype], 5, 300001)
        y = x.copy()
        ctx.sort(y)
        assert np.array_equal(y, np.sort(x))


def test_allocation_failures_are_statuses():
    with gqs_ctypes.Context() as ctx:
        with pytest.raises(gqs_ctypes.GqsError) as e:
            ctx.reserve("u32", 1 << 36, 1, True)  # 2 x 256 GiB of keys: cudaMalloc fails
        assert e.value.code == 3
        x = gqs_ctypes.generate("u32", "uniform", 6, 1 << 16)
        y = x.copy()
        ctx.sort(y)
        assert np.array_equal(y, np.sort(x))
    with pytest.raises(gqs_ctypes.GqsError) as e:
        gqs_ctypes.Batch("u32", 1 << 36, 16)
    assert e.value.code == 3
    with pytest.raises(gqs_ctypes.GqsError) as e:
        gqs_ctypes.Server(budget_bytes=1 << 50)
    assert e.value.code == 3


def test_request_larger_than_the_budget_is_rejected():
    with gqs_ctypes.Server(budget_bytes=1 << 28, batch_keys=1 << 26, lanes=1) as srv:
        arena = srv.stats()["arena_bytes"]
        n = arena // 4 + 1024  # one more key than the arena holds
        if n > (1 << 26):
            pytest.skip("the arena exceeds the batch limit")
        with pytest.raises(gqs_ctypes.GqsError) as e:
            srv.submit(np.zeros(n, np.uint32))
        assert e.value.code == 3


def test_cancelled_requests_complete_as_cancelled():
    big = gqs_ctypes.generate("u32", "uniform", 8, 1 << 24)
    small = [gqs_ctypes.generate("u32", "uniform", 100 + i, 5000) for i in range(20)]
    kw = dict(batch_keys=1 << 24, batch_segments=64, lanes=1)
    probe = 1 << 30
    with gqs_ctypes.Server(budget_bytes=probe, **kw) as srv:
        overhead = probe - 2 * srv.stats()["arena_bytes"]
    # the arena holds the big request and little else, so the small ones wait for admission
    with gqs_ctypes.Server(budget_bytes=overhead + 2 * (big.nbytes + 4096), **kw) as srv:
        outs = [np.empty_like(a) for a in small]
        big_out = np.empty_like(big)
        ids = [srv.submit(big, big_out)] + [srv.submit(a, o) for a, o in zip(small, outs)]
        cancelled = {rid for rid in ids[1::2] if srv.cancel(rid) == 0}
        assert cancelled, "no request was still waiting"
        assert srv.cancel(ids[0]) in (0, 1)
        for rid, a, o in zip(ids, [big] + small, [big_out] + outs):
            code, info = srv.wait(rid)
            if rid in cancelled:
                assert code == 8 and info["status"] == 8
            elif code == 8:
                continue  # the big request, cancelled before it started
            else:
                assert code == 0 and np.array_equal(o, np.sort(a))
        st = srv.stats()
        assert st["cancelled"] >= len(cancelled) and st["failed"] == 0
        assert srv.cancel(ids[1]) == 1  # unknown now
