"""GPU tests for the sort server (gqs_srv_*): a mixed stream of requests of all three key types
sorts to exactly the same bits as each request sorted alone by the plain sort, whatever it was
batched with, under a memory budget that forces requests to wait for admission."""
import numpy as np
import pytest

import gqs_ctypes

pytestmark = pytest.mark.gpu

DIST = {"u32": "uniform", "f32": "gaussian", "f64": "uniform"}


def mixed_requests(seed, count, lo_log2, hi_log2):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        u = rng.random()
        dtype = "u32" if u < 0.6 else ("f32" if u < 0.9 else "f64")
        n = int(np.exp(rng.uniform(np.log(2 ** lo_log2), np.log(2 ** hi_log2))))
        reqs.append(gqs_ctypes.generate(dtype, DIST[dtype], seed * 100003 + i, n))
    return reqs


def serve_all(srv, reqs):
    outs = [np.empty_like(a) for a in reqs]
    ids = [srv.submit(a, o) for a, o in zip(reqs, outs)]
    infos = []
    for rid in ids:
        code, info = srv.wait(rid)
        assert code == 0, info
        infos.append(info)
    return outs, infos


def test_mixed_stream_same_alone_and_in_mix(gpu_ctx):
    reqs = mixed_requests(7, 240, 10, 18)
    with gqs_ctypes.Server(budget_bytes=1 << 30, batch_keys=1 << 22, batch_segments=4096, lanes=3) as srv:
        outs, infos = serve_all(srv, reqs)
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] < len(reqs)  # requests were batched together
    assert max(i["batch_requests"] for i in infos) > 1
    for a, b in zip(reqs, outs):
        alone = a.copy()
        gpu_ctx.sort(alone)  # the plain sort, one request alone
        assert np.array_equal(b.view(np.uint8), alone.view(np.uint8))
        assert np.array_equal(b, np.sort(a))


def test_tight_budget_admits_as_memory_frees():
    reqs = mixed_requests(8, 60, 14, 17)
    biggest = max(a.nbytes for a in reqs)
    kw = dict(batch_keys=1 << 17, batch_segments=64, lanes=2)
    probe_budget = 1 << 28
    with gqs_ctypes.Server(budget_bytes=probe_budget, **kw) as srv:
        overhead = probe_budget - 2 * srv.stats()["arena_bytes"]  # the lanes' job records and rings
    # the arena holds about three of the largest requests at a time
    with gqs_ctypes.Server(budget_bytes=overhead + 2 * (3 * biggest + 4096), **kw) as srv:
        outs, _ = serve_all(srv, reqs)
        st = srv.stats()
    assert st["arena_bytes"] < sum(a.nbytes for a in reqs) // 4  # requests had to wait for room
    assert st["arena_peak"] <= st["arena_bytes"] and st["completed"] == len(reqs)
    for a, b in zip(reqs, outs):
        assert np.array_equal(b, np.sort(a))


def test_per_request_mode_matches():
    reqs = mixed_requests(9, 30, 10, 16)
    with gqs_ctypes.Server(budget_bytes=1 << 30, batch_keys=1 << 20, per_request=True) as srv:
        outs, infos = serve_all(srv, reqs)
        st = srv.stats()
    assert all(i["batch_requests"] == 1 for i in infos) and st["batches"] == len(reqs)
    for a, b in zip(reqs, outs):
        assert np.array_equal(b, np.sort(a))


def test_in_place_requests_and_timestamps():
    reqs = mixed_requests(10, 20, 10, 15)
    ref = [np.sort(a) for a in reqs]
    with gqs_ctypes.Server(budget_bytes=1 << 30, batch_keys=1 << 20) as srv:
        ids = [srv.submit(a) for a in reqs]  # in place
        seen = set()
        while len(seen) < len(ids):
            code, rid, info = srv.wait_any(10000)
            assert code == 0 and rid in ids and rid not in seen
            assert info["t_submit_ns"] <= info["t_admit_ns"] <= info["t_launch_ns"] <= info["t_done_ns"]
            seen.add(rid)
        assert srv.wait_any(1)[0] == 4  # nothing left: times out
    for a, r in zip(reqs, ref):
        assert np.array_equal(a, r)


def test_rejects_oversized_and_bad_requests():
    with gqs_ctypes.Server(budget_bytes=1 << 30, batch_keys=1 << 12) as srv:
        with pytest.raises(gqs_ctypes.GqsError):
            srv.submit(np.zeros(1 << 13, np.uint32))  # above batch_keys
        with pytest.raises(gqs_ctypes.GqsError):
            srv.submit(np.zeros(0, np.uint32))
        assert srv.wait(12345)[0] == 1  # unknown id
