"""GPU parity: the CUDA sort through the C ABI against the oracle, bit for bit.

Small and medium sizes compare with std::sort (the reference's verifier, run by the oracle
library) and with the committed golden vectors; every benchmark configuration at its full size
compares with std::sort through committed SHA-256 digests of its output (and with torch.sort);
the largest arrays compare with torch.sort and check sortedness.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import gqs_ctypes
import oracle_ctypes

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]
DISTS = {
    "u32": ["uniform", "sorted", "reverse", "distinct16", "zipf", "gaussian", "kat", "allequal"],
    "f32": ["gaussian", "uniform", "sorted", "reverse", "distinct16", "kat", "allequal"],
    "f64": ["uniform", "gaussian", "sorted", "reverse", "distinct16", "kat", "allequal"],
}
# sizes around the register sort (256), the chunk grid, the on-chip tile, and the first levels
SIZES = [2, 3, 31, 32, 33, 255, 256, 257, 1000, 2047, 2048, 2049, 4095, 4096, 4097, 8191, 8193, 16383,
         16384, 16385, 32769, 100_003, 1 << 20]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_sorted(a):
    r = a.copy()
    oracle_ctypes.std_sort(r)
    return r


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
@pytest.mark.parametrize("n", SIZES)
def test_sizes_match_oracle(gpu_ctx, dtype, n):
    for dist in ("uniform", "distinct16", "reverse"):
        a = gqs_ctypes.generate(dtype, dist, 1000 + n, n)
        b = a.copy()
        gpu_ctx.sort(b)
        assert np.array_equal(b.view(np.uint8), oracle_sorted(a).view(np.uint8)), (dtype, dist, n)


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_distributions_match_oracle(gpu_ctx, dtype):
    for dist in DISTS[dtype]:
        for n in (5000, 70_001, 1_000_003):
            a = gqs_ctypes.generate(dtype, dist, 77, n)
            b = a.copy()
            gpu_ctx.sort(b)
            assert np.array_equal(b.view(np.uint8), oracle_sorted(a).view(np.uint8)), (dtype, dist, n)


@pytest.mark.parametrize("case", [c for c in GOLDEN if c["n"] >= 1000],
                         ids=lambda c: f"{c['dtype']}-{c['dist']}-{c['n']}")
def test_golden_vectors(gpu_ctx, case):
    a = gqs_ctypes.generate(case["dtype"], case["dist"], case["seed"], case["n"])
    assert sha(a) == case["input_sha256"]
    gpu_ctx.sort(a)
    assert sha(a) == case["sorted_sha256"]


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_known_answer(gpu_ctx, dtype):
    # sizes up to the reference's own CTest run of its shuffled 1..N check, N = 2^22
    # (GPU-Quicksort_OpenCL_1.2/CMakeLists.txt:42-44, check at QuicksortMain.cpp:415-416)
    for n in (1, 2, 1024, 1 << 16, 1 << 20, 3_000_000, 1 << 22):
        a = gqs_ctypes.generate(dtype, "kat", 5, n)
        gpu_ctx.sort(a)
        assert np.array_equal(a, np.arange(1, n + 1, dtype=a.dtype))


def test_oracle_restatement_agrees(gpu_ctx):
    for dtype in ("u32", "f32", "f64"):
        a = gqs_ctypes.generate(dtype, "gaussian", 3, 1 << 18)
        b, c = a.copy(), a.copy()
        gpu_ctx.sort(b)
        oracle_ctypes.gpuqsort(c, threads=8)
        assert np.array_equal(b.view(np.uint8), c.view(np.uint8))


def test_signed_zero_and_extremes(gpu_ctx):
    """-0.0 sorts before +0.0 (std::sort may order them either way); every bit is kept."""
    vals = np.array([0.0, -0.0, 1.5, -1.5, np.finfo(np.float32).max, -np.finfo(np.float32).max,
                     np.finfo(np.float32).tiny, -np.finfo(np.float32).tiny, np.inf, -np.inf], dtype=np.float32)
    a = np.tile(vals, 5000)
    rng = np.random.default_rng(0)
    rng.shuffle(a)
    b = a.copy()
    gpu_ctx.sort(b)
    expect = np.sort(a)
    assert np.array_equal(b, expect)  # value order
    zeros = b[b == 0]
    nneg = int(np.sum(np.signbit(a) & (a == 0)))
    assert np.all(np.signbit(zeros[:nneg])) and not np.any(np.signbit(zeros[nneg:]))
    u = np.array([0, 1, 0xFFFFFFFF, 0x80000000, 0x7FFFFFFF] * 4000, dtype=np.uint32)
    rng.shuffle(u)
    v = u.copy()
    gpu_ctx.sort(v)
    assert np.array_equal(v, np.sort(u))


def test_repeated_calls_reuse_context(gpu_ctx):
    a = gqs_ctypes.generate("u32", "uniform", 99, 1 << 20)
    ref = oracle_sorted(a)
    for _ in range(5):
        b = a.copy()
        gpu_ctx.sort(b)
        assert np.array_equal(b, ref)
    st = gpu_ctx.stats()
    assert st["status"] == 0 and st["keys"] == 1 << 20
    assert st["part_keys"] + st["local_keys"] + st["tiny_keys"] >= 1 << 20


# ---------------------------------------------------------------------------
# device pointers (torch supplies HBM buffers and the stream)

def _torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
@pytest.mark.parametrize("shift", [0, 1, 3])
def test_device_api_unaligned_views(gpu_ctx, dtype, shift):
    torch = _torch()
    tdt = {"u32": torch.int32, "f32": torch.float32, "f64": torch.float64}[dtype]
    n = 1_000_001
    a = gqs_ctypes.generate(dtype, "uniform" if dtype != "f32" else "gaussian", 8, n)
    host = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a)
    buf = torch.empty(n + 8, dtype=tdt, device="cuda")
    scr = torch.empty(n + 8, dtype=tdt, device="cuda")
    d = buf[shift:shift + n]
    d.copy_(host)
    s = scr[(shift + 1) % 4:(shift + 1) % 4 + n]  # scratch misaligned differently from d
    stream = torch.cuda.current_stream().cuda_stream
    rc = gpu_ctx.sort_dev(dtype, d.data_ptr(), s.data_ptr(), n, stream)
    assert rc == 0
    out = d.cpu().numpy()
    if dtype == "u32":
        out = out.view(np.uint32)
    assert np.array_equal(out.view(np.uint8), oracle_sorted(a).view(np.uint8))


def test_device_api_guard_words_untouched(gpu_ctx):
    torch = _torch()
    n = 300_007
    a = gqs_ctypes.generate("u32", "uniform", 12, n)
    buf = torch.full((n + 64,), -7, dtype=torch.int32, device="cuda")
    d = buf[32:32 + n]
    d.copy_(torch.from_numpy(a.view(np.int32)))
    assert gpu_ctx.sort_dev("u32", d.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
    host = buf.cpu().numpy()
    assert np.all(host[:32] == -7) and np.all(host[32 + n:] == -7)
    assert np.array_equal(host[32:32 + n].view(np.uint32), np.sort(a))


def test_async_calls_then_sync():
    torch = _torch()
    ctx = gqs_ctypes.Context(sync=False, timing=True)
    try:
        n = 1 << 22
        a = gqs_ctypes.generate("u32", "uniform", 13, n)
        ref = np.sort(a)
        bufs = [torch.from_numpy(a.view(np.int32)).cuda() for _ in range(3)]
        side = torch.cuda.Stream()
        for i, b in enumerate(bufs):
            st = side if i == 1 else torch.cuda.current_stream()
            assert ctx.sort_dev("u32", b.data_ptr(), None, n, st.cuda_stream) == 0
        assert ctx.sync() == 0
        torch.cuda.synchronize()
        for b in bufs:
            assert np.array_equal(b.cpu().numpy().view(np.uint32), ref)
        st = ctx.stats()
        assert st["kernel_ms"] > 0
    finally:
        ctx.close()


# ---------------------------------------------------------------------------
# full configuration sizes: bit-exact against std::sort, through its committed digests

FULL_SIZE = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "full_size.json")))
FULL = [c for c in FULL_SIZE["cases"] if c["kind"] == "plain"]


def _device_sort_and_digest(gpu_ctx, dtype, a):
    """Sorts a copy of host array `a` through the device-pointer C ABI call; returns the result
    on the host, and torch.sort's result as a second, independent check."""
    torch = _torch()
    n = a.size
    t = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
    ref = torch.sort(t.to(torch.int64) & 0xFFFFFFFF).values if dtype == "u32" else torch.sort(t).values
    assert gpu_ctx.sort_dev(dtype, t.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
    got = (t.to(torch.int64) & 0xFFFFFFFF) if dtype == "u32" else t
    same_as_torch = bool(torch.equal(got, ref))
    out = t.cpu().numpy()
    del t, ref, got
    torch.cuda.empty_cache()
    return (out.view(np.uint32) if dtype == "u32" else out), same_as_torch


@pytest.mark.parametrize("case", FULL, ids=lambda c: f"{c['dtype']}-{c['dist']}-{c['n']}")
def test_full_size_configs(gpu_ctx, case):
    """Every plain configuration of the benchmark at its real size (2^28 u32 in six
    distributions, 2^27 f32, 2^26 f64, and 2^20 u32), on the benchmark's own seeded input: the
    output's SHA-256 equals that of std::sort's output (the reference's verifier,
    GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:1120-1138), recorded on the CPU by
    tests/golden/make_full_size.py."""
    dtype, n = case["dtype"], case["n"]
    a = gqs_ctypes.generate(dtype, case["dist"], case["seed"], n)
    assert sha(a) == case["input_sha256"], "the generator is not the one the digests were made with"
    out, same_as_torch = _device_sort_and_digest(gpu_ctx, dtype, a)
    assert sha(out) == case["sorted_sha256"]
    assert out[:4].tobytes().hex() == case["head"] and out[-4:].tobytes().hex() == case["tail"]
    assert same_as_torch
    st = gpu_ctx.stats()
    assert st["status"] == 0 and st["keys"] == n


BATCH_CASE = next(c for c in FULL_SIZE["cases"] if c["kind"] == "segments")


def _segment_digests_match(out, off, case):
    bad = [i for i in range(len(off) - 1)
           if hashlib.sha256(out[int(off[i]):int(off[i + 1])].tobytes()).hexdigest()[:16] != case["segment_sha256_16"][i]]
    return bad


def test_batched_config_graph_replay():
    """The batched configuration at its real shape (4096 uint32 arrays, lengths log-uniform in
    [32, 2^20], about 3.9e8 keys): autotuned, then one graph replay; every segment's digest and
    the whole output's digest equal std::sort's."""
    case = BATCH_CASE
    off = gqs_ctypes.segment_offsets(case["seed"], case["segments"], case["min_len"], case["max_len"])
    assert sha(off.astype(np.uint64)) == case["offsets_sha256"]
    n = int(off[-1])
    a = gqs_ctypes.generate("u32", "uniform", case["seed"], n)
    assert sha(a) == case["input_sha256"]
    with gqs_ctypes.Batch("u32", n, case["segments"]) as b:
        b.set_segments(off)
        b.copy_in(a)
        best, ms = b.autotune(case["segments"], reps=1)
        assert 0 <= best < len(ms)
        b.copy_in(a)  # the autotuner leaves the keys sorted; replay on the unsorted input
        assert b.launch(case["segments"]) == 0
        code, st = b.wait()
        assert code == 0 and st["keys"] == n
        out = np.empty_like(a)
        b.copy_out(out)
    assert _segment_digests_match(out, off, case) == []
    assert sha(out) == case["sorted_sha256"]


def test_batched_config_segmented_call(gpu_ctx):
    """The same configuration through the context's segmented device-pointer call."""
    torch = _torch()
    case = BATCH_CASE
    off = gqs_ctypes.segment_offsets(case["seed"], case["segments"], case["min_len"], case["max_len"])
    n = int(off[-1])
    a = gqs_ctypes.generate("u32", "uniform", case["seed"], n)
    t = torch.from_numpy(a.view(np.int32)).cuda()
    o = torch.from_numpy(off.astype(np.int64)).cuda()
    assert gpu_ctx.sort_segments_dev("u32", t.data_ptr(), None, n, o.data_ptr(), case["segments"],
                                     torch.cuda.current_stream().cuda_stream) == 0
    out = t.cpu().numpy().view(np.uint32)
    del t, o
    torch.cuda.empty_cache()
    assert _segment_digests_match(out, off, case) == []
    assert sha(out) == case["sorted_sha256"]


# The largest arrays: the top of the reference's benchmark sweep, 2 x 16384 x 16384 = 2^29
# keys (build_me.sh:3-20), and 2 GiB of doubles and 2 GiB of floats.
MAXSIZE = [("u32", "uniform", 1 << 29), ("f64", "uniform", 1 << 28), ("f32", "gaussian", 1 << 29)]


@pytest.mark.parametrize("dtype,dist,n", MAXSIZE, ids=lambda x: str(x))
def test_maximum_sizes(gpu_ctx, dtype, dist, n):
    """Beyond the committed digests: exact equality with torch.sort and sortedness."""
    a = gqs_ctypes.generate(dtype, dist, 2026, n)
    out, same_as_torch = _device_sort_and_digest(gpu_ctx, dtype, a)
    assert same_as_torch
    assert bool(np.all(out[1:] >= out[:-1]))
    st = gpu_ctx.stats()
    assert st["status"] == 0 and st["keys"] == n


# ---------------------------------------------------------------------------
# every compiled kernel variant sorts correctly

@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_all_variants(dtype):
    for v in gqs_ctypes.variants(dtype):
        ctx = gqs_ctypes.Context(variant=v["index"], timing=True)
        try:
            for dist in ("uniform", "distinct16", "sorted"):
                for n in (3000, v["tile"] + 1, 3 * v["chunk"] + 17, 1_500_007):
                    a = gqs_ctypes.generate(dtype, dist if dtype == "u32" or dist != "uniform" else "uniform", 31 + n, n)
                    b = a.copy()
                    ctx.sort(b)
                    assert np.array_equal(b.view(np.uint8), oracle_sorted(a).view(np.uint8)), (v["name"], dist, n)
                    assert ctx.stats()["variant"] == v["index"]
        finally:
            ctx.close()


@pytest.mark.parametrize("dtype,dist,n", [("u32", "uniform", 1 << 24), ("u32", "distinct16", (1 << 24) + 5),
                                          ("u32", "sorted", 3 * (1 << 23) + 7), ("f32", "gaussian", (1 << 24) + 3),
                                          ("f64", "uniform", (1 << 24) + 1), ("u32", "reverse", 1 << 25)])
def test_pipelined_host_sort(gpu_ctx, dtype, dist, n):
    """Host-pointer sorts of 2^24 keys and more are copied in four pieces, each sorted as soon as
    it arrives, and the sorted pieces merged: the result is the same as a single sort."""
    x = gqs_ctypes.generate(dtype, dist, 123 + n, n)
    y = x.copy()
    gpu_ctx.sort(y)
    assert np.array_equal(y.view(np.uint8), np.sort(x).view(np.uint8))
    st = gpu_ctx.stats()
    assert st["status"] == 0 and st["keys"] == n


@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_random_sizes_every_variant(dtype):
    """Seeded stress of the job scheduling: every kernel variant sorts 30 arrays of random
    log-uniform sizes in [1, 2^22] and random distributions, through the host and the device
    entry points in turn; each result is bit-exact against numpy's sort (no NaN or -0.0)."""
    torch = _torch()
    tdt = {"u32": torch.int32, "f32": torch.float32, "f64": torch.float64}[dtype]
    rng = np.random.default_rng(20260404)
    for v in gqs_ctypes.variants(dtype):
        ctx = gqs_ctypes.Context(variant=v["index"])
        try:
            for i in range(30):
                n = int(np.exp(rng.uniform(0.0, np.log(1 << 22))))
                dist = DISTS[dtype][int(rng.integers(len(DISTS[dtype])))]
                a = gqs_ctypes.generate(dtype, dist, int(rng.integers(1 << 30)), n)
                ref = np.sort(a)
                if i % 2 == 0:
                    b = a.copy()
                    ctx.sort(b)
                else:
                    d = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
                    assert ctx.sort_dev(dtype, d.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
                    b = d.cpu().numpy()
                    b = b.view(np.uint32) if dtype == "u32" else b
                assert np.array_equal(b.view(np.uint8), ref.view(np.uint8)), (v["name"], dist, n)
                assert ctx.stats()["status"] == 0
        finally:
            ctx.close()


# ---------------------------------------------------------------------------
# size-aware variant choice (the counterpart of the reference's optp size rule)

def _tuning_rows():
    import re
    text = open(os.path.join(os.path.dirname(os.path.dirname(__file__)), "gpu-quicksort_gb300", "csrc",
                             "gqs_tuning.h")).read()
    body = text[text.index("kTuneRows[] = {"):]
    return [tuple(int(x) for x in m) for m in re.findall(r"\{(\d+), (\d+), (\d+), (\d+)\}", body)]


def _expected_variant(rows, dtype_id, n, sms):
    lg = max(0, int(np.ceil(np.log2(max(n, 1)))))
    cand = [r for r in rows if r[1] == dtype_id]
    near = min(cand, key=lambda r: abs(r[0] - sms))[0]
    return min((r for r in cand if r[0] == near), key=lambda r: abs(r[2] - lg))[3]


def test_variant_follows_size(gpu_ctx):
    """A context created with variant -1 runs each sort with the variant the tuning table names
    for its key type and size class; the table picks different variants at different sizes, and
    every result stays bit-exact against std::sort. A fixed variant is kept at every size."""
    torch = _torch()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rows = _tuning_rows()
    sizes = [1 << k for k in range(10, 25)] + [3000, 100_003, 1_500_007]
    seen = set()
    for dtype, did in (("u32", 0), ("f32", 1), ("f64", 2)):
        for n in sizes:
            a = gqs_ctypes.generate(dtype, "uniform" if dtype != "f32" else "gaussian", 900 + n, n)
            b = a.copy()
            gpu_ctx.sort(b)
            assert np.array_equal(b.view(np.uint8), oracle_sorted(a).view(np.uint8)), (dtype, n)
            st = gpu_ctx.stats()
            want = _expected_variant(rows, did, n if n < (1 << 24) else n // 4, sms)
            assert st["variant"] == want, (dtype, n, st["variant"], want)
            seen.add((did, st["variant"]))
    assert len({v for d, v in seen if d == 0}) > 1, "the table names one variant for every u32 size"
    assert gpu_ctx.get_variant("u32") == -1
    ctx = gqs_ctypes.Context(variant=2)
    try:
        for n in (1 << 12, 1 << 18, 1 << 21):
            a = gqs_ctypes.generate("u32", "uniform", 5, n)
            ctx.sort(a)
            assert ctx.stats()["variant"] == 2 and ctx.get_variant("u32") == 2
    finally:
        ctx.close()


# ---------------------------------------------------------------------------
# the top split of small plain sorts (2^15 .. 2^21 keys)

@pytest.mark.parametrize("dtype", ["u32", "f32", "f64"])
def test_top_split_range(gpu_ctx, dtype):
    """Plain sorts of 2^15 .. 2^21 keys start with a multi-way split whose buckets are then sorted
    as segments: sizes at both ends of that range and just outside it, every distribution
    (all-equal keys put the whole array in one bucket), through both entry points, bit-exact
    against std::sort; the split is counted as one partition pass."""
    torch = _torch()
    for n in ((1 << 15) - 1, 1 << 15, 40_000, 300_007, 1 << 21, (1 << 21) + 1):
        for dist in (DISTS[dtype] if n <= 300_007 else ("uniform", "distinct16", "allequal")):
            a = gqs_ctypes.generate(dtype, dist, 4400 + n, n)
            ref = oracle_sorted(a)
            b = a.copy()
            gpu_ctx.sort(b)
            assert np.array_equal(b.view(np.uint8), ref.view(np.uint8)), (dtype, dist, n)
            st = gpu_ctx.stats()
            assert st["status"] == 0 and st["keys"] == n
            if (1 << 15) <= n <= (1 << 21):
                assert st["part_keys"] >= n, "the split pass is counted"
        t = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
        assert gpu_ctx.sort_dev(dtype, t.data_ptr(), None, n, torch.cuda.current_stream().cuda_stream) == 0
        out = t.cpu().numpy()
        assert np.array_equal(out.view(np.uint8), ref.view(np.uint8)), (dtype, "dev", n)


def test_top_split_pairs(gpu_ctx):
    """Key-value sorts in the split range: stable argsort equal to numpy's."""
    for n in (1 << 15, 123_457, 1 << 20):
        keys = gqs_ctypes.generate("u32", "distinct16", 77 + n, n)
        idx = gpu_ctx.argsort(keys)
        assert np.array_equal(idx, np.argsort(keys, kind="stable").astype(np.uint32))
