"""Benchmark: GPU-Quicksort on GB300, one JSON line.

Default workload (the metric's configuration): one plain sort of 2^28 uint32 keys drawn
uniformly over [0, 2^32) from a fixed seed. A step is one sort of that array.

  value     keys/s with the keys already in HBM (device-pointer C ABI call, CUDA events around
            each sort on the launching stream; the input is restored between steps outside the
            timed interval; 1 GiB of keys exceeds the 129 MB L2, and the restore copy rewrites it)
  e2e       the same metric through the host-pointer C ABI call (pinned host buffer -> HBM,
            sort, -> host), wall clock per call
  roofline  algorithmic bytes of the persistent kernel (key bytes * 2 * keys read by partition
            chunks + keys sorted on chip + keys sorted in registers, from the kernel's own
            counters) / its CUDA-event duration, against the measured HBM copy bandwidth

  configs   every other configuration of the benchmark, each with its own kernel time, roofline
            fraction, clock record and a bit-exact check against the std::sort digest committed in
            tests/golden/full_size.json: 2^20 u32; 2^28 u32 sorted / reverse / 16 distinct /
            Zipf(1.1) / Gaussian; 2^27 f32 N(0, 1e3); 2^26 f64 U[-1e9, 1e9]; the batched sort of
            4096 arrays (autotuned variant, against one plain call per array, end to end)
  phases    the split of the 2^28 kernel's time between partition chunks and on-chip sorts

Options: --impl reference times the reference's CPU path (the oracle's restatement of
GPUQSort<T>, all host threads) on the same 2^28 array, beside std::sort on one core and the
parallel std::sort on all cores; --config batched runs the segmented form alone.
Multi-GPU (torchrun): every rank sorts its own array (replicas; no collective on the data path).
"""
from __future__ import annotations

import argparse
import gc
import hashlib
import json
import math
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gpu-quicksort_gb300")
sys.path.insert(0, PKG)

SEED = 20260301
L2_BYTES = 129 * 1024 * 1024

METRIC = "Gkeys/s @2^28 u32"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="plain", choices=["plain", "batched", "tiles", "serve", "pairs"])
    p.add_argument("--dtype", default="u32", choices=["u32", "f32", "f64"])
    p.add_argument("--dist", default="uniform")
    p.add_argument("--log2n", type=int, default=28)
    p.add_argument("--variant", type=int, default=-1)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-clocks", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the list of the other configurations")
    p.add_argument("--profile", action="store_true", help="use libgqs_prof.so and print its cycle counters")
    p.add_argument("--serve-requests", type=int, default=20000,
                   help="requests of the serving stream (--config serve, and the summary in the plain line; 0: skip)")
    p.add_argument("--serve-load", type=float, default=0.5,
                   help="Poisson offered load as a fraction of each server's measured saturation capacity "
                        "(Poisson arrivals form smaller batches than saturation, so the batched server's "
                        "capacity under them is lower: 0.7 sits at its edge)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, dist):
    """The largest value of x over all ranks; x itself without a process group."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_name(args, n, batched=False):
    if batched or args.config == "batched":
        return f"batched segmented sort: 4096 uint32 arrays, lengths log-uniform in [32, 2^20], {n} keys"
    if args.config == "tiles":
        return f"segmented sort of 8000-key {args.dtype} arrays (on-chip sort only), {n} keys"
    return f"plain sort, 2^{args.log2n} {args.dtype} keys, {args.dist}"


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic(workload_key):
    """Per-launch DRAM bytes of the persistent kernel from a committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(workload_key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi samples (every 50 ms) of the SM clock and the throttle reasons, read by a thread
    as they arrive and stamped with the host's monotonic clock, so that each timed region can be
    given the samples taken during it."""

    REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, enabled, index=0):
        self.proc = None
        self.samples = []  # (t, sm_mhz, sm_max_mhz, reasons)
        self.lock = threading.Lock()
        if not enabled:
            return
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm, mx = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            reasons = {nm for nm, v in zip(self.REASONS, parts[5:9]) if v.lower() == "active"}
            with self.lock:
                self.samples.append((time.perf_counter(), sm, mx, reasons))

    def ready(self, timeout=5.0):
        """Waits until the first sample has arrived (the sampler takes a moment to start)."""
        t_end = time.perf_counter() + timeout
        while self.proc and time.perf_counter() < t_end:
            with self.lock:
                if self.samples:
                    return True
            time.sleep(0.02)
        return False

    def window(self, t0=None, t1=None):
        """Summary of the samples taken in [t0, t1] (all samples without bounds); a region shorter
        than the sampling interval gets the nearest sample on each side."""
        if not self.proc:
            return None
        time.sleep(0.06)  # let the sample that closes the region arrive
        with self.lock:
            smp = list(self.samples)
        if not smp:
            return None
        if t0 is not None:
            inside = [x for x in smp if t0 <= x[0] <= t1]
            if not inside:
                before = [x for x in smp if x[0] < t0][-1:]
                after = [x for x in smp if x[0] > t1][:1]
                inside = before + after
            smp = inside or smp[-1:]
        sm = [x[1] for x in smp]
        reasons = set().union(*[x[3] for x in smp])
        return {"sm_mhz": float(np.median(sm)), "sm_min_mhz": float(min(sm)),
                "sm_max_mhz": float(max(x[2] for x in smp)), "reasons": sorted(reasons), "samples": len(smp)}

    def stop(self):
        summary = self.window()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.proc = None
        return summary


# ---------------------------------------------------------------------------
# Bit-exact checks against the committed std::sort digests of every configuration

def sha256_of(a) -> str:
    return hashlib.sha256(memoryview(np.ascontiguousarray(a)).cast("B")).hexdigest()


def golden_case(dtype, dist, n, seed, kind="plain"):
    """The std::sort digest of one configuration (tests/golden/full_size.json), or None."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "full_size.json")) as f:
            cases = json.load(f)["cases"]
    except Exception:
        return None
    for c in cases:
        if c["kind"] == kind and c["dtype"] == dtype and c["dist"] == dist and c["n"] == n and c["seed"] == seed:
            return c
    return None


def golden_check(case, host_in, host_out):
    """Compares the seeded input and the GPU's output (host arrays) with the golden digests."""
    if case is None:
        return {"golden": "no committed digest for this input"}
    return {"input_sha256_equal_to_golden": sha256_of(host_in) == case["input_sha256"],
            "bit_exact_vs_std_sort_digest": sha256_of(host_out) == case["sorted_sha256"]}


def cpu_baseline(args, n_full):
    """The oracle's restatement of GPUQSort<T> on all host threads, on a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gqs_ctypes
    import oracle_ctypes
    threads = os.cpu_count() or 1
    ns = min(n_full, 1 << 25)
    a = gqs_ctypes.generate(args.dtype, args.dist, SEED, ns)
    b = a.copy()
    t0 = time.perf_counter()
    oracle_ctypes.gpuqsort(b, threads=threads)
    t = time.perf_counter() - t0
    # the reference's own CPU baseline, std::sort on one core, on a smaller sample
    ns1 = min(n_full, 1 << 24)
    c = a[:ns1].copy()
    t1 = time.perf_counter()
    oracle_ctypes.std_sort(c)
    t_std = time.perf_counter() - t1
    # the reference's own CPU quicksort<T> (GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:213-259,
    # unused by its driver), restated in the oracle, one core
    d = a[:ns1].copy()
    t2 = time.perf_counter()
    oracle_ctypes.cpu_quicksort(d)
    t_q = time.perf_counter() - t2
    # the reference's parallel CPU sort (tbb::parallel_sort, QuicksortMain.cpp:993), here GCC's
    # parallel mode sort on all threads
    e = a.copy()
    t3 = time.perf_counter()
    oracle_ctypes.parallel_sort(e, threads)
    t_p = time.perf_counter() - t3
    return {"value": ns / t / 1e9, "unit": "Gkeys/s", "cores": threads, "kind": "port",
            "sample": f"GPUQSort<T> restatement (oracle/gqs_oracle.cpp) on {ns} {args.dtype} keys of the same "
                      f"distribution, {threads} threads, one sort of {t:.3f} s",
            "std_sort_1core": {"value": ns1 / t_std / 1e9, "unit": "Gkeys/s", "keys": ns1},
            "reference_cpu_quicksort_1core": {"value": ns1 / t_q / 1e9, "unit": "Gkeys/s", "keys": ns1,
                                              "bit_exact_vs_std_sort": bool(np.array_equal(c, d))},
            "parallel_sort_all_cores": {"value": ns / t_p / 1e9, "unit": "Gkeys/s", "keys": ns, "threads": threads,
                                        "what": "__gnu_parallel::sort, standing in for tbb::parallel_sort"},
            "cpu": platform.processor() or platform.machine()}


def run_reference(args):
    """The reference's CPU path on the benchmark's own array (2^log2n keys, not a sample): the
    oracle's restatement of GPUQSort<T> on all host threads, `warmup` + `steps` sorts; beside it,
    once each on the same array, std::sort on one core (the reference's verifier) and GCC's
    parallel sort on all cores (for the reference's tbb::parallel_sort)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gqs_ctypes
    import oracle_ctypes
    threads = os.cpu_count() or 1
    n = 1 << args.log2n
    a = gqs_ctypes.generate(args.dtype, args.dist, SEED, n)
    b = np.empty_like(a)
    for _ in range(args.warmup):
        np.copyto(b, a)
        oracle_ctypes.gpuqsort(b, threads=threads)
    times = []
    for _ in range(args.steps):
        np.copyto(b, a)
        t0 = time.perf_counter()
        oracle_ctypes.gpuqsort(b, threads=threads)
        times.append(time.perf_counter() - t0)
    v = n * len(times) / sum(times) / 1e9
    np.copyto(b, a)
    t0 = time.perf_counter()
    oracle_ctypes.std_sort(b)
    t_std = time.perf_counter() - t0
    c = a.copy()
    t0 = time.perf_counter()
    oracle_ctypes.parallel_sort(c, threads)
    t_par = time.perf_counter() - t0
    same = bool(np.array_equal(b, c))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gkeys/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
            "config": {"workload": workload_name(args, n), "keys": n, "seed": SEED},
            "cpu_baseline": {"value": v, "unit": "Gkeys/s", "cores": threads, "kind": "port",
                             "sample": f"the whole {n}-key array every step (no sample): the oracle's restatement "
                                       "of GPUQSort<T> (oracle/gqs_oracle.cpp), all host threads",
                             "std_sort_1core": {"value": n / t_std / 1e9, "unit": "Gkeys/s", "keys": n,
                                                "s": t_std},
                             "parallel_sort_all_cores": {"value": n / t_par / 1e9, "unit": "Gkeys/s", "keys": n,
                                                         "threads": threads, "s": t_par,
                                                         "what": "__gnu_parallel::sort, for tbb::parallel_sort"},
                             "std_sort_equal_to_parallel_sort": same,
                             "cpu": platform.processor() or platform.machine()},
            "e2e": {"value": v, "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class CudaView:
    """Exposes a raw device pointer to torch.as_tensor (no copy)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2}


# ---------------------------------------------------------------------------
# Serving stream: 60/30/10 % u32/f32/f64 requests, sizes log-uniform in [2^10, 2^24]

SERVE_DIST = {"u32": "uniform", "f32": "gaussian", "f64": "uniform"}
SERVE_TYPES = ("u32", "f32", "f64")


class OutPool:
    """First-fit allocator over one pinned host buffer for request outputs (the client-side
    window: a submit waits while the buffer holds no room). Blocks are freed in any order and
    merged with free neighbours, so one slow request does not hold back the space behind it.
    Records how long allocations waited."""

    def __init__(self, nbytes):
        import threading
        import torch
        self.buf = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        self.base = self.buf.data_ptr()
        self.size = nbytes
        self.free_list = [[0, nbytes]]  # [start, end), sorted by start, never adjacent
        self.cv = threading.Condition()
        self.wait_s = 0.0
        self.waits = 0

    def alloc(self, nbytes):
        nbytes = (nbytes + 255) // 256 * 256
        t0 = None
        with self.cv:
            while True:
                for blk in self.free_list:
                    if blk[1] - blk[0] >= nbytes:
                        lo = blk[0]
                        blk[0] += nbytes
                        if blk[0] == blk[1]:
                            self.free_list.remove(blk)
                        if t0 is not None:
                            self.wait_s += time.perf_counter() - t0
                            self.waits += 1
                        return [lo, lo + nbytes]
                if t0 is None:
                    t0 = time.perf_counter()
                self.cv.wait()

    def free(self, rec):
        import bisect
        lo, hi = rec
        with self.cv:
            fl = self.free_list
            k = bisect.bisect_left([b[0] for b in fl], lo)
            if k > 0 and fl[k - 1][1] == lo:
                fl[k - 1][1] = hi
                if k < len(fl) and fl[k][0] == hi:
                    fl[k - 1][1] = fl[k][1]
                    del fl[k]
            elif k < len(fl) and fl[k][0] == hi:
                fl[k][0] = lo
            else:
                fl.insert(k, [lo, hi])
            self.cv.notify_all()


def serve_stream(count, seed):
    rng = np.random.default_rng(seed)
    u = rng.random(count)
    dt = np.where(u < 0.6, 0, np.where(u < 0.9, 1, 2))
    n = np.exp(rng.uniform(np.log(2.0 ** 10), np.log(2.0 ** 24), count)).astype(np.int64)
    src = (rng.integers(0, 1 << 20, count) // 64) * 64
    return dt, n, src


def run_serve_arm(gqs_ctypes, templates, stream, per_request, rate, pool, sample_every=97):
    """Runs the stream through one server. rate None: saturation (submit as fast as the output
    window allows); else Poisson arrivals at `rate` requests/s. Returns latencies and samples."""
    import threading
    dt, n, src = stream
    count = len(n)
    srv = gqs_ctypes.Server(budget_bytes=64 << 30, batch_keys=1 << 27, batch_segments=4096, lanes=3,
                            per_request=per_request)
    esz = [4, 4, 8]
    arrive = np.zeros(count)
    if rate:
        arrive = np.cumsum(np.random.default_rng(12345).exponential(1.0 / rate, count))
    info = [None] * count
    recs = [None] * count
    idx_of = {}
    samples = {}
    lock = threading.Lock()

    def collect():
        got = 0
        while got < count:
            code, rid, inf = srv.wait_any(60000)
            if code == 4 and rid == 0:
                raise RuntimeError("serving stream stalled")
            with lock:
                i = idx_of.pop(rid)
            if code != 0:
                raise RuntimeError(f"request {i} failed: {gqs_ctypes.STATUS.get(code, code)}")
            info[i] = inf
            if i % sample_every == 0 and n[i] <= (1 << 21):
                a = np.frombuffer(pool.buf.numpy(), dtype=gqs_ctypes.NP_DTYPES[SERVE_TYPES[dt[i]]],
                                  count=int(n[i]), offset=recs[i][0])
                samples[i] = a.copy()
            pool.free(recs[i])
            got += 1

    col = threading.Thread(target=collect)
    # no garbage-collector pauses inside the measured stream (they would show as request
    # latency of the Python load generator, not of the server)
    gc.collect()
    gc.disable()
    col.start()
    t0 = srv.now_ns()
    t_wall0 = time.perf_counter()
    w0, nw0 = pool.wait_s, pool.waits
    call_s = np.zeros(count)
    for i in range(count):
        if rate:
            delay = arrive[i] - (time.perf_counter() - t_wall0)
            if delay > 0:
                time.sleep(delay)
        t = SERVE_TYPES[dt[i]]
        nb = int(n[i]) * esz[dt[i]]
        rec = pool.alloc(nb)
        recs[i] = rec
        tmpl = templates[t]
        tc = time.perf_counter()
        with lock:
            rid = srv.submit_raw(t, tmpl.data_ptr() + int(src[i]) * esz[dt[i]], pool.base + rec[0], int(n[i]))
            idx_of[rid] = i
        call_s[i] = time.perf_counter() - tc
    col.join()
    gc.enable()
    st = srv.stats()
    srv.close()
    done = np.array([x["t_done_ns"] for x in info], dtype=np.float64)
    sub = np.array([x["t_submit_ns"] for x in info], dtype=np.float64)
    adm = np.array([x["t_admit_ns"] for x in info], dtype=np.float64)
    lau = np.array([x["t_launch_ns"] for x in info], dtype=np.float64)
    arr_ns = t0 + arrive * 1e9 if rate else sub
    lat_ms = (done - np.minimum(arr_ns, sub)) / 1e6
    span = (done.max() - min(t0, sub.min())) / 1e9
    # where the latency goes, per key type: arrival -> submit (the load generator's own lag),
    # submit -> admit (waiting for arena memory), admit -> launch (resident, waiting for a lane
    # and for its type's turn), launch -> done (its batch's sort and copy back)
    split = {}
    for k, t in enumerate(SERVE_TYPES):
        m = dt == k
        if not m.any():
            continue
        parts = {"arrive_submit": (sub[m] - np.minimum(arr_ns[m], sub[m])) / 1e6, "submit_admit": (adm[m] - sub[m]) / 1e6,
                 "admit_launch": (lau[m] - adm[m]) / 1e6, "launch_done": (done[m] - lau[m]) / 1e6,
                 "total": lat_ms[m]}
        split[t] = {name: {"p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99))}
                    for name, v in parts.items()}
        split[t]["requests"] = int(m.sum())
    client = {"output_window_waits": pool.waits - nw0, "output_window_wait_s": pool.wait_s - w0,
              "submit_call_p99_ms": float(np.percentile(call_s, 99) * 1e3),
              "submit_call_max_ms": float(call_s.max() * 1e3)}
    srv_ms = (done - sub) / 1e6
    return {"keys_per_s": float(n.sum()) / span, "span_s": span, "lat_ms": lat_ms, "split": split,
            "server_p50_ms": float(np.percentile(srv_ms, 50)), "server_p99_ms": float(np.percentile(srv_ms, 99)),
            "client": client,
            "batches": st["batches"], "max_batch_requests": st["max_batch_requests"],
            "arena_peak_gb": st["arena_peak"] / 1e9}, samples


def run_serve(args, gqs_ctypes):
    """The serving comparison: batched server vs per-request plain sorts on the same stream."""
    import torch
    count = args.serve_requests
    stream = serve_stream(count, SEED)
    dt, n, src = stream
    templates = {}
    for k, t in enumerate(SERVE_TYPES):
        tdt = {"u32": torch.int32, "f32": torch.float32, "f64": torch.float64}[t]
        buf = torch.empty((1 << 24) + (1 << 20), dtype=tdt, pin_memory=True)
        v = buf.numpy().view(gqs_ctypes.NP_DTYPES[t])
        gqs_ctypes.generate(t, SERVE_DIST[t], SEED + 7 * k, v.size, out=v)
        templates[t] = buf
    pool = OutPool(6 << 30)
    # warm-up: a short stream through both modes (graph capture, pool growth)
    warm = serve_stream(64, SEED + 1)
    run_serve_arm(gqs_ctypes, templates, warm, False, None, pool)
    run_serve_arm(gqs_ctypes, templates, warm, True, None, pool)
    sat_b, samp_b = run_serve_arm(gqs_ctypes, templates, stream, False, None, pool)
    sat_p, samp_p = run_serve_arm(gqs_ctypes, templates, stream, True, None, pool)
    mean_keys = float(n.mean())
    rate = args.serve_load * sat_b["keys_per_s"] / mean_keys
    poi_b, _ = run_serve_arm(gqs_ctypes, templates, stream, False, rate, pool)
    poi_p, _ = run_serve_arm(gqs_ctypes, templates, stream, True, rate, pool)
    # the same stream at the per-request server's own load point, which both modes sustain
    rate_p = args.serve_load * sat_p["keys_per_s"] / mean_keys
    low_b, _ = run_serve_arm(gqs_ctypes, templates, stream, False, rate_p, pool)
    low_p, _ = run_serve_arm(gqs_ctypes, templates, stream, True, rate_p, pool)
    # bit-exact checks on the sampled requests: both modes, against numpy's sort of the input
    ok = True
    for i, a in samp_b.items():
        t = SERVE_TYPES[dt[i]]
        ref = np.sort(templates[t].numpy().view(gqs_ctypes.NP_DTYPES[t])[src[i]:src[i] + n[i]])
        ok &= bool(np.array_equal(a.view(np.uint8), ref.view(np.uint8)))
        if i in samp_p:
            ok &= bool(np.array_equal(a.view(np.uint8), samp_p[i].view(np.uint8)))

    def lat(r):
        return {"p50_ms": float(np.percentile(r["lat_ms"], 50)), "p99_ms": float(np.percentile(r["lat_ms"], 99)),
                "gkeys_s": r["keys_per_s"] / 1e9, "span_s": r["span_s"], "batches": r["batches"],
                "server_p50_ms": r["server_p50_ms"], "server_p99_ms": r["server_p99_ms"], "client": r["client"],
                "split_by_type": r["split"]}

    total_keys = int(n.sum())
    in_bytes = int(sum(int(n[i]) * (8 if dt[i] == 2 else 4) for i in range(count)))
    return {
        "requests": count, "keys": total_keys, "bytes_each_way": in_bytes,
        "mix": "60/30/10 % u32/f32/f64", "sizes": "log-uniform in [2^10, 2^24]",
        "values": "u32 uniform, f32 N(0, 1e3), f64 U[-1e9, 1e9]",
        "server": {"budget_gb": 64, "lanes": 3, "batch_keys": 1 << 27, "batch_segments": 4096},
        "host_buffers": "pinned inputs and outputs",
        "saturation": {"batched_gkeys_s": sat_b["keys_per_s"] / 1e9, "per_request_gkeys_s": sat_p["keys_per_s"] / 1e9,
                       "speedup": sat_b["keys_per_s"] / sat_p["keys_per_s"], "batched_batches": sat_b["batches"],
                       "batched_max_batch_requests": sat_b["max_batch_requests"],
                       "batched_arena_peak_gb": sat_b["arena_peak_gb"]},
        "poisson": {"offered_load": f"{args.serve_load:.2f} x batched capacity", "rate_req_s": rate,
                    "offered_gkeys_s": rate * mean_keys / 1e9, "batched": lat(poi_b), "per_request": lat(poi_p)},
        "poisson_per_request_load": {"offered_load": f"{args.serve_load:.2f} x per-request capacity",
                                     "rate_req_s": rate_p, "offered_gkeys_s": rate_p * mean_keys / 1e9,
                                     "batched": lat(low_b), "per_request": lat(low_p)},
        "check": {"sampled_requests": len(samp_b), "bit_exact_vs_numpy_and_per_request": ok},
    }


def run_pairs(args, gqs_ctypes, rank, local, world, dist, barrier):
    """Key-value sort: 2^log2n u32 (or f32) keys, each carrying its uint32 index."""
    import torch
    n = 1 << args.log2n
    dtype = args.dtype if args.dtype in ("u32", "f32") else "u32"
    keys = gqs_ctypes.generate(dtype, args.dist if dtype == "u32" else "gaussian", SEED + rank, n)
    kp = torch.from_numpy(keys.view(np.int32)).cuda()
    vp = torch.arange(n, dtype=torch.int32, device="cuda")
    k, v = torch.empty_like(kp), torch.empty_like(vp)
    ctx = gqs_ctypes.Context(device=local, sync=False, timing=True)
    stream = torch.cuda.current_stream()

    def step():
        rc = ctx.sort_pairs_dev(dtype, k.data_ptr(), v.data_ptr(), n, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"pair sort failed: {gqs_ctypes.STATUS.get(rc, rc)}")

    for _ in range(args.warmup):
        k.copy_(kp)
        v.copy_(vp)
        step()
        if ctx.stats()["status"] != 0:
            raise RuntimeError("pair sort failed")
    order = torch.sort(kp.to(torch.int64) & 0xFFFFFFFF if dtype == "u32" else kp.view(torch.float32),
                       stable=True).indices
    check = {"stable_argsort_equal_to_torch": bool(torch.equal(v.to(torch.int64), order))}
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    kms = []
    barrier()
    for i in range(args.steps):
        k.copy_(kp)
        v.copy_(vp)
        ev0[i].record(stream)
        step()
        ev1[i].record(stream)
        st = ctx.stats()
        kms.append(st["kernel_ms"])
    torch.cuda.synchronize()
    barrier()
    t = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)) / 1e3, dist)
    ctx.close()
    if rank != 0:
        return None
    peak, peak_src = measured_peak()
    km = float(np.mean(kms))
    ab = float(st["algo_bytes"])
    return {"metric": f"Gpairs/s (key-value sort, 2^{args.log2n} {dtype} keys + uint32 values)",
            "value": n * world * args.steps / t / 1e9, "unit": "Gpairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": f"{dtype} keys + u32 values (packed u64 words)",
            "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
            "config": {"workload": f"key-value sort of 2^{args.log2n} pairs", "keys": n,
                       "l2": "inputs larger than L2 (rewritten from pristine copies before every step)"},
            "roofline": {"bound": "hbm", "achieved": ab / (km / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": ab / (km / 1e3) / 1e9 / peak, "kernel": "gqs::persistent_kernel (u64 words)",
                         "kernel_ms": km, "algo_bytes_per_launch": ab, "peak_source": peak_src},
            "check": check, "gpu_launches": 4 * args.steps}


def run_batched(args, gqs_ctypes, rank, local, world, dist, barrier, clocks=None, steps=None, warmup=None):
    """4096 uint32 arrays, lengths log-uniform in [32, 2^20], as one graph-captured batch: the
    autotuned variant's replays (value, roofline), the same arrays by one plain call each, and
    the batch end to end through its host copy calls."""
    import torch
    steps = steps or args.steps
    warmup = warmup or args.warmup
    nseg = 4096
    off = gqs_ctypes.segment_offsets(SEED + rank, nseg, 32, 1 << 20)
    n = int(off[-1])
    esize = 4
    host_in = torch.empty(n, dtype=torch.int32, pin_memory=True)
    hv = host_in.numpy().view(np.uint32)
    gqs_ctypes.generate("u32", "uniform", SEED + rank, n, out=hv)
    batch = gqs_ctypes.Batch("u32", n, nseg, device=local, variant=args.variant)
    batch.set_segments(off)
    batch.copy_in(hv)
    arena = torch.as_tensor(CudaView(batch.keys_ptr, n, "<i4"), device="cuda")
    pristine = host_in.cuda()
    tune = None
    if args.variant < 0:
        best, ms = batch.autotune(nseg, reps=2)
        tune = {"chosen": gqs_ctypes.variants("u32")[best]["name"],
                "median_ms": {gqs_ctypes.variants("u32")[v]["name"]: m for v, m in enumerate(ms)}}
    stream = torch.cuda.current_stream()
    own_clocks = clocks is None
    if own_clocks:
        clocks = ClockSampler(enabled=(not args.no_clocks and rank == 0), index=local)
        clocks.ready()

    def step():
        rc = batch.launch(nseg, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"batch launch failed: {gqs_ctypes.STATUS.get(rc, rc)}")

    for _ in range(warmup):
        arena.copy_(pristine)
        step()
        code, st = batch.wait()
        if code != 0:
            raise RuntimeError(f"batch failed: {st}")
    # bit-exact checks of the last warm-up result: the std::sort digest of the whole output and of
    # every segment, and (segment, key) pairs sorted lexicographically by torch
    out_h = torch.empty_like(host_in, pin_memory=True)
    ov = out_h.numpy().view(np.uint32)
    out_h.copy_(arena)
    case = golden_case("u32", "uniform", n, SEED + rank, kind="segments")
    check = golden_check(case, hv, ov)
    if case is not None:
        bad = [i for i in range(nseg)
               if hashlib.sha256(memoryview(ov[int(off[i]):int(off[i + 1])]).cast("B")).hexdigest()[:16]
               != case["segment_sha256_16"][i]]
        check["segments_equal_to_std_sort_digest"] = nseg - len(bad)
        check["first_bad_segment"] = bad[0] if bad else None
    seg_id = torch.repeat_interleave(torch.arange(nseg, device="cuda", dtype=torch.int64),
                                     torch.from_numpy(np.diff(off).astype(np.int64)).cuda())
    keyed = (seg_id << 32) | (pristine.to(torch.int64) & 0xFFFFFFFF)
    ref = torch.sort(keyed).values & 0xFFFFFFFF
    check["bit_exact_vs_torch_sort_per_segment"] = bool(torch.equal(arena.to(torch.int64) & 0xFFFFFFFF, ref))
    del seg_id, keyed, ref
    torch.cuda.empty_cache()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    kms, abytes = [], []
    barrier()
    torch.cuda.synchronize()
    t_0 = time.perf_counter()
    for i in range(steps):
        arena.copy_(pristine)
        ev0[i].record(stream)
        step()
        ev1[i].record(stream)
        code, st = batch.wait()
        if code != 0:
            raise RuntimeError(f"batch failed: {st}")
        kms.append(st["kernel_ms"])
        abytes.append(st["algo_bytes"])
    torch.cuda.synchronize()
    barrier()
    t_1 = time.perf_counter()
    clk = clocks.window(t_0, t_1)
    if own_clocks:
        clocks.stop()
    t = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)) / 1e3, dist)
    value = n * world * steps / t / 1e9
    # end to end through the public batch calls: pinned host -> arena, replay, arena -> host
    times = []
    for i in range(steps + 1):
        t0 = time.perf_counter()
        batch.copy_in(hv)
        step()
        code, _ = batch.wait()
        batch.copy_out(ov)
        if i:
            times.append(time.perf_counter() - t0)
    tsum = max_over_ranks(sum(times), dist)
    e2e = {"value": n * world * steps / tsum / 1e9, "unit": "Gkeys/s", "h2d_bytes_per_step": n * esize,
           "d2h_bytes_per_step": n * esize, "ms_per_step": 1e3 * tsum / steps,
           "api": "gqs_batch_copy_in + gqs_batch_launch + gqs_batch_wait + gqs_batch_copy_out (pinned)",
           "check": golden_check(case, hv, ov)}
    # the same arrays sorted by one plain call each (device pointers, enqueued back to back)
    ctx = gqs_ctypes.Context(device=local, sync=False, timing=False, variant=0)
    d = pristine.clone()
    dn = torch.empty_like(d)
    ctx.reserve("u32", int(np.diff(off).max()), 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(nseg):
        rc = ctx.sort_dev("u32", d.data_ptr() + int(off[i]) * 4, dn.data_ptr() + int(off[i]) * 4,
                          int(off[i + 1] - off[i]), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("plain sort failed")
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_same = bool(torch.equal(d, arena))
    ctx.close()
    chosen = gqs_ctypes.variants("u32")[batch.variant]["name"]
    batch.close()
    del d, dn, arena, pristine
    torch.cuda.empty_cache()
    if rank != 0:
        return None
    peak, peak_src = measured_peak()
    km, ab = float(np.mean(kms)), float(np.mean(abytes))
    achieved = ab / (km / 1e3) / 1e9
    return {
        "metric": f"Gkeys/s ({workload_name(args, n, batched=True)})", "workload": workload_name(args, n, batched=True),
        "value": value, "unit": "Gkeys/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
        "config": {"workload": workload_name(args, n, batched=True), "keys": n, "segments": nseg, "seed": SEED,
                   "l2": "inputs larger than L2 (arena rewritten from a pristine copy before every step)",
                   "variant": chosen,
                   "graph": "one cudaGraphLaunch per step", "parallelism": f"replicas x{world}"},
        "autotune": tune,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": ncu_traffic("batched_u32"), "kernel": "gqs::persistent_kernel (graph replay)",
                     "kernel_ms": km, "algo_bytes_per_launch": ab, "peak_source": peak_src},
        "kernel_ms": km,
        "plain_per_array": {"gkeys_s": n / (plain_ms / 1e3) / 1e9, "ms": plain_ms, "calls": nseg,
                            "same_output": plain_same, "batched_speedup": value / (n / (plain_ms / 1e3) / 1e9)},
        "cpu_baseline": None, "e2e": e2e, "gpu_launches": 2 * steps, "clocks": clk, "check": check,
    }


def run_tiles(args, gqs_ctypes, rank, local, world, dist, barrier, peak, peak_src):
    """The on-chip sort alone: a segmented sort of 8000-key arrays (6000 for f64), every array
    one tile, so the kernel does no partition chunk."""
    import torch
    npdt = gqs_ctypes.NP_DTYPES[args.dtype]
    esize = np.dtype(npdt).itemsize
    seg = 6000 if args.dtype == "f64" else 8000
    nseg = (1 << args.log2n) // seg
    off = np.arange(nseg + 1, dtype=np.int64) * seg
    n = int(off[-1])
    offsets = torch.from_numpy(off).cuda()
    host_in = torch.empty(n * esize, dtype=torch.uint8, pin_memory=True)
    hv = host_in.numpy().view(npdt)
    gqs_ctypes.generate(args.dtype, args.dist, SEED + rank, n, out=hv)
    pristine = host_in.cuda()
    d, dn = torch.empty_like(pristine), torch.empty_like(pristine)
    ctx = gqs_ctypes.Context(device=local, sync=False, timing=True, variant=args.variant)
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(enabled=(not args.no_clocks and rank == 0), index=local)
    clocks.ready()

    def sort_once():
        rc = ctx.sort_segments_dev(args.dtype, d.data_ptr(), dn.data_ptr(), n, offsets.data_ptr(), nseg,
                                   stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"sort enqueue failed: {gqs_ctypes.STATUS.get(rc, rc)}")

    for _ in range(args.warmup):
        d.copy_(pristine)
        sort_once()
        if ctx.stats()["status"] != 0:
            raise RuntimeError("sort failed")
    out = d.cpu().numpy().view(npdt)
    ok = all(np.array_equal(out[int(off[i]):int(off[i + 1])], np.sort(hv[int(off[i]):int(off[i + 1])]))
             for i in range(0, nseg, max(1, nseg // 64)))
    kms, abytes, step_ms = [], [], []
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        d.copy_(pristine)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sort_once()
        e1.record(stream)
        st = ctx.stats()
        if st["status"] != 0:
            raise RuntimeError("sort failed")
        kms.append(st["kernel_ms"])
        abytes.append(st["algo_bytes"])
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier()
    clk = clocks.window(t0, time.perf_counter())
    clocks.stop()
    phases = ctx.phases()
    ctx.close()
    t = max_over_ranks(sum(step_ms) / 1e3, dist)
    km, ab = float(np.mean(kms)), float(np.mean(abytes))
    return {"metric": f"Gkeys/s ({workload_name(args, n)})", "value": n * world * args.steps / t / 1e9,
            "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.dtype, "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
            "config": {"workload": workload_name(args, n), "keys": n, "segments": nseg, "segment_keys": seg,
                       "variant": gqs_ctypes.variants(args.dtype)[st["variant"]]["name"]},
            "roofline": {"bound": "hbm", "achieved": ab / (km / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": ab / (km / 1e3) / 1e9 / peak, "kernel_ms": km, "algo_bytes_per_launch": ab,
                         "peak_source": peak_src},
            "kernel_gkeys_s": n / (km / 1e3) / 1e9, "phases": phases, "clocks": clk,
            "check": {"sampled_segments_equal_numpy_sort": bool(ok)}, "gpu_launches": 2 * args.steps}


class PlainRunner:
    """Times plain device-pointer sorts of one configuration at a time on one context, with the
    keys resident in HBM: buffers are sized once for the largest configuration; the seeded input
    is generated into pinned host memory and copied to a pristine device copy, which is copied
    over the sort's buffer before every step, outside the timed interval."""

    def __init__(self, gqs_ctypes, local, rank, max_bytes, variant):
        import torch
        self.torch = torch
        self.gq = gqs_ctypes
        self.rank = rank
        self.host_in = torch.empty(max_bytes, dtype=torch.uint8, pin_memory=True)
        self.host_out = torch.empty(max_bytes, dtype=torch.uint8, pin_memory=True)
        self.pristine = torch.empty(max_bytes, dtype=torch.uint8, device="cuda")
        self.d = torch.empty(max_bytes, dtype=torch.uint8, device="cuda")
        self.dn = torch.empty(max_bytes, dtype=torch.uint8, device="cuda")
        self.flush = None
        self.ctx = gqs_ctypes.Context(device=local, sync=False, timing=True, variant=variant)
        self.stream = torch.cuda.current_stream()

    def host_view(self, buf, dtype, n):
        return buf.numpy()[: n * np.dtype(self.gq.NP_DTYPES[dtype]).itemsize].view(self.gq.NP_DTYPES[dtype])

    def prepare(self, dtype, dist, n, seed):
        hv = self.host_view(self.host_in, dtype, n)
        self.gq.generate(dtype, dist, seed, n, out=hv)
        nb = hv.nbytes
        self.pristine[:nb].copy_(self.host_in[:nb], non_blocking=False)
        return hv

    def sort_once(self, dtype, n):
        rc = self.ctx.sort_dev(dtype, self.d.data_ptr(), self.dn.data_ptr(), n, self.stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"sort enqueue failed: {self.gq.STATUS.get(rc, rc)}")

    def run(self, dtype, dist, log2n, warmup, steps, clocks, seed, min_time_s=0.0, torch_check=False,
            barrier=lambda: None):
        """Warm-up sorts, the bit-exact check of the last one, then `steps` timed sorts (more when
        min_time_s asks for a longer timed region). Returns the timings and the check."""
        torch = self.torch
        n = 1 << log2n
        esize = np.dtype(self.gq.NP_DTYPES[dtype]).itemsize
        nb = n * esize
        hv = self.prepare(dtype, dist, n, seed)
        # inputs smaller than twice the L2 are timed after an L2 flush (a 256 MiB write) per step
        if nb < 2 * L2_BYTES and self.flush is None:
            self.flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        flush = self.flush if nb < 2 * L2_BYTES else None
        warm_ms = []
        for _ in range(warmup):
            self.d[:nb].copy_(self.pristine[:nb])
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self.sort_once(dtype, n)
            e1.record(self.stream)
            st = self.ctx.stats()
            if st["status"] != 0:
                raise RuntimeError(f"sort failed: {st}")
            warm_ms.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        # bit-exact check of the last warm-up result, outside any timed interval
        self.host_out[:nb].copy_(self.d[:nb])
        out = self.host_view(self.host_out, dtype, n)
        check = golden_check(golden_case(dtype, dist, n, seed), hv, out)
        if torch_check:
            tdt = {"u32": torch.int32, "f32": torch.float32, "f64": torch.float64}[dtype]
            src, got = self.pristine[:nb].view(tdt), self.d[:nb].view(tdt)
            if dtype == "u32":
                got, ref = got.to(torch.int64) & 0xFFFFFFFF, torch.sort(src.to(torch.int64) & 0xFFFFFFFF).values
            else:
                ref = torch.sort(src).values
            check["bit_exact_vs_torch_sort"] = bool(torch.equal(got, ref))
            del got, ref
            torch.cuda.empty_cache()
        if min_time_s > 0 and warm_ms:
            steps = min(400, max(steps, math.ceil(min_time_s / (min(warm_ms) / 1e3))))
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        kernel_ms, algo_bytes, st = [], [], None
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(steps):
            self.d[:nb].copy_(self.pristine[:nb])
            if flush is not None:
                flush.zero_()
            ev0[i].record(self.stream)
            self.sort_once(dtype, n)
            ev1[i].record(self.stream)
            st = self.ctx.stats()  # waits for this sort; kernel time from events on the launching stream
            if st["status"] != 0:
                raise RuntimeError(f"sort failed: {st}")
            kernel_ms.append(st["kernel_ms"])
            algo_bytes.append(st["algo_bytes"])
        torch.cuda.synchronize()
        barrier()
        t1 = time.perf_counter()
        step_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
        return {"n": n, "esize": esize, "steps": steps, "step_ms": step_ms, "kernel_ms": kernel_ms,
                "algo_bytes": algo_bytes, "stats": st, "check": check, "t0": t0, "t1": t1, "hv": hv,
                "clocks": clocks.window(t0, t1) if clocks else None,
                "l2": ("inputs larger than L2 (keys rewritten from a pristine copy before every step)"
                       if flush is None else "L2 flushed before every step (256 MiB write)")}


def roofline_of(r, peak, peak_src, traffic=None):
    km = float(np.mean(r["kernel_ms"]))
    ab = float(np.mean(r["algo_bytes"]))
    achieved = ab / (km / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": "gqs::persistent_kernel", "kernel_ms": km, "algo_bytes_per_launch": ab,
            "peak_source": peak_src,
            "per_unit": f"{r['esize']} B x 2 per key per pass (partition chunks + on-chip sort + register sort)"}


PLAIN_CONFIGS = [
    ("u32", "uniform", 20),
    ("u32", "sorted", 28),
    ("u32", "reverse", 28),
    ("u32", "distinct16", 28),
    ("u32", "zipf", 28),
    ("u32", "gaussian", 28),
    ("f32", "gaussian", 27),
    ("f64", "uniform", 26),
]


def run_configs(args, runner, clocks, peak, peak_src):
    """Every configuration of the benchmark other than the headline, one entry each."""
    out = []
    for dtype, dist, log2n in PLAIN_CONFIGS:
        r = runner.run(dtype, dist, log2n, warmup=max(3, args.warmup), steps=max(5, args.steps), clocks=clocks,
                       seed=SEED, min_time_s=0.25)
        t = sum(r["step_ms"]) / 1e3
        rf = roofline_of(r, peak, peak_src)
        st = r["stats"]
        v = runner.gq.variants(dtype)[st["variant"]]
        out.append({"workload": f"plain sort, 2^{log2n} {dtype} keys, {dist}", "dtype": dtype, "dist": dist,
                    "keys": r["n"], "value": r["n"] * r["steps"] / t / 1e9, "unit": "Gkeys/s",
                    "ms_per_step": 1e3 * t / r["steps"], "steps": r["steps"], "kernel_ms": rf["kernel_ms"],
                    "roofline": {"achieved": rf["achieved"], "frac": rf["frac"], "peak": peak,
                                 "algo_bytes_per_launch": rf["algo_bytes_per_launch"]},
                    "passes_per_key": (st["part_keys"] + st["local_keys"] + st["tiny_keys"]) / r["n"],
                    "variant": v["name"], "check": r["check"], "clocks": r["clocks"], "l2": r["l2"]})
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile and not os.environ.get("GQS_LIB"):
        import build_lib
        os.environ["GQS_LIB"] = build_lib.build(profile=True)["lib"]
    import torch
    import gqs_ctypes

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    else:
        dist = None

    def barrier():
        if dist is not None:
            dist.barrier()

    if args.config in ("batched", "pairs"):
        runner = run_batched if args.config == "batched" else run_pairs
        line = runner(args, gqs_ctypes, rank, local, world, dist, barrier)
        if line is not None:
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    if args.config == "serve":
        if rank == 0:
            sv = run_serve(args, gqs_ctypes)
            line = {"metric": "Gkeys/s (serving stream, batched server, saturation)",
                    "value": sv["saturation"]["batched_gkeys_s"], "unit": "Gkeys/s", "n_gpus": 1,
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "mixed u32/f32/f64",
                    "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
                    "config": {"workload": "serving stream of mixed sort requests"}, "serve": sv,
                    "e2e": {"value": sv["saturation"]["batched_gkeys_s"], "unit": "Gkeys/s",
                            "h2d_bytes_per_step": sv["bytes_each_way"], "d2h_bytes_per_step": sv["bytes_each_way"],
                            "step": "the whole stream"}}
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    npdt = gqs_ctypes.NP_DTYPES[args.dtype]
    esize = np.dtype(npdt).itemsize
    peak, peak_src = measured_peak()

    if args.config == "tiles":
        print(json.dumps(run_tiles(args, gqs_ctypes, rank, local, world, dist, barrier, peak, peak_src)), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    n = 1 << args.log2n
    want_configs = (not args.no_configs and world == 1 and args.dtype == "u32" and args.dist == "uniform"
                    and args.log2n == 28)
    max_bytes = n * esize
    if want_configs:
        max_bytes = max(max_bytes, max((1 << l2n) * np.dtype(gqs_ctypes.NP_DTYPES[t]).itemsize
                                       for t, _, l2n in PLAIN_CONFIGS))
    runner = PlainRunner(gqs_ctypes, local, rank, max_bytes, args.variant)
    # clocks are sampled from before the warm-up on, through every timed region
    clocks = ClockSampler(enabled=(not args.no_clocks and rank == 0), index=local)
    clocks.ready()
    r = runner.run(args.dtype, args.dist, args.log2n, args.warmup, args.steps, clocks, seed=SEED + rank,
                   torch_check=True, barrier=barrier)
    t_sort = max_over_ranks(sum(r["step_ms"]) / 1e3, dist)
    value = n * world * args.steps / t_sort / 1e9
    stats_last = r["stats"]
    phases = runner.ctx.phases()

    # ---- end to end through the host-pointer call
    e2e = None
    if not args.no_e2e:
        import torch as _t
        work = _t.empty(n * esize, dtype=_t.uint8, pin_memory=True)
        wv = work.numpy().view(npdt)
        for _ in range(max(1, min(args.warmup, 2))):
            np.copyto(wv, r["hv"])
            runner.ctx.sort(wv)
        times = []
        for _ in range(args.steps):
            np.copyto(wv, r["hv"])
            t0 = time.perf_counter()
            runner.ctx.sort(wv)
            times.append(time.perf_counter() - t0)
        tsum = max_over_ranks(sum(times), dist)
        # this machine's host link, for reading the end-to-end number: one pinned copy each way
        nb = n * esize
        link = {}
        for name, dst, src in (("h2d_gbs", runner.d[:nb], work), ("d2h_gbs", work, runner.d[:nb])):
            e0, e1 = _t.cuda.Event(enable_timing=True), _t.cuda.Event(enable_timing=True)
            dst.copy_(src, non_blocking=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            _t.cuda.synchronize()
            link[name] = nb / (e0.elapsed_time(e1) / 1e3) / 1e9
        e2e = {"value": n * world * args.steps / tsum / 1e9, "unit": "Gkeys/s",
               "h2d_bytes_per_step": n * esize, "d2h_bytes_per_step": n * esize,
               "ms_per_step": 1e3 * tsum / args.steps, "api": "gqs_sort_" + args.dtype + " (host pointers, pinned)",
               "median_ms_per_step": 1e3 * float(np.median(times)), "max_ms_per_step": 1e3 * max(times),
               "link": link,
               "copies_alone_ms": 1e3 * (nb / (link["h2d_gbs"] * 1e9) + nb / (link["d2h_gbs"] * 1e9)),
               "check": golden_check(golden_case(args.dtype, args.dist, n, SEED + rank), r["hv"], wv)}
        del work

    if rank != 0:
        runner.ctx.close()
        if dist is not None:
            dist.destroy_process_group()
        return

    wkey = f"plain_{args.dtype}_{args.dist}_2^{args.log2n}"
    roofline = roofline_of(r, peak, peak_src, ncu_traffic(wkey))
    cpu = None if args.no_cpu else cpu_baseline(args, n)
    v0 = gqs_ctypes.variants(args.dtype)[stats_last["variant"]]
    configs = None
    if want_configs:
        configs = run_configs(args, runner, clocks, peak, peak_src)
    prof = runner.ctx.profile() if args.profile else None
    levels = runner.ctx.levels() if args.profile else None
    runner.ctx.close()
    del runner
    import torch as _t
    _t.cuda.empty_cache()
    if want_configs:
        configs.append(run_batched(args, gqs_ctypes, rank, local, world, dist, barrier, clocks=clocks,
                                   steps=max(5, min(args.steps, 10)), warmup=3))
    clk = r["clocks"]
    serve = None
    if args.config == "plain" and args.serve_requests > 0 and world == 1:
        serve = run_serve(args, gqs_ctypes)
    clocks.stop()
    line = {
        "metric": METRIC if (args.config == "plain" and args.log2n == 28 and args.dtype == "u32")
        else f"Gkeys/s ({workload_name(args, n)})",
        "value": value, "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_sort / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded generator, gpu-quicksort_gb300/workload)",
        "config": {"workload": workload_name(args, n), "keys": n, "distribution": args.dist, "seed": SEED,
                   "l2": r["l2"], "variant": v0["name"], "grid": stats_last["grid"],
                   "threads": stats_last["threads"], "parallelism": f"replicas x{world}"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
        "check": r["check"],
        "stats": {k: stats_last[k] for k in ("part_keys", "local_keys", "tiny_keys", "fill_keys", "chunks",
                                             "part_jobs", "local_jobs", "fill_chunks", "max_depth")},
        "passes_per_key": (stats_last["part_keys"] + stats_last["local_keys"] + stats_last["tiny_keys"]) / n,
        "phases": phases,
        "configs": configs,
        "serve": serve,
        "profile": prof,
        "levels": levels,
        "wall_s": r["t1"] - r["t0"],
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
