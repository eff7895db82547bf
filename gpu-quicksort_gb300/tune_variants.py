"""Times every kernel variant of every key type at every size class on the GPU and writes the
tuning table csrc/gqs_tuning.h (and a JSON copy of the timings).

For each key type (u32, f32, f64 keys; u64 for the packed words of the pair sort) and each size
2^lo .. 2^hi, every variant sorts the same seeded keys (device-pointer call, keys resident in
HBM, the L2 flushed before each sort of less than 256 MiB): `reps` timed sorts after two warm-up
sorts, median kept by CUDA events around the call on its stream. The fastest variant of each
(key type, size) becomes a row keyed by the GPU's SM count. A context created with variant -1
then uses it for every sort whose size rounds up to that class. Run on the target GPU from the
repository root, then rebuild:

    python gpu-quicksort_gb300/tune_variants.py [--lo 10] [--hi 29] [--reps 7] [--json out.json]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import gqs_ctypes  # noqa: E402

DT = {"u32": 0, "f32": 1, "f64": 2, "u64": 3}
DIST = {"u32": "uniform", "f32": "gaussian", "f64": "uniform", "u64": "uniform"}
L2_FLUSH = 256 << 20


def time_variant(torch, dtype, v, d, dn, pristine, vals, n, reps, flush):
    """Median ms of `reps` sorts of n keys with variant v (u64: n (key, index) pairs)."""
    ctx = gqs_ctypes.Context(device=0, sync=False, timing=False, variant=v)
    stream = torch.cuda.current_stream()
    ms = []
    try:
        for i in range(reps + 2):
            d.copy_(pristine)
            if vals is not None:
                dn.copy_(vals)
            if flush is not None:
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if dtype == "u64":
                rc = ctx.sort_pairs_dev("u32", d.data_ptr(), dn.data_ptr(), n, stream.cuda_stream)
            else:
                rc = ctx.sort_dev(dtype, d.data_ptr(), dn.data_ptr(), n, stream.cuda_stream)
            e1.record(stream)
            if rc != 0 or ctx.sync() != 0:
                return None
            if i >= 2:
                ms.append(e0.elapsed_time(e1))
    finally:
        ctx.close()
    return float(np.median(ms))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lo", type=int, default=10)
    ap.add_argument("--hi", type=int, default=29)
    ap.add_argument("--reps", type=int, default=7)
    ap.add_argument("--types", default="u32,f32,f64,u64")
    ap.add_argument("--json", default=None)
    ap.add_argument("--header", default=os.path.join(HERE, "csrc", "gqs_tuning.h"))
    args = ap.parse_args()
    import torch
    props = torch.cuda.get_device_properties(0)
    sms = props.multi_processor_count
    flush = torch.empty(L2_FLUSH, dtype=torch.uint8, device="cuda")
    rows, timings = [], {}
    for dtype in args.types.split(","):
        nvar = len(gqs_ctypes.variants("f64" if dtype == "u64" else dtype))
        hi = min(args.hi, 28) if dtype in ("f64", "u64") else args.hi
        for lg in range(args.lo, hi + 1):
            n = 1 << lg
            if dtype == "u64":  # pair sort: u32 keys, u32 values 0..n-1 (packed into u64 words)
                keys = gqs_ctypes.generate("u32", "uniform", 20260501 + lg, n)
                pristine = torch.from_numpy(keys.view(np.int32)).cuda()
                vals = torch.arange(n, dtype=torch.int32, device="cuda")
                d, dn = torch.empty_like(pristine), torch.empty_like(vals)
                nbytes = 8 * n
            else:
                a = gqs_ctypes.generate(dtype, DIST[dtype], 20260501 + lg, n)
                pristine = torch.from_numpy(a.view(np.int32) if dtype == "u32" else a).cuda()
                vals = None
                d, dn = torch.empty_like(pristine), torch.empty_like(pristine)
                nbytes = a.nbytes
            f = flush if nbytes < L2_FLUSH else None
            ms = [time_variant(torch, dtype, v, d, dn, pristine, vals, n, args.reps, f) for v in range(nvar)]
            ok = [(m, v) for v, m in enumerate(ms) if m is not None]
            best = min(ok)[1] if ok else 0
            rows.append((sms, DT[dtype], lg, best))
            timings[f"{dtype}_2^{lg}"] = {"ms": ms, "best": best, "gkeys_s": n / (min(ok)[0] / 1e3) / 1e9 if ok else None}
            print(f"{dtype} 2^{lg}: best variant {best}  " + " ".join(f"{m:.4f}" if m else "-" for m in ms), flush=True)
            del d, dn, pristine, vals
            torch.cuda.empty_cache()
    body = ",\n".join(f"    {{{s_}, {t}, {lg}, {v}}}" for s_, t, lg, v in rows)
    text = f"""// The fastest kernel variant per (SM count, key type, size class), the counterpart of the
// reference's size-dependent launch parameters (optp, GPU-Quicksort_Full_SYCL/QuicksortMain.cpp:
// 831-833). A context created with variant -1 looks up every sort here by the device's SM count
// and ceil(log2 n); rows are written by gpu-quicksort_gb300/tune_variants.py from timed sorts.
// Rows below: {props.name}, {sms} SMs, median of {args.reps} sorts per variant and size.
#pragma once

namespace gqs {{

struct TuneRow {{
  int sms;      // SMs of the GPU the row was measured on
  int dtype;    // DT_U32, DT_F32, DT_F64, DT_U64 (the packed pairs)
  int log2n;    // size class: n in (2^(log2n - 1), 2^log2n]
  int variant;  // fastest variant
}};

constexpr TuneRow kTuneRows[] = {{
{body},
}};

}}  // namespace gqs
"""
    with open(args.header, "w") as fh:
        fh.write(text)
    if args.json:
        with open(args.json, "w") as fh:
            json.dump({"gpu": props.name, "sms": sms, "reps": args.reps, "timings": timings}, fh, indent=1)
    print("wrote", args.header)


if __name__ == "__main__":
    main()
