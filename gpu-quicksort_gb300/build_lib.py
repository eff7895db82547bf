"""Builds the gqs shared libraries in-tree (no cmake, no pip).

    libgqs.so           the CUDA sort library behind include/gqs.h (sm_103a only)
    libgqs_workload.so  seeded synthetic workload generators (host C++)
    libgqs_prof.so      on request (profile=True): the library with per-role cycle counters
    libgqs_check.so     on request (check=True): the library with device bounds checks

Objects go to _build/ next to this file; the libraries land beside this file.
Run as a script or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + CSRC, "-I" + INCLUDE]
CU_SOURCES = ["gqs_sort_dispatch.cu", "gqs_capi.cu", "gqs_noalloc.cu", "gqs_batch.cu", "gqs_serve.cu",
              "gqs_merge.cu", "gqs_split.cu"]
VARIANT_TU = "gqs_variant_tu.cu"  # compiled once per (key type, variant index)

LIB = os.path.join(HERE, "libgqs.so")
PROF_LIB = os.path.join(HERE, "libgqs_prof.so")  # -DGQS_PROFILE: per-role cycle counters
CHECK_LIB = os.path.join(HERE, "libgqs_check.so")  # -DGQS_CHECK: bounds checks on the device
WORKLOAD_LIB = os.path.join(HERE, "libgqs_workload.so")
CLI = os.path.join(HERE, "quicksort")  # the reference-compatible benchmark command line


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "gqs.h"))
    return hs


def variant_count() -> int:
    """Variants per key type, as gqs_variant_table.h defines them."""
    with open(os.path.join(CSRC, "gqs_variant_table.h")) as f:
        for line in f:
            if line.startswith("#define GQS_VARIANT_COUNT"):
                return int(line.split()[2])
    raise RuntimeError("GQS_VARIANT_COUNT not found")


def _units() -> list[tuple[str, str, list[str]]]:
    """(source, object name, extra flags) of every CUDA translation unit."""
    units = [(src, src.replace(".cu", ".o"), []) for src in CU_SOURCES]
    for t in ("u32", "f32", "f64", "u64"):
        for v in range(variant_count()):
            units.append((VARIANT_TU, "gqs_v_%s_%d.o" % (t, v),
                          ["-DGQS_TU_LIST=GQS_VARIANTS_" + t.upper(), "-DGQS_TU_TYPE=" + t,
                           "-DGQS_TU_INDEX=%d" % v]))
    return units


def build(force: bool = False, verbose: bool = False, profile: bool = False, check: bool = False) -> dict:
    """Compiles what is out of date; returns the library paths. profile=True builds
    libgqs_prof.so with the device cycle counters, check=True libgqs_check.so with the device
    bounds checks, instead of libgqs.so."""
    if profile and check:
        raise ValueError("one library flavour at a time")
    bdir = BUILD + ("_prof" if profile else "_check" if check else "")
    lib = PROF_LIB if profile else CHECK_LIB if check else LIB
    extra = ["-DGQS_PROFILE"] if profile else ["-DGQS_CHECK"] if check else []
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src, obj, defs in _units():
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, obj)
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + extra + defs + ["-c", s, "-o", o])
    wsrc = os.path.join(HERE, "workload", "gqs_workload.cpp")
    whdr = os.path.join(HERE, "workload", "gqs_workload.h")
    wjob = None
    if force or _stale(WORKLOAD_LIB, [wsrc, whdr]):
        wjob = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                "-fno-fast-math", "-I" + os.path.join(HERE, "workload"), wsrc, "-o", WORKLOAD_LIB]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))) as ex:
        futs = [ex.submit(_run, j) for j in jobs]
        if wjob:
            futs.append(ex.submit(_run, wjob))
        for f in futs:
            f.result()
    if force or jobs or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-fPIC"])
    out = {"lib": lib, "workload": WORKLOAD_LIB}
    csrc = os.path.join(HERE, "cli", "quicksort_main.cpp")
    if not profile and not check and os.path.exists(csrc):
        if force or _stale(CLI, [csrc, LIB, WORKLOAD_LIB, os.path.join(INCLUDE, "gqs.h")]):
            _run([nvcc, "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + os.path.join(HERE, "workload"), csrc,
                  "-L" + HERE, "-lgqs", "-lgqs_workload", "-Xlinker", "-rpath,$ORIGIN", "-o", CLI])
        out["cli"] = CLI
    if verbose:
        print("built", lib, WORKLOAD_LIB, out.get("cli", ""))
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, profile="--profile" in sys.argv, check="--check" in sys.argv)
