"""The serving loop's device-arena allocator (gpu-quicksort_gb300/csrc/gqs_arena.h), on the
CPU: a randomized C++ driver checks first fit, merging frees and the byte accounting after
every operation."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "arena_check.cpp")
CSRC = os.path.join(ROOT, "gpu-quicksort_gb300", "csrc")


@pytest.fixture(scope="module")
def arena_check(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("arena") / "arena_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + CSRC, SRC, "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3, 20260301])
def test_arena_allocator_invariants(arena_check, seed):
    r = subprocess.run([arena_check, str(seed), "20000"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
