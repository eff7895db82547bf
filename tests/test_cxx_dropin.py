"""The C++ drop-in entry (include/gqs/Quicksort.h): a caller written like the reference's
big_test<T> compiles with plain g++ against libgqs.so; without a GB300 it stops cleanly at
context creation, and on a GB300 it sorts the shuffled 1..N for uint32, float and double
exactly as std::sort does."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-quicksort_gb300")
SRC = os.path.join(ROOT, "tests", "cxx_dropin.cpp")


@pytest.fixture(scope="module")
def dropin(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("dropin") / "cxx_dropin")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), SRC, "-L" + PKG, "-lgqs",
                    "-Wl,-rpath," + PKG, "-o", exe], check=True)
    return exe


def test_dropin_without_a_gb300_stops_at_context_creation(dropin):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([dropin, "4096"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert r.returncode == 3 and "no usable device" in r.stdout, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 4096, 1 << 22, (1 << 24) + 3])
def test_dropin_sorts_like_std_sort(dropin, n):
    r = subprocess.run([dropin, str(n)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    assert r.stdout.count("verifying: true") == 3
