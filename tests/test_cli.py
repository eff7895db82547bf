"""The reference-compatible command line (gpu-quicksort_gb300/quicksort): argument handling
on the CPU, full runs on the GPU (same statistics lines as the reference's driver)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "gpu-quicksort_gb300", "quicksort")


def run(*args, timeout=300):
    return subprocess.run([CLI, *map(str, args)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=timeout)


def test_usage_on_wrong_argument_count():
    r = run()
    assert r.returncode == 2 and r.stdout.startswith("Usage: quicksort [num test iterations]")
    r = run(1, "gpu", "nvidia", 4)
    assert r.returncode == 2 and "Usage" in r.stdout


def test_only_the_gpu_device_type_exists():
    r = run(1, "cpu", "intel", 16, 16, "no_show_cl")
    assert r.returncode == 2 and "GB300 GPU only" in r.stdout
    r = run(1, "gpu", "intel", 16, 16, "no_show_cl")
    assert r.returncode == 2 and "NVIDIA" in r.stdout


def test_without_a_gb300_the_context_fails_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(1, "gpu", "nvidia", 16, 16, "no_show_cl")
    assert r.returncode == 3 and "no sm_103" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(64, 64), (1024, 1024), (2048, 1024)])
def test_cli_sorts_all_three_key_types(w, h):
    r = run(3, "gpu", "nvidia", w, h, "show_cl")
    assert r.returncode == 0, r.stdout
    out = r.stdout
    assert out.count("verifying: true") == 9 and "verifying: false" not in out
    assert out.count(" Number of failures: 0 out of 3") == 3
    for line in ("Average Time:", "Standard Deviation:", "%error (3*stdDev)/Average:", "min time:", "max time:",
                 "Average speedup over CPU std::sort:", "Using device 0:"):
        assert line in out
    assert f"Allocating array size of {w * h} (uint)" in out and f"Allocating array size of {w * h} (double)" in out


SWEEP = os.path.join(ROOT, "gpu-quicksort_gb300", "cli", "sweep.sh")


def test_sweep_script_stops_without_a_gb300():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert subprocess.run(["bash", "-n", SWEEP]).returncode == 0
    r = subprocess.run(["bash", SWEEP, "256", "1", "1"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=120)
    assert r.returncode != 0 and "Trial 1 ---- 256 x 256" in r.stdout and "no sm_103" in r.stdout


@pytest.mark.gpu
def test_sweep_script_small_sizes():
    # count 256 and 512: 2^16, 2^17, 2^18 and 2^19 keys, one trial of two iterations each
    r = subprocess.run(["bash", SWEEP, "512", "1", "2"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    out = r.stdout
    for w, h in ((256, 256), (512, 256), (512, 512), (1024, 512)):
        assert f"---- {w} x {h} ----" in out and f"Allocating array size of {w * h} (float)" in out
    assert out.count("verifying: true") == 4 * 3 * 2 and "verifying: false" not in out
