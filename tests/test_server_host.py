"""CPU tests of the serving loop's host parts: the pool's range allocator
(tests/host/pool_check.cpp against a unit-by-unit model), the batching
decision driven by a CPU executor on a simulated clock
(tests/host/sched_check.cpp), and the request trace generator."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pool_allocator_against_model():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "pool_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "fft_onchip_gb300", "csrc"),
                    "-o", exe, os.path.join(ROOT, "tests", "host", "pool_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout


def test_batching_decision_with_cpu_executor():
    """Admission order, batch limits, the batching window, split-form size
    groups and pool accounting of fft_onchip_gb300/csrc/batching.h, with a CPU
    stand-in for the device that moves and transforms each request's data."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "sched_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "fft_onchip_gb300", "csrc"),
                    "-o", exe, os.path.join(ROOT, "tests", "host", "sched_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout


def test_trace_generator_shapes():
    from fft_onchip_gb300 import _lib
    from fft_onchip_gb300.serve import make_trace
    items, transforms, nbytes = make_trace(1e5, 2000, 1 << 24, seed=0, engines=(1, 2))
    arr = np.array([items[i].arrival_us for i in range(2000)])
    assert arr[0] == 0 and np.all(np.diff(arr) >= 0)
    rate = 2000 / (arr[-1] * 1e-6)
    assert 0.9e5 < rate < 1.1e5
    counts = np.array([items[i].count for i in range(2000)])
    assert counts.min() >= 1 and counts.max() <= 4096
    assert 0.4 < np.mean(counts <= 64) < 0.6  # log-uniform: half below sqrt(4096)
    ns = {items[i].n for i in range(2000)}
    assert ns == set(_lib.SIZES)
    engs = np.array([items[i].engine for i in range(2000)])
    assert 0.45 < np.mean(engs == 1) < 0.55
    assert transforms == counts.sum()
    for i in range(2000):
        assert items[i].in_offset % 8 == 0 and items[i].in_offset + items[i].count * items[i].n <= 1 << 24
